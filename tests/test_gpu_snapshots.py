"""Source snapshots (rtm_ctx_set_snapshots): the forward run stores the source
field's interior, and its running sum, every K steps; the backward run
advances the receiver field alone and applies the imaging condition at the
snapshot steps with end-corrected time weights.

* K = 1 with fp32 storage takes every step with weight 1, so it gives the
  ring scheme's rel1 / rel2 to fp32 round-off (the source field comes from
  the forward run instead of its reconstruction, and the source's running
  sum is the forward total minus the stored prefix): both imaging
  conditions, one shot and a batch, and a batch of uneven windows.  These
  cases run fewer steps than the wavelet's cut-off NT2: past it, the
  reconstruction of the ring scheme adds two wavelet samples that the forward
  run did not inject (kernel.cu's backward wavelet f((k+1)tao) with the cut
  k < NT2), so the reconstructed field differs from the forward field by
  their small wave, which snapshots do not carry (about 5e-4 in rel1 on a
  25 Hz, 300-step case);
* K = 4 with 16-bit storage against the FP64 oracle at the benchmark sizes:
  tests/test_gpu_configs.py (C1 and one C2 shot, modelled gathers);
* argument checks, storage bytes, and turning snapshots off again.
"""
import numpy as np
import pytest

from oracle.port_problem import window_problem
from rtm_gpu_gb300 import Engine, capi
from util import interior, rel_l2, small_problem

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.mark.parametrize("compen", [True, False])
def test_every_step_fp32_equals_ring_scheme(product_lib, cuda_ok, compen):
    p = small_problem(adaptive=True, compen=compen, M=8, N2=16, nz=80, nx=160, NT=300,
                      vlo=1800, vhi=3200, smooth=3.0, f0=2.5)  # NT2 = 801 > NT
    rng = np.random.default_rng(7)
    seis = (rng.standard_normal((2, p.nrec, p.NT)) * 1e-2).astype(np.float32)
    srcs = [p.src_flat(), p.src_flat(p.N2 + 2, p.N2 + 40)]
    with Engine(p, batch=2) as e:
        r1, r2 = e.migrate(srcs, seis)
    with Engine(p, batch=2) as e:
        e.set_snapshots(1, capi.RTM_RING_F32)
        s1, s2 = e.migrate(srcs, seis)
        e.set_snapshots(0)
        t1, t2 = e.migrate(srcs, seis)  # snapshots off again: the ring scheme
    for i in range(2):
        d1 = rel_l2(interior(p, s1[i]), interior(p, r1[i]))
        d2 = rel_l2(interior(p, s2[i]), interior(p, r2[i]))
        print("compen=%d shot %d: snapshots K=1 fp32 vs rings: rel1 %.2e rel2 %.2e" % (compen, i, d1, d2))
        assert d1 < TOL and d2 < TOL
    assert np.array_equal(t1, r1) and np.array_equal(t2, r2)


def test_every_step_fp32_windows_equal_ring_scheme(product_lib, cuda_ok):
    N2 = 8
    p = small_problem(nz=50, nx=160, N2=N2, M=4, NT=150, rec=(N2 + 4, N2 + 70, 2, 0, 18), f0=2.5)
    wins = [(0, 160), (30, 90), (56, 100), (12, 120)]
    rng = np.random.default_rng(12)
    srcs = []
    for i, (xa, nx) in enumerate(wins):
        q = window_problem(p, xa, nx)
        srcs.append((N2 + 1) * q.NX + N2 + nx // 2 + (i - 2) * 3)
    seis = (rng.standard_normal((len(wins), p.nrec, p.NT)) * 1e-2).astype(np.float32)
    args = (srcs, [w[0] for w in wins], [w[1] for w in wins], seis, 1e-4, len(wins), True)
    with Engine(p, batch=4) as e:
        img, ill = e.migrate_stack_windows(*args)
    with Engine(p, batch=4) as e:
        e.set_snapshots(1, capi.RTM_RING_F32)
        simg, sill = e.migrate_stack_windows(*args)
    d_img, d_ill = rel_l2(simg, img), rel_l2(sill, ill)
    print("windows, snapshots K=1 fp32 vs rings: image %.2e illumination %.2e" % (d_img, d_ill))
    assert d_img < TOL and d_ill < TOL


def _band_cells(p, half=24):
    """Cells of the band imaged at every step: `half` cells on each side of
    the receiver line, rows clipped to the interior."""
    rz0, rx0, rdz, rdx, n = p.rec
    zl, zh = min(rz0, rz0 + (n - 1) * rdz), max(rz0, rz0 + (n - 1) * rdz)
    z0 = max(p.N2, zl - half)
    zn = min(p.NZ - p.N2 - 1, zh + half) - z0 + 1
    return zn * (abs((n - 1) * rdx) + 2 * half + 1)


def test_snapshot_arguments_and_bytes(product_lib, cuda_ok):
    p = small_problem(M=4, N2=8, nz=40, nx=60, NT=103)
    with Engine(p, batch=3) as e:
        lib = capi.lib()
        assert lib.rtm_ctx_set_snapshots(e._h, -1, capi.RTM_RING_F16) == capi.RTM_ERR_ARG
        assert lib.rtm_ctx_set_snapshots(e._h, 4, 7) == capi.RTM_ERR_ARG
        assert e.snapshots() == {"every": 0, "precision": 0, "bytes": 0}
        base = e.device_bytes
        e.set_snapshots(4, capi.RTM_RING_I16)
        got = e.snapshots()
        slots = 3 + (p.NT - 5) // 4  # steps 0, 1, 2, 6, 10, .. <= NT-3
        pitch = (p.nx + p.N2 % 8 + 7) // 8 * 8
        assert got["every"] == 4 and got["precision"] == capi.RTM_RING_I16
        band = 3 * (p.NT - 2) * _band_cells(p) * (4 + 4)  # the receiver band, every step, fp32
        assert got["bytes"] == 3 * slots * p.nz * pitch * (2 + 4) + band  # S in 2 bytes, its sum in 4
        assert e.device_bytes >= base + got["bytes"]
        e.set_snapshots(2, capi.RTM_RING_F32)
        assert e.snapshots()["bytes"] == 3 * (3 + (p.NT - 5) // 2) * p.nz * pitch * (4 + 4) + band
        e.set_snapshots(0)
        assert e.snapshots()["bytes"] == 0 and e.device_bytes == base


@pytest.mark.parametrize("prec", [capi.RTM_RING_F16, capi.RTM_RING_I16, capi.RTM_RING_BF16])
def test_every_step_16bit_pad30(product_lib, cuda_ok, prec):
    """16-bit snapshot codes with the benchmark's 30-cell pad (the stored
    interior starts at column N2 % 8 of its plane so every snapshot tile
    begins on 16 bytes): every step, against fp32 snapshots -- the codes'
    rounding alone (one scale per slot and quantity)."""
    p = small_problem(adaptive=True, M=8, N2=30, nz=60, nx=200, NT=200, vlo=1800, vhi=3200,
                      smooth=3.0, f0=5.0)
    rng = np.random.default_rng(9)
    seis = (rng.standard_normal((1, p.nrec, p.NT)) * 1e-2).astype(np.float32)
    out = {}
    for pr in (capi.RTM_RING_F32, prec):
        with Engine(p, batch=1) as e:
            e.set_snapshots(1, pr)
            out[pr] = e.migrate([p.src_flat()], seis)
    d1 = rel_l2(interior(p, out[prec][0][0]), interior(p, out[capi.RTM_RING_F32][0][0]))
    d2 = rel_l2(interior(p, out[prec][1][0]), interior(p, out[capi.RTM_RING_F32][1][0]))
    print("storage %d vs fp32 snapshots: rel1 %.2e rel2 %.2e" % (prec, d1, d2))
    tol = 2e-2 if prec == capi.RTM_RING_BF16 else 2e-3
    assert d1 < tol and d2 < tol
