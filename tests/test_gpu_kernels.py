"""The two stencil kernel forms (one CTA per tile; persistent CTAs walking
the batch's tiles through a two-stage TMA pipeline) give bit-identical
results, including batches of uneven aperture windows, and the autotuner
leaves the context on a valid setting whose results still match the
oracle."""
import numpy as np
import pytest

from oracle import oracle as orc
from rtm_gpu_gb300 import Engine, capi
from test_gpu_windows import window_problem
from util import interior, rel_l2, small_problem

pytestmark = pytest.mark.gpu
TILED, PERSISTENT, SPLIT, X2, X2S = (capi.RTM_KERNEL_TILED, capi.RTM_KERNEL_PERSISTENT, capi.RTM_KERNEL_SPLIT,
                                     capi.RTM_KERNEL_X2, capi.RTM_KERNEL_X2_SPLIT)


def _seis(p, n, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((n, p.nrec, p.NT)) * 1e-2).astype(np.float32)


@pytest.mark.parametrize("adaptive", [True, False])
def test_forms_bit_identical(product_lib, cuda_ok, adaptive):
    p = small_problem(nx=150, nz=45, adaptive=adaptive)
    srcs = [p.src_flat(p.N2 + 1, p.N2 + x) for x in (3, 40, 77, 120, 149)]
    seis = _seis(p, len(srcs), 3)
    out = {}
    with Engine(p, batch=5) as e:
        for fwd, bwd in ((TILED, TILED), (PERSISTENT, PERSISTENT), (TILED, PERSISTENT), (SPLIT, SPLIT),
                         (PERSISTENT, SPLIT), (X2, TILED), (X2S, SPLIT), (X2S, TILED)):
            e.set_kernel(fwd, bwd)
            assert e.kernel() == {"fwd": fwd, "bwd": bwd, "shots_per_launch": 5}
            out[(fwd, bwd)] = e.migrate(srcs, seis)
    ref = out[(TILED, TILED)]
    for k, (g1, g2) in out.items():
        assert np.array_equal(g1, ref[0]) and np.array_equal(g2, ref[1]), k


def test_forms_bit_identical_uneven_windows(product_lib, cuda_ok):
    N2 = 8
    p = small_problem(nz=50, nx=300, N2=N2, M=4, NT=80, rec=(N2 + 4, N2 + 140, 2, 0, 18))
    wins = [(0, 300), (60, 90), (100, 200), (10, 131), (140, 17)]  # all contain the well
    srcs = []
    for i, (xa, nx) in enumerate(wins):
        q = window_problem(p, xa, nx)
        srcs.append((N2 + 1) * q.NX + N2 + nx // 2)
    seis = _seis(p, len(wins), 4)
    res = []
    with Engine(p, batch=5) as e:
        for fwd, bwd in ((TILED, TILED), (PERSISTENT, PERSISTENT), (SPLIT, SPLIT), (X2, TILED), (X2S, TILED)):
            e.set_kernel(fwd, bwd)
            res.append(e.migrate_stack_windows(srcs, [w[0] for w in wins], [w[1] for w in wins],
                                               seis, 1e-4, len(wins), True))
    for r in res[1:]:
        assert np.array_equal(res[0][0], r[0]) and np.array_equal(res[0][1], r[1])


def test_shots_per_launch(product_lib, cuda_ok):
    p = small_problem(nx=100)
    srcs = [p.src_flat(p.N2 + 1, p.N2 + x) for x in (10, 50, 90)]
    seis = _seis(p, len(srcs), 5)
    with Engine(p, batch=3) as e:
        a = e.migrate(srcs, seis)
        e.set_kernel(PERSISTENT, PERSISTENT, 2)  # groups of 2 + 1
        b = e.migrate(srcs, seis)
        with pytest.raises(RuntimeError):
            e.set_kernel(PERSISTENT, PERSISTENT, 4)  # above the context's batch
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_autotune_then_oracle(product_lib, cuda_ok):
    p = small_problem(nx=120, nz=40, NT=120)
    srcs = [p.src_flat(p.N2 + 1, p.N2 + x) for x in (5, 30, 60, 90, 110, 119, 2, 47)]
    seis = _seis(p, len(srcs), 6)
    with Engine(p, batch=8) as e:
        rate = e.autotune(srcs, nsteps=10)
        k = e.kernel()
        assert rate > 0
        assert k["fwd"] in (TILED, PERSISTENT, SPLIT, X2, X2S) and k["bwd"] in (TILED, PERSISTENT, SPLIT)
        assert k["shots_per_launch"] in (8, 4)
        g1, g2 = e.migrate(srcs, seis)
    for i in (0, 5, 7):
        q = p.with_source(srcs[i] // p.NX, srcs[i] % p.NX)
        o1, o2 = orc.migrate(q, seis[i])
        assert rel_l2(interior(p, g1[i]), interior(p, o1)) < 1e-4
        assert rel_l2(interior(p, g2[i]), interior(p, o2)) < 1e-4


def test_few_and_many_bins_per_tile(product_lib, cuda_ok):
    """A model whose first tile column has few velocity bins and whose others
    have nearly a bin per cell (1100 bins, scattered coefficient gathers):
    both kernel forms bit-identical and against the oracle."""
    from rtm_gpu_gb300.problem import build_problem
    from util import oracle_table
    N2, nz, nx = 8, 40, 300
    rng = np.random.default_rng(21)
    vin = np.full((nz, nx), 2000.0, np.float32)
    vin += (np.arange(nz)[:, None] * 2.0).astype(np.float32)          # ~80 bins down the tile
    vin[:, 150:] = rng.uniform(1500.0, 2600.0, (nz, nx - 150)).astype(np.float32)  # ~1100 bins
    p = build_problem(vin, N2=N2, M=4, NT=120, h=10.0, tao=0.001, f0=25.0, adaptive=True, compen=True,
                      rec=(N2 + 1, N2, 0, 3, 100), coef_table=oracle_table(4, 0.001, 10.0, 50.0))
    srcs = [p.src_flat(N2 + 2, N2 + x) for x in (40, 220)]
    seis = _seis(p, len(srcs), 9)
    with Engine(p, batch=2) as e:
        res = {}
        for v in (TILED, PERSISTENT, X2):
            e.set_kernel(v, TILED if v == X2 else v)
            res[v] = e.migrate(srcs, seis)
    assert np.array_equal(res[TILED][0], res[PERSISTENT][0])
    assert np.array_equal(res[TILED][0], res[X2][0])
    for i, s in enumerate(srcs):
        q = p.with_source(s // p.NX, s % p.NX)
        o1, o2 = orc.migrate(q, seis[i])
        assert rel_l2(interior(p, res[TILED][0][i]), interior(p, o1)) < 1e-4
        assert rel_l2(interior(p, res[TILED][1][i]), interior(p, o2)) < 1e-4


def test_split_modelling_and_fp16_rings(product_lib, cuda_ok):
    """Forward modelling (receiver recording in the pad launches) and FP16
    rings with per-step scaling under the two-stream split: identical to one
    stream."""
    p = small_problem(nx=120, nz=40, NT=100)
    srcs = [p.src_flat(p.N2 + 1, p.N2 + x) for x in (5, 30, 60, 90, 110)]
    seis = _seis(p, len(srcs), 11)
    out = {}
    with Engine(p, batch=5, ring_precision=capi.RTM_RING_F16) as e:
        for v in (TILED, SPLIT):
            e.set_kernel(v)
            out[v] = (e.model(srcs), e.migrate(srcs, seis))
    assert np.array_equal(out[TILED][0], out[SPLIT][0])
    assert np.array_equal(out[TILED][1][0], out[SPLIT][1][0])
    assert np.array_equal(out[TILED][1][1], out[SPLIT][1][1])


def test_odd_pad_width_all_forms(product_lib, cuda_ok):
    """An odd pad width and grid width (column pairs of the two-column
    forward kernel straddle the pad edge): every form against the oracle."""
    p = small_problem(nx=97, nz=41, N2=7, M=4, NT=110)
    srcs = [p.src_flat(p.N2 + 1, p.N2 + x) for x in (0, 48, 96)]
    seis = _seis(p, len(srcs), 13)
    res = {}
    with Engine(p, batch=3) as e:
        for fwd, bwd in ((TILED, TILED), (X2, TILED), (PERSISTENT, PERSISTENT), (SPLIT, SPLIT)):
            e.set_kernel(fwd, bwd)
            res[(fwd, bwd)] = e.migrate(srcs, seis)
    ref = res[(TILED, TILED)]
    for k, (g1, g2) in res.items():
        assert np.array_equal(g1, ref[0]) and np.array_equal(g2, ref[1]), k
    for i, s in enumerate(srcs):
        q = p.with_source(s // p.NX, s % p.NX)
        o1, o2 = orc.migrate(q, seis[i])
        assert rel_l2(interior(p, ref[0][i]), interior(p, o1)) < 1e-4
        assert rel_l2(interior(p, ref[1][i]), interior(p, o2)) < 1e-4
