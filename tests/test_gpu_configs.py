"""Parity at the benchmark configurations themselves, at full size.

* C1 (one shot, 201x401, dx=10 m, 2000 steps, M=6 adaptive least-squares
  coefficients, 30-cell hybrid ABC, 20 Hz source at (2,200), 401 surface
  receivers; observed gathers = true model minus smoothed model);
* one shot of C2, the benched multi-shot workload (401x1201, dx=12.5 m, 4000
  steps, M=8 adaptive, full-spread receivers, FP16 boundary rings as benched);
* one batched set of C3 aperture windows (the narrowest, the widest and one
  middle window of the reverse-VSP survey, 300 well receivers), at full size.

References: the reference's own kernels (kernel.cu:18-517) compiled
unchanged for the GPU and driven by its per-shot launch sequence
(oracle/_ref/libref_gpu.so) and for the CPU (oracle/_ref/libref_rtm.so), and
the FP64 oracle.  Tolerances, relative L2 over the interior:

* against the reference's GPU build: 1e-4 for the cross-correlation rel1,
  the illumination rel2 and the finished image (up / down after the
  Laplacian filter and stabilisation); measured 1e-6 .. 5e-5;
* against the reference's CPU build (no multiply-add contraction) at C1:
  gathers 1e-4; rel1 and image 2e-4, because the reference's own GPU and CPU
  builds differ by 1.2e-4 (rel1) and 1.5e-4 (image) on these same inputs;
* against FP64: image NRMSE 1e-3 (the stated accuracy bar) for one shot;
  measured 9e-5 at C1, 5.5e-4 at C2 with FP16 rings (the reference's GPU
  build: 5.6e-4).  The stacked C3 window image is held to the reference's
  own FP32 distance from FP64 (see its test);
* source snapshots (no source reconstruction), 16-bit storage, against
  FP64: the same 1e-3 bar, every 4 steps at C1 (measured 1.4e-4) and on the
  C2 shot every step and every 4 steps (5.7e-4; rings 5.5e-4).
"""
import numpy as np
import pytest

from oracle import oracle as orc
from oracle.port_problem import window_problem
from rtm_gpu_gb300 import Engine, capi, coeffs, synth
from rtm_gpu_gb300.problem import build_problem
from util import rel_l2

pytestmark = pytest.mark.gpu
WHITE = 1e-4


def _interior(p, g):
    return np.asarray(g)[p.N2:p.NZ - p.N2, p.N2:p.NX - p.N2]


def _image(p, r1, r2):
    up, dn = orc.finish_shot(p, r1, r2, WHITE)
    return up / dn


def _errors(p, a, b):
    """rel-L2 of rel1, rel2 and the finished image of run a against run b."""
    return {"rel1": rel_l2(_interior(p, a[0]), _interior(p, b[0])),
            "rel2": rel_l2(_interior(p, a[1]), _interior(p, b[1])),
            "image": rel_l2(_image(p, *a), _image(p, *b))}


def _problems(vtrue, *, N2, M, NT, h, f0, rec, src):
    table = coeffs.table_source(nfdmax=M, nfdmin=2, tao=0.001, h=h, fmax=2 * f0)
    kw = dict(N2=N2, M=M, NT=NT, h=h, tao=0.001, f0=f0, adaptive=True, compen=True, rec=rec,
              coef_table=table)
    vmig = synth.smooth_model(vtrue, 10.0)
    return (build_problem(vtrue, **kw).with_source(*src),
            build_problem(vmig, **kw).with_source(*src))


@pytest.fixture(scope="module")
def c1(product_lib, cuda_ok):
    N2 = 30
    pt, ps = _problems(synth.model_c1(), N2=N2, M=6, NT=2000, h=10.0, f0=20.0,
                       rec=synth.full_spread(401, N2), src=(N2 + 1, N2 + 199))
    gt_ref, gs_ref = orc.model(pt, use_ref=True), orc.model(ps, use_ref=True)
    with Engine(pt, batch=1) as e:
        gt = e.model([pt.src_flat()])[0]
    with Engine(ps, batch=1) as e:
        gs = e.model([ps.src_flat()])[0]
    seis = (gt_ref - gs_ref).astype(np.float32)
    with Engine(ps, batch=1) as e:
        g1, g2 = e.migrate([ps.src_flat()], seis[None])
    with Engine(ps, batch=1) as e:
        e.set_snapshots(4, capi.RTM_RING_F16)
        n1, n2 = e.migrate([ps.src_flat()], seis[None])
    runs = {"engine": (g1[0], g2[0]), "snap4_f16": (n1[0], n2[0]),
            "ref_gpu": orc.ref_gpu_migrate(ps, seis)[:2],
            "ref_cpu": orc.migrate(ps, seis, use_ref=True),
            "f64": orc.migrate(ps, seis, precision="f64")}
    return ps, runs, {"true": (gt, gt_ref), "smooth": (gs, gs_ref)}


def test_c1_gathers_match_reference(c1):
    _, _, gathers = c1
    for name, (g, r) in gathers.items():
        assert rel_l2(g, r) < 1e-4, name


def test_c1_migration_matches_reference_gpu_build(c1):
    p, runs, _ = c1
    e = _errors(p, runs["engine"], runs["ref_gpu"])
    print("C1 engine vs reference GPU build:", e)
    assert max(e.values()) < 1e-4, e


def test_c1_migration_matches_reference_cpu_build(c1):
    p, runs, _ = c1
    e = _errors(p, runs["engine"], runs["ref_cpu"])
    own = _errors(p, runs["ref_gpu"], runs["ref_cpu"])  # the reference against itself
    print("C1 engine vs reference CPU build:", e, "reference GPU vs CPU build:", own)
    assert e["rel2"] < 1e-4
    assert e["rel1"] < 2e-4 and e["image"] < 2e-4, e


def test_c1_image_vs_fp64(c1):
    p, runs, _ = c1
    e = _errors(p, runs["engine"], runs["f64"])
    print("C1 engine vs FP64:", e)
    assert e["image"] < 1e-3 and e["rel2"] < 1e-4


def test_c1_snapshots_vs_fp64(c1):
    """Source snapshots every 4 steps in FP16 (no source reconstruction,
    imaging at every 4th step): finished image within the 1e-3 bar of FP64."""
    p, runs, _ = c1
    e = _errors(p, runs["snap4_f16"], runs["f64"])
    own = _errors(p, runs["snap4_f16"], runs["engine"])
    print("C1 snapshots K=4 FP16 vs FP64:", e, "vs the ring scheme:", own)
    assert e["image"] < 1e-3


@pytest.fixture(scope="module")
def c2(product_lib, cuda_ok):
    N2 = 30
    pt, ps = _problems(synth.model_c2(), N2=N2, M=8, NT=4000, h=12.5, f0=25.0,
                       rec=synth.full_spread(1201, N2),
                       src=synth.surface_shots(1201, 64, N2)[32])
    with Engine(pt, batch=1) as e:
        gt = e.model([pt.src_flat()])[0]
    with Engine(ps, batch=1) as e:
        gs = e.model([ps.src_flat()])[0]
    seis = (gt - gs).astype(np.float32)
    with Engine(ps, batch=1, ring_precision=capi.RTM_RING_F16) as e:
        g1, g2 = e.migrate([ps.src_flat()], seis[None])
    runs = {"engine_f16": (g1[0], g2[0]), "ref_gpu": orc.ref_gpu_migrate(ps, seis)[:2],
            "f64": orc.migrate(ps, seis, precision="f64")}
    for name, K, prec in (("snap1_f16", 1, capi.RTM_RING_F16), ("snap1_i16", 1, capi.RTM_RING_I16),
                          ("snap4_f16", 4, capi.RTM_RING_F16)):
        with Engine(ps, batch=1) as e:
            e.set_snapshots(K, prec)
            n1, n2 = e.migrate([ps.src_flat()], seis[None])
        runs[name] = (n1[0], n2[0])
    return ps, runs


def test_c2_shot_matches_reference_gpu_build(c2):
    p, runs = c2
    e = _errors(p, runs["engine_f16"], runs["ref_gpu"])
    print("C2 shot, FP16 rings, engine vs reference GPU build:", e)
    assert max(e.values()) < 1e-4, e


def test_c2_shot_snapshots_vs_fp64(c2):
    """Source snapshots (no source reconstruction) on the C2 shot, stored
    every step (FP16 / int16 codes) and every 4th step (C4's spacing, FP16;
    the band around the receiver line imaged at every step): the image within
    the 1e-3 bar of FP64 and within 2e-4 of the ring scheme's own distance."""
    p, runs = c2
    err = {k: _errors(p, runs[k], runs["f64"]) for k in ("snap1_f16", "snap1_i16", "snap4_f16")}
    rings = _errors(p, runs["engine_f16"], runs["f64"])
    print("C2 shot, snapshots vs FP64:", err, "ring scheme:", rings)
    for k in err:
        assert err[k]["image"] <= 1e-3 and err[k]["image"] <= rings["image"] + 2e-4, (k, err[k])


def test_c2_shot_image_nrmse_vs_fp64(c2):
    p, runs = c2
    e = _errors(p, runs["engine_f16"], runs["f64"])
    own = _errors(p, runs["ref_gpu"], runs["f64"])
    print("C2 shot, FP16 rings, engine vs FP64:", e, "reference GPU build vs FP64:", own)
    assert e["image"] <= 1e-3
    assert e["image"] <= own["image"] + 2e-4  # no worse than the reference's own FP32


@pytest.fixture(scope="module")
def c3(product_lib, cuda_ok):
    import bench
    N2 = 30

    class _A:
        workload, small, nt, shots, coef, ring = "rvsp", False, 0, 0, "adaptive", None
    cfg = bench.Config(_A())
    src, xa, wn, rec = bench.rvsp_geometry(cfg, nshot=128)
    pick = [int(np.argmin(wn)), int(np.argmax(wn)), 64]
    pt, ps = _problems(synth.model_c2(), N2=N2, M=8, NT=4000, h=12.5, f0=25.0, rec=rec,
                       src=(0, 0))
    full = [ps.src_flat(*src[i]) for i in pick]
    with Engine(pt, batch=3) as e:
        gt = e.model(full)
    with Engine(ps, batch=3) as e:
        gs = e.model(full)
    seis = (gt - gs).astype(np.float32)
    wx = [int(xa[i]) for i in pick]
    ww = [int(wn[i]) for i in pick]
    wsrc = [src[i][0] * (w + 2 * N2) + src[i][1] - x0 for i, x0, w in zip(pick, wx, ww)]
    # the three uneven windows advance together (one batch, shared launches);
    # stacked without normalisation: sums of the shots' up / down images
    with Engine(ps, batch=3) as e:
        sup, sdn = e.migrate_stack_windows(wsrc, wx, ww, seis, WHITE, 1, False)
    return ps, seis, wsrc, wx, ww, sup, sdn


def _window_stack(ps, seis, wsrc, wx, ww, migrate):
    """Sums of the per-window up / down images in the survey frame (float64)."""
    sup = np.zeros((ps.nz, ps.nx))
    sdn = np.zeros_like(sup)
    for k in range(len(wx)):
        q = window_problem(ps, wx[k], ww[k])
        q = q.with_source(wsrc[k] // q.NX, wsrc[k] % q.NX)
        up, dn = orc.finish_shot(q, *migrate(q, seis[k]), WHITE)
        sup[:, wx[k]:wx[k] + ww[k]] += up.T
        sdn[:, wx[k]:wx[k] + ww[k]] += dn.T
    return sup, sdn


def test_c3_window_batch_matches_reference_gpu_build_and_fp64(c3):
    """The batched uneven windows against the reference's GPU build run on each
    window: within 1e-4.  Against FP64 the stacked image (sum of up over sum
    of down) of this three-window set lies about 2e-3 away for every FP32
    build -- the windows' edges, where few shots and little energy enter the
    ratio, weigh in -- so the engine is held to the reference's own FP32
    distance (plus 2e-4), its illumination and up-sum to 1e-4 and 1e-3."""
    ps, seis, wsrc, wx, ww, sup, sdn = c3
    m = sdn > 0  # survey cells some window covers
    got_img = sup[m] / sdn[m]
    stacks = {"ref_gpu": _window_stack(ps, seis, wsrc, wx, ww, lambda q, s: orc.ref_gpu_migrate(q, s)[:2]),
              "f64": _window_stack(ps, seis, wsrc, wx, ww, lambda q, s: orc.migrate(q, s, precision="f64"))}
    err = {}
    for name, (rup, rdn) in stacks.items():
        err[name] = {"image": rel_l2(got_img, rup[m] / rdn[m]), "illumination": rel_l2(sdn[m], rdn[m]),
                     "up_sum": rel_l2(sup[m], rup[m])}
    rup, rdn = stacks["ref_gpu"]
    dup, ddn = stacks["f64"]
    own = rel_l2(rup[m] / rdn[m], dup[m] / ddn[m])  # the reference's GPU build against FP64
    print("C3 windows %s, batched engine: vs reference GPU build %s; vs FP64 %s; reference GPU "
          "build vs FP64, image %.3e" % (list(zip(wx, ww)), err["ref_gpu"], err["f64"], own))
    assert max(err["ref_gpu"].values()) < 1e-4, err["ref_gpu"]
    assert err["f64"]["illumination"] < 1e-4 and err["f64"]["up_sum"] < 1e-3, err["f64"]
    assert err["f64"]["image"] <= own + 2e-4, (err["f64"], own)
