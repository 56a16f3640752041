"""Pins the CPU oracle to the reference: bit-for-bit equality with the golden
fixtures that tests/golden/make_golden.py produced from the reference's own
code (kernel.cu kernel bodies, LSMOrCon_rec_2D.cpp, GPU_velocity_real.cpp,
the Ricker function)."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import oracle as orc
from rtm_gpu_gb300.problem import Problem

GOLD = os.path.join(os.path.dirname(__file__), "golden")
F = C.c_float


def load(name):
    return dict(np.load(os.path.join(GOLD, name)))


def vp(a):
    return C.c_void_p(a.ctypes.data)


@pytest.fixture(scope="module")
def K():
    orc.set_threads(1)
    return load("kernels.npz")


def _c(a):
    return np.ascontiguousarray(a).copy()


def test_kernel_add(K):
    L = orc.lib()
    NZ, NX, M, N2 = int(K["NZ"]), int(K["NX"]), int(K["M"]), int(K["N2"])
    tao2, h2, hzx2_1, taoh, taoh2 = [float(x) for x in K["scal"]]
    for name, fn, adaptive, coef in (("out_Add", L.or_add_f32, 1, K["coef"]),
                                     ("out_Add_Con", L.or_add_f32, 0, K["ccon"])):
        o = _c(K["u2"])
        fn(vp(K["v"]), vp(o), vp(K["u0"]), vp(K["u1"]), vp(coef), vp(K["index"]), adaptive, F(tao2),
           F(h2), F(float(K["vmin"])), F(1.0), M, NZ, NX, 12, 20, F(0.7), F(hzx2_1))
        assert np.array_equal(o, K[name]), name
    for name, adaptive, coef in (("out_BKAdd_EFF", 1, K["coef"]), ("out_BKAdd_EFF_Con", 0, K["ccon"])):
        o = _c(K["u2"])
        L.or_bkadd_eff_f32(vp(K["v"]), vp(o), vp(K["u0"]), vp(K["u1"]), vp(coef), vp(K["index"]),
                           adaptive, F(tao2), F(h2), F(float(K["vmin"])), F(1.0), M, N2, NZ, NX, 12,
                           20, F(0.7), F(hzx2_1))
        assert np.array_equal(o, K[name]), name
    s_l, s_r, s_z, ds = [int(x) for x in K["line"]]
    for name, adaptive, coef in (("out_BKAdd", 1, K["coef"]), ("out_BKAdd_Con", 0, K["ccon"])):
        o = _c(K["u2"])
        L.or_bkadd_f32(vp(K["v"]), vp(o), vp(K["u1"]), vp(K["u0"]), vp(coef), vp(K["index"]),
                       adaptive, vp(K["seis"]), F(tao2), F(h2), F(float(K["vmin"])), F(1.0), M, NZ,
                       NX, s_l, s_r, s_z, ds, F(hzx2_1))
        assert np.array_equal(o, K[name]), name


def test_kernel_boundary_and_rings(K):
    L = orc.lib()
    NZ, NX, M, N2 = int(K["NZ"]), int(K["NX"]), int(K["M"]), int(K["N2"])
    tao2, h2, hzx2_1, taoh, taoh2 = [float(x) for x in K["scal"]]
    ob = _c(K["b"])
    L.or_hybrid1_f32(K["u1"], K["u0"], K["u2"], ob, K["v"], K["r1"], NZ, NX, N2, taoh, taoh2, 1)
    assert np.array_equal(ob, K["out_Hybrid1"])
    o = _c(K["u2"])
    L.or_hybrid2_f32(o, K["b"], K["w"], NZ, NX, N2)
    assert np.array_equal(o, K["out_Hybrid2"])
    rings = [_c(K[n]) for n in ("lf", "rt", "up", "dw")]
    L.or_ring_save_f32(*[vp(q) for q in rings], vp(K["u2"]), NZ, NX, N2, M, 4)
    assert np.array_equal(np.concatenate(rings), K["out_Hybrid3"])
    rings = [_c(K[n]) for n in ("lf", "rt", "up", "dw")]
    L.or_equal_f32(*[vp(q) for q in rings], vp(K["u0"]), vp(K["u1"]), NZ, NX, N2, M)
    assert np.array_equal(np.concatenate(rings), K["out_Equal"])
    o = _c(K["u1"])
    L.or_bkequal_f32(vp(K["lf"]), vp(K["rt"]), vp(K["up"]), vp(K["dw"]), vp(o), NZ, NX, N2, M, 2)
    assert np.array_equal(o, K["out_BKEqual"])
    for name, interior in (("out_Deliver", 0), ("out_Deliver_EFF", 1)):
        o1, o0 = _c(K["u1"]), _c(K["u0"])
        L.or_deliver_f32(vp(o1), vp(o0), vp(K["u2"]), NZ, NX, N2, interior)
        assert np.array_equal(np.stack([o1, o0]), K[name]), name


def test_kernel_imaging(K):
    L = orc.lib()
    NZ, NX = int(K["NZ"]), int(K["NX"])
    # source S = u2, receiver R = u1
    q1, q2 = _c(K["rel1"]), _c(K["rel2"])
    L.or_rel_f32(vp(K["u2"]), vp(K["u1"]), None, None, vp(q1), vp(q2), NZ, NX, 0)
    assert np.array_equal(np.stack([q1, q2]), K["out_Rel_NonCompen"])
    q1, q2, sa, ra = _c(K["rel1"]), _c(K["rel2"]), _c(K["sacc"]), _c(K["racc"])
    L.or_rel_f32(vp(K["u2"]), vp(K["u1"]), vp(sa), vp(ra), vp(q1), vp(q2), NZ, NX, 1)
    assert np.array_equal(np.stack([q1, q2, sa, ra]), K["out_Rel_Compen"])


def _shot_problem(S, compen):
    return Problem(nz=int(S["nz"]), nx=int(S["nx"]), N2=int(S["N2"]), M=int(S["M"]),
                   NT=int(S["NT"]), h=float(S["h"]), hz=float(S["h"]), tao=float(S["tao"]),
                   f0=float(S["f0"]), adaptive=True, compen=bool(compen), v=S["v"], r1=S["r1"],
                   w=S["w"], vmin=float(S["vmin"]), vmax=float(S["vmax"]), dv=1.0,
                   nvel=int(S["nvel"]), length=S["length"], index=S["index"], coef=S["coef"],
                   wav=S["wav"], rec=(int(S["N2"]) + 1, int(S["N2"]), 0, 2, (int(S["nx"]) + 1) // 2),
                   src_cell=(int(S["N2"]) + 2, int(S["N2"]) + int(S["nx"]) // 2))


def test_full_shot_bit_exact():
    S = load("shot.npz")
    orc.set_threads(2)
    for compen in (1, 0):
        p = _shot_problem(S, compen)
        r1, r2 = orc.migrate(p, S["seis_c%d" % compen])
        assert np.array_equal(r1, S["rel1_c%d" % compen])
        assert np.array_equal(r2, S["rel2_c%d" % compen])
    rec = orc.model(_shot_problem(S, 1))
    assert np.array_equal(rec, S["rec"])


def test_shot_list_geometry_equals_line():
    """The receiver-list form of the injection reproduces the line rule."""
    S = load("shot.npz")
    p = _shot_problem(S, 1)
    r1, r2 = orc.migrate(p, S["seis_c1"], force_list=True)
    assert np.array_equal(r1, S["rel1_c1"]) and np.array_equal(r2, S["rel2_c1"])


def test_fp64_oracle_close_to_fp32():
    S = load("shot.npz")
    p = _shot_problem(S, 1)
    d1, d2 = orc.migrate(p, S["seis_c1"], precision="f64")
    N2 = p.N2
    a, b = d1[N2:-N2, N2:-N2], S["rel1_c1"][N2:-N2, N2:-N2]
    assert np.linalg.norm(a - b) / np.linalg.norm(a) < 1e-3


def test_lsm_pins():
    G = load("lsm.npz")
    for N in range(2, 22, 2):
        assert np.array_equal(orc.taylor(N // 2), G["order_%d" % N]), N
    for (r, bb, M), ref in zip(G["cases"], G["coefs"]):
        M = int(M)
        assert np.array_equal(orc.ls_coefs(r, bb, M), ref[: M + 1]), (r, bb, M)
    c = np.zeros(7, np.float64)
    orc.lib().ls_coefs(c, 0.25, 2.2, 6, 1.6)
    assert np.array_equal(c, G["aniso"])
    for vel, ln in zip(G["callen_vel"], G["callen"]):
        got = orc.lib().ls_min_len(2, 10, float(vel), float(np.float32(0.001)),
                                   float(np.float32(10.0)), 1.0, 51, 40, 1e-4, 1.0)
        assert got == ln, vel
    L, I, Cf = orc.fun_m_and_c(40, 8, 2, 301, float(np.float32(0.001)), float(np.float32(10.0)),
                               1.0, 1e-4, 50.0, 1500.0, 1.0, G["table_need"], 1.0)
    assert np.array_equal(L, G["table_len"])
    assert np.array_equal(I, G["table_index"])
    assert np.array_equal(Cf, G["table_coef"])


def test_velocity_and_ricker_pins():
    G = load("velocity_ricker.npz")
    nx, nz = G["vin"].shape
    N2 = (G["v_flip0"].shape[0] - nz) // 2
    for flip in (0, 1):
        v, r1 = orc.pad_velocity(G["vin"], nz + 2 * N2, nx + 2 * N2, N2, np.float32(0.001),
                                 np.float32(10.0), flip)
        assert np.array_equal(v, G["v_flip%d" % flip])
        assert np.array_equal(r1, G["r1_flip%d" % flip])
    for f0 in (20, 25):
        got = np.array([orc.lib().or_ricker(float(t), float(f0)) for t in G["ricker_t"]], np.float32)
        assert np.array_equal(got, G["ricker_f%d" % f0])


@pytest.mark.skipif(not orc.ref_available(), reason="reference kernel fragments not built here")
def test_live_oracle_vs_reference_random_problem():
    """Beyond the fixtures: a fresh seeded problem through both."""
    from util import small_problem
    p = small_problem(seed=9, NT=90, nz=33, nx=41, N2=6, M=4, compen=True)
    rng = np.random.default_rng(2)
    seis = (rng.standard_normal((p.nrec, p.NT)) * 1e-2).astype(np.float32)
    a1, a2 = orc.migrate(p, seis)
    b1, b2 = orc.migrate(p, seis, use_ref=True)
    assert np.array_equal(a1, b1) and np.array_equal(a2, b2)


def test_resample_pins():
    """Trace resampling (Resample.cpp:193-225) bit for bit."""
    G = load("resample.npz")
    n = len([k for k in G if k.endswith("_param")])
    assert n >= 7
    for i in range(n):
        nxin, dxin, dxout, nxout = G["case%d_param" % i]
        got = orc.resample(G["case%d_in" % i], np.float32(dxin), int(nxout), np.float32(dxout))
        assert np.array_equal(got, G["case%d_out" % i]), i


def test_poststack_pins():
    """D2T / T2D / phase_correction (the reference's post-stack chain) bit
    for bit on the seeded traces of the fixture."""
    import hashlib
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden import poststack_inputs
    G = load("poststack.npz")
    seed, ntr, nz, dz, dt, nt, nz2 = G["params"]
    v, img = poststack_inputs(int(seed), int(ntr), int(nz))
    t = orc.depth_to_time(v, img, np.float32(dz), np.float32(dt))
    assert t.shape == (int(ntr), int(nt))
    assert np.array_equal(t[:2, :64], G["d2t_slice"])
    assert hashlib.sha256(t.tobytes()).digest() == G["d2t_sha"].tobytes()
    d = orc.time_to_depth(v, t, np.float32(dt), np.float32(dz))
    assert d.shape == (int(ntr), int(nz2))
    assert hashlib.sha256(d.tobytes()).digest() == G["t2d_sha"].tobytes()
    for i in range(3):
        ph = orc.phase_rotate(t, float(G["phase%d_angle" % i][0]))
        assert np.array_equal(ph[:2, :64], G["phase%d_slice" % i])
        assert hashlib.sha256(ph.tobytes()).digest() == G["phase%d_sha" % i].tobytes()
