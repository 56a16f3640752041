"""Kernel-level drop-in entry points (rtm_k_*) against the oracle's restated
kernels, one call each on seeded random inputs, and the reference's per-shot
launch sequence (kernel.cu:798-933) run through them against the oracle's
driver loop.  Tolerance 1e-5 relative L2 per kernel call (FP32)."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as orc
from rtm_gpu_gb300 import capi
from util import interior, rel_l2, small_problem

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def vp(t):
    return C.c_void_p(t.data_ptr())


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _fields(p, seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((p.NZ, p.NX)).astype(np.float32) for _ in range(4)]


def test_add_and_bkadd(product_lib, cuda_ok):
    L = capi.lib()
    p = small_problem(adaptive=True)
    u0, u1, _, _ = _fields(p, 1)
    v = p.v
    exp = np.zeros_like(u0)
    orc.lib().or_add_f32.argtypes = None
    # oracle
    c = p.coef
    idx = p.index
    o = np.zeros(p.NZ * p.NX, np.float32)
    fn = orc.lib().or_add_f32
    fn(v.ctypes.data_as(C.c_void_p), o.ctypes.data_as(C.c_void_p), u0.ctypes.data_as(C.c_void_p),
       u1.ctypes.data_as(C.c_void_p), c.ctypes.data_as(C.c_void_p), idx.ctypes.data_as(C.c_void_p),
       C.c_int(1), C.c_float(p.tao2), C.c_float(p.h2), C.c_float(p.vmin), C.c_float(p.dv),
       C.c_int(p.M), C.c_int(p.NZ), C.c_int(p.NX), C.c_int(7), C.c_int(9), C.c_float(0.5),
       C.c_float(p.hzx2_1))
    dv_, d0, d1, d2 = dev(v), dev(u0), dev(u1), dev(exp)
    dc, di = dev(c), dev(idx)
    rc = L.rtm_k_Add(vp(dv_), vp(d2), vp(d0), vp(d1), vp(dc), vp(di), p.tao2, p.h2, p.vmin, p.dv,
                     p.M, p.NZ, p.NX, p.NZ * p.NX, 7, 9, 0.5, p.hzx2_1, None)
    assert rc == 0
    assert rel_l2(host(d2), o.reshape(p.NZ, p.NX)) < 1e-5


def test_reference_loop_through_dropin(product_lib, cuda_ok):
    """The reference's launch sequence, kernel for kernel, on the drop-in
    entry points (as a rewritten kernel.cu main would call them)."""
    L = capi.lib()
    for adaptive in (True, False):
        p = small_problem(adaptive=adaptive, NT=120)
        rng = np.random.default_rng(5)
        s_l, s_z, ds, n = p.rec_line
        seis = (rng.standard_normal((n, p.NT)) * 1e-2).astype(np.float32)
        seis[:, ::4] = 0
        o1, o2 = orc.migrate(p, seis)
        got1, got2 = run_reference_loop(L, p, seis)
        assert rel_l2(interior(p, got1), interior(p, o1)) < 1e-4
        assert rel_l2(interior(p, got2), interior(p, o2)) < 1e-4


def run_reference_loop(L, p, seis):
    NZ, NX, N2, M, NT = p.NZ, p.NX, p.N2, p.M, p.NT
    nz, nx = p.nz, p.nx
    z = lambda: torch.zeros((NZ, NX), dtype=torch.float32, device="cuda")
    FW0, FW1, FW2, FWb = z(), z(), z(), z()
    BW0, BW1, BW2 = z(), z(), z()
    FA, BA, R1, R2 = z(), z(), z(), z()
    lf = torch.zeros(M * nz * NT, device="cuda")
    rt = torch.zeros_like(lf)
    up = torch.zeros(M * nx * NT, device="cuda")
    dw = torch.zeros_like(up)
    v, r1, w = dev(p.v), dev(p.r1), dev(p.w)
    c, idx = dev(p.coef), dev(p.index)
    r_u, r_x = p.src_cell
    s_l, s_z, ds, n = p.rec_line
    s_r = (n - 1) * ds + s_l
    FW1[r_u, r_x] = p.spike
    ok = lambda rc: (_ for _ in ()).throw(RuntimeError(rc)) if rc else None
    ok(L.rtm_k_Equal(vp(lf), vp(rt), vp(up), vp(dw), vp(FW0), vp(FW1), NZ, NX, N2, M, None))
    for k in range(2, NT):
        wv = float(p.wav[k - 1]) if k < p.NT2 else 0.0
        if p.adaptive:
            ok(L.rtm_k_Add(vp(v), vp(FW2), vp(FW0), vp(FW1), vp(c), vp(idx), p.tao2, p.h2, p.vmin,
                           p.dv, M, NZ, NX, NZ * NX, r_u, r_x, wv, p.hzx2_1, None))
        else:
            ok(L.rtm_k_Add_Con(vp(v), vp(FW2), vp(FW0), vp(FW1), vp(c), p.tao2, p.h2, M, NZ, NX,
                               NZ * NX, r_u, r_x, wv, p.hzx2_1, None))
        args = [vp(FW1), vp(FW0), vp(FW2), vp(FWb), vp(lf), vp(rt), vp(up), vp(dw), vp(v), vp(r1),
                vp(w), NZ, NX, N2, M, k, p.taoh, p.taoh2, None]
        ok(L.rtm_k_Hybrid1(*args))
        ok(L.rtm_k_Hybrid2(*args))
        ok(L.rtm_k_Hybrid3(*args))
        ok(L.rtm_k_Deliver(vp(FW1), vp(FW0), vp(FW2), NZ, NX, None))
    BW0.copy_(FW1)
    BW1.copy_(FW0)
    src_spike = torch.zeros_like(FW0)
    src_spike[r_u, r_x] = p.spike
    if p.compen:
        BA.copy_(BW0 + BW1)
        FA.copy_(src_spike)
        R1.copy_(src_spike * BA)
        FW2.copy_(src_spike)
    else:
        R1.copy_(src_spike * BW1)
        FW2.zero_()
    R2.copy_(BW1 * BW1 + BW0 * BW0)
    FW0.zero_(); FW1.zero_(); FWb.zero_()
    dseis = torch.zeros(n, device="cuda")
    for k in range(NT - 3, -1, -1):
        wv = float(p.wav[k + 1]) if k < p.NT2 else 0.0
        ok(L.rtm_k_BKEqual(vp(lf), vp(rt), vp(up), vp(dw), vp(BW1), NZ, NX, N2, M, k, None))
        if p.adaptive:
            ok(L.rtm_k_BKAdd_EFF(vp(v), vp(BW2), vp(BW0), vp(BW1), vp(c), vp(idx), p.tao2, p.h2,
                                 p.vmin, p.dv, N2, NZ, NX, NZ * NX, r_u, r_x, wv, p.hzx2_1, None))
        else:
            ok(L.rtm_k_BKAdd_EFF_Con(vp(v), vp(BW2), vp(BW0), vp(BW1), vp(c), p.tao2, p.h2, N2, NZ,
                                     NX, NZ * NX, r_u, r_x, M, wv, p.hzx2_1, None))
        ok(L.rtm_k_Deliver_EFF(vp(BW1), vp(BW0), vp(BW2), N2, NZ, NX, None))
        dseis.copy_(torch.from_numpy(np.ascontiguousarray(seis[:, k + 1])))
        if p.adaptive:
            ok(L.rtm_k_BKAdd(vp(v), vp(FW2), vp(FW1), vp(FW0), vp(c), vp(idx), vp(dseis), p.tao2,
                             p.h2, p.vmin, p.dv, M, NZ, NX, NZ * NX, s_l, s_r, s_z, ds, p.hzx2_1,
                             None))
        else:
            ok(L.rtm_k_BKAdd_Con(vp(v), vp(FW2), vp(FW1), vp(FW0), vp(c), vp(dseis), p.tao2, p.h2,
                                 M, NZ, NX, NZ * NX, s_l, s_r, s_z, ds, p.hzx2_1, None))
        bargs = [vp(FW1), vp(FW0), vp(FW2), vp(FWb), vp(v), vp(r1), vp(w), NZ, NX, N2, p.taoh,
                 p.taoh2, None]
        ok(L.rtm_k_BKHybrid1(*bargs))
        ok(L.rtm_k_BKHybrid2(*bargs))
        ok(L.rtm_k_Deliver(vp(FW1), vp(FW0), vp(FW2), NZ, NX, None))
        if p.compen:
            ok(L.rtm_k_Rel_Compen(vp(FW2), vp(BW2), vp(FA), vp(BA), vp(R1), vp(R2), NZ, NX, None))
        else:
            ok(L.rtm_k_Rel_NonCompen(vp(FW2), vp(BW2), vp(R1), vp(R2), NZ, NX, None))
    return host(R1), host(R2)


def test_plain_shot_driver(product_lib, cuda_ok):
    """rtm_plain_migrate_shot (the reference's loop in C++ on the drop-in
    kernels) against the oracle."""
    from rtm_gpu_gb300.engine import plain_migrate_shot
    for adaptive, compen in ((True, True), (False, False)):
        p = small_problem(adaptive=adaptive, compen=compen, NT=120)
        rng = np.random.default_rng(8)
        seis = (rng.standard_normal((p.nrec, p.NT)) * 1e-2).astype(np.float32)
        o1, o2 = orc.migrate(p, seis)
        g1, g2 = plain_migrate_shot(p, p.src_flat(), seis)
        assert rel_l2(interior(p, g1), interior(p, o1)) < 1e-4
        assert rel_l2(interior(p, g2), interior(p, o2)) < 1e-4
