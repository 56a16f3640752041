"""Shot-level engine on the GPU against the CPU oracle (same seeded inputs).

Tolerance: relative L2 <= 1e-4 on the interior of rel1/rel2 and on gathers
(FP32 on both sides; the GPU contracts multiply-adds, the oracle does not).
"""
import numpy as np
import pytest

from oracle import oracle as orc
from rtm_gpu_gb300 import Engine, capi
from rtm_gpu_gb300.problem import build_problem, prep_taylor
from util import interior, layered_model, rel_l2, small_problem

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _seis(prob, seed=0):
    rng = np.random.default_rng(seed)
    s = (rng.standard_normal((prob.nrec, prob.NT)) * 1e-2).astype(np.float32)
    s[:, ::5] = 0.0  # zero samples are not injected (kernel.cu:351)
    return s


@pytest.mark.parametrize("adaptive", [True, False])
@pytest.mark.parametrize("compen", [True, False])
def test_migrate_one_shot(product_lib, cuda_ok, adaptive, compen):
    p = small_problem(adaptive=adaptive, compen=compen)
    seis = _seis(p)
    o1, o2 = orc.migrate(p, seis)
    with Engine(p, batch=1) as e:
        g1, g2 = e.migrate([p.src_flat()], seis[None])
    assert rel_l2(interior(p, g1[0]), interior(p, o1)) < TOL
    assert rel_l2(interior(p, g2[0]), interior(p, o2)) < TOL


def test_model_gathers(product_lib, cuda_ok):
    p = small_problem()
    ref = orc.model(p)
    with Engine(p, batch=1) as e:
        got = e.model([p.src_flat()])
    assert rel_l2(got[0], ref) < TOL


@pytest.mark.parametrize("M,eps_nt", [(8, 200), (12, 200)])
def test_taylor_long_operators(product_lib, cuda_ok, M, eps_nt):
    p = small_problem(adaptive=False, M=M, N2=M + 2, NT=eps_nt, nz=48, nx=150)
    seis = _seis(p, 3)
    o1, o2 = orc.migrate(p, seis)
    with Engine(p, batch=1) as e:
        g1, g2 = e.migrate([p.src_flat()], seis[None])
    assert rel_l2(interior(p, g1[0]), interior(p, o1)) < TOL
    assert rel_l2(interior(p, g2[0]), interior(p, o2)) < TOL


def _long_table(vmin, dv, nvel, need, hzx):
    """Per-bin table of the longest operators (Taylor coefficients of M=9 and
    M=10 on alternate bins): the least-squares optimiser's own M=10 designs
    on a test-sized grid come from ill-conditioned normal equations (|c| in
    the thousands) and blow up in the reference's own code as well."""
    taylor = {9: prep_taylor(9), 10: prep_taylor(10)}
    length = np.zeros(nvel, np.int32)
    index = np.zeros(nvel + 1, np.int32)
    coef, n = [], 0
    for b in range(nvel):
        index[b] = n
        if need[b]:
            c = taylor[10 if b % 2 else 9]
            length[b] = len(c) - 1
            coef.extend(c)
            n += len(c)
    index[nvel] = n
    return length, index, np.asarray(coef, np.float32)


def long_operator_problem():
    """Adaptive (per-bin) coefficients of operator length 9 and 10 -- the
    longest of the C5 range, run by the kernels' 12-wide instantiation."""
    N2, M, nz, nx, tao, h, f0 = 12, 10, 48, 150, 0.001, 10.0, 25.0
    vin = layered_model(nz, nx, 1500.0, 3500.0, 1)
    p = build_problem(vin, N2=N2, M=M, NT=160, h=h, tao=tao, f0=f0, adaptive=True, compen=True,
                      rec=(N2 + 1, N2, 0, 2, (nx + 1) // 2), coef_table=_long_table)
    assert set(np.diff(p.index)) == {0, 10, 11}
    return p.with_source(N2 + 2, N2 + nx // 2)


def test_adaptive_long_operators(product_lib, cuda_ok):
    p = long_operator_problem()
    seis = _seis(p, 5)
    o1, o2 = orc.migrate(p, seis)
    with Engine(p, batch=1) as e:
        g1, g2 = e.migrate([p.src_flat()], seis[None])
        rec = e.model([p.src_flat()])[0]
    assert rel_l2(interior(p, g1[0]), interior(p, o1)) < TOL
    assert rel_l2(interior(p, g2[0]), interior(p, o2)) < TOL
    assert rel_l2(rec, orc.model(p)) < TOL


def test_adaptive_long_operators_forms(product_lib, cuda_ok):
    p = long_operator_problem()
    srcs = [p.src_flat(p.N2 + 1, p.N2 + x) for x in (3, 77, 149)]
    seis = np.stack([_seis(p, s) for s in range(len(srcs))])
    out = []
    with Engine(p, batch=3) as e:
        for fwd, bwd in ((capi.RTM_KERNEL_TILED, capi.RTM_KERNEL_TILED),
                         (capi.RTM_KERNEL_PERSISTENT, capi.RTM_KERNEL_PERSISTENT),
                         (capi.RTM_KERNEL_X2_SPLIT, capi.RTM_KERNEL_SPLIT)):
            e.set_kernel(fwd, bwd)
            out.append(e.migrate(srcs, seis))
    for g in out[1:]:
        assert np.array_equal(g[0], out[0][0]) and np.array_equal(g[1], out[0][1])


def test_batch_of_shots_matches_single(product_lib, cuda_ok):
    p = small_problem(nx=150, nz=45)
    srcs = [p.src_flat(p.N2 + 1, p.N2 + x) for x in (3, 40, 77, 120, 149)]
    seis = np.stack([_seis(p, s) for s in range(len(srcs))])
    with Engine(p, batch=3) as e:  # 5 shots through a batch of 3 (uneven last group)
        g1, g2 = e.migrate(srcs, seis)
    for i, s in enumerate(srcs):
        q = p.with_source(s // p.NX, s % p.NX)
        o1, o2 = orc.migrate(q, seis[i])
        assert rel_l2(interior(p, g1[i]), interior(p, o1)) < TOL
        assert rel_l2(interior(p, g2[i]), interior(p, o2)) < TOL


def test_vertical_well_receivers(product_lib, cuda_ok):
    # reverse-VSP style geometry: receivers down a well column
    N2 = 8
    p = small_problem(nz=60, nx=70, rec=(N2 + 5, N2 + 30, 2, 0, 20))
    seis = _seis(p, 7)
    o1, o2 = orc.migrate(p, seis)
    with Engine(p, batch=1) as e:
        g1, g2 = e.migrate([p.src_flat()], seis[None])
    assert rel_l2(interior(p, g1[0]), interior(p, o1)) < TOL
    assert rel_l2(interior(p, g2[0]), interior(p, o2)) < TOL


def test_graph_and_stepwise_agree(product_lib, cuda_ok):
    p = small_problem()
    seis = _seis(p)
    with Engine(p, batch=1) as e:
        a1, a2 = e.migrate([p.src_flat()], seis[None], graph=True)
        b1, b2 = e.migrate([p.src_flat()], seis[None], graph=False)
    assert np.array_equal(a1, b1) and np.array_equal(a2, b2)


@pytest.mark.parametrize("vhi", [1800.0, 1797.37])  # the second has a non-integer maximum
def test_migrate_stack_matches_oracle(product_lib, cuda_ok, vhi):
    p = small_problem(nx=100, vhi=vhi)
    assert p.vmax >= float(p.v.max())  # snapped outward to the 1 m/s bin grid
    srcs = [p.src_flat(p.N2 + 1, p.N2 + x) for x in (10, 50, 90)]
    seis = np.stack([_seis(p, s) for s in range(len(srcs))])
    whitecoe = 1e-4
    ups, downs = [], []
    for i, s in enumerate(srcs):
        q = p.with_source(s // p.NX, s % p.NX)
        o1, o2 = orc.migrate(q, seis[i])
        u, d = orc.finish_shot(q, o1, o2, whitecoe)
        ups.append(u.T)   # oracle writes column-major [nx, nz]
        downs.append(d.T)
    img_o, ill_o = orc.stack(np.stack(ups), np.stack(downs), nrec=len(srcs), inorm=1, kahan=1)
    with Engine(p, batch=2) as e:
        gu = np.zeros((len(srcs), p.nz, p.nx), np.float32)
        gd = np.zeros_like(gu)
        img, ill = e.migrate_stack(srcs, seis, whitecoe, len(srcs), True, ups=gu, downs=gd)
    assert rel_l2(gu, np.stack(ups)) < TOL
    assert rel_l2(gd, np.stack(downs)) < TOL
    assert rel_l2(ill, ill_o) < TOL
    assert rel_l2(img, img_o) < TOL


def test_bounded_wait_gives_up_and_context_survives(product_lib, cuda_ok):
    """A wait that nothing completes ends with the timeout flag in the device
    error word (no hang, no trap); the next migration still runs and matches
    the oracle."""
    import ctypes as C
    from rtm_gpu_gb300 import capi
    code = C.c_uint(0)
    capi.check(capi.lib().rtm_selftest_wait_timeout(2000, C.byref(code)), "selftest")
    assert code.value == 1
    code2 = C.c_uint(7)
    capi.check(capi.lib().rtm_device_error(C.byref(code2)), "device_error")
    assert code2.value == 0  # read and cleared
    p = small_problem()
    seis = _seis(p)
    o1, o2 = orc.migrate(p, seis)
    with Engine(p, batch=1) as e:
        g1, g2 = e.migrate([p.src_flat()], seis[None])
    assert rel_l2(interior(p, g1[0]), interior(p, o1)) < TOL
