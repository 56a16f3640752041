"""rtm_k_HybridStatic: the absorbing-boundary update with its one-way
scratch in a fixed device array of the library, for callers that cannot
allocate device memory where they advance the wavefield.  Compared, through
the C ABI, with the caller-scratch pair rtm_k_Hybrid1 + rtm_k_Hybrid2 on two
calls in a row (the second on a smaller grid, so stale scratch contents from
the first call would show).  Kept last in collection order."""
import ctypes as C

import numpy as np
import pytest

from rtm_gpu_gb300 import capi

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
TOL = 1e-6


def _case(NZ, NX, N2, seed):
    rng = np.random.default_rng(seed)
    f = lambda: torch.from_numpy(rng.standard_normal((NZ, NX)).astype(np.float32)).cuda()
    v = torch.from_numpy(rng.uniform(1500, 4500, (NZ, NX)).astype(np.float32)).cuda()
    r1 = v * 0.001 / 10.0 / np.sqrt(2.0)
    w = torch.from_numpy(np.array([i / N2 for i in range(N2 + 1)], np.float32)).cuda()
    return f(), f(), f(), v, r1.contiguous(), w


def _vp(t):
    return C.c_void_p(t.data_ptr())


def test_static_scratch_matches_caller_scratch(product_lib, cuda_ok):
    L = capi.lib()
    L.rtm_k_HybridStatic.argtypes = [C.c_void_p] * 6 + [C.c_int] * 3 + [C.c_float] * 2 + [C.c_void_p]
    taoh, taoh2 = 1e-4, 5e-9
    for NZ, NX, N2, seed in ((461, 1261, 30, 1), (97, 131, 12, 2)):
        u1, u0, u2, v, r1, w = _case(NZ, NX, N2, seed)
        ref2 = u2.clone()
        b = torch.zeros_like(u2)
        dummy = torch.zeros(1, device="cuda")
        args = [_vp(u1), _vp(u0), _vp(ref2), _vp(b), _vp(dummy), _vp(dummy), _vp(dummy), _vp(dummy),
                _vp(v), _vp(r1), _vp(w), NZ, NX, N2, 8, 3, taoh, taoh2, None]
        assert L.rtm_k_Hybrid1(*args) == 0
        assert L.rtm_k_Hybrid2(*args) == 0
        got = u2.clone()
        rc = L.rtm_k_HybridStatic(_vp(u1), _vp(u0), _vp(got), _vp(v), _vp(r1), _vp(w), NZ, NX, N2,
                                  taoh, taoh2, None)
        assert rc == 0, L.rtm_last_error()
        torch.cuda.synchronize()
        d = (got - ref2).double().norm() / ref2.double().norm()
        assert float(d) <= TOL


def test_static_scratch_rejects_oversized_pad(product_lib, cuda_ok):
    L = capi.lib()
    L.rtm_k_HybridStatic.argtypes = [C.c_void_p] * 6 + [C.c_int] * 3 + [C.c_float] * 2 + [C.c_void_p]
    t = torch.zeros(1, device="cuda")
    # a 2000 x 2000 grid with a 200-cell pad has 1,440,000 pad cells
    rc = L.rtm_k_HybridStatic(*[_vp(t)] * 6, 2000, 2000, 200, 1e-4, 5e-9, None)
    assert rc == -1  # RTM_ERR_ARG
    assert b"fixed scratch" in L.rtm_last_error()
