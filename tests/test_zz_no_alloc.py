"""rtm_k_HybridStatic: the absorbing-boundary update with its one-way
scratch in a fixed device array of the library, for callers that cannot
allocate device memory where they advance the wavefield.  Compared, through
the C ABI, with the caller-scratch pair rtm_k_Hybrid1 + rtm_k_Hybrid2 on two
calls in a row on different grids, on a pad of exactly the array's size
(1,048,576 cells, which must be accepted) and on a non-default stream.
Each call writes every scratch value it reads, so the second call checks
that the shared array carries nothing from the first that matters.  Kept
last in collection order."""
import ctypes as C

import numpy as np
import pytest

from rtm_gpu_gb300 import capi

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
TOL = 1e-6
LIMIT = 1 << 20  # pad cells the fixed scratch holds


def _case(NZ, NX, N2, seed):
    rng = np.random.default_rng(seed)
    f = lambda: torch.from_numpy(rng.standard_normal((NZ, NX)).astype(np.float32)).cuda()
    v = torch.from_numpy(rng.uniform(1500, 4500, (NZ, NX)).astype(np.float32)).cuda()
    r1 = v * 0.001 / 10.0 / np.sqrt(2.0)
    w = torch.from_numpy(np.array([i / N2 for i in range(N2 + 1)], np.float32)).cuda()
    return f(), f(), f(), v, r1.contiguous(), w


def _vp(t):
    return C.c_void_p(t.data_ptr())


def _bind(L):
    L.rtm_k_HybridStatic.argtypes = [C.c_void_p] * 6 + [C.c_int] * 3 + [C.c_float] * 2 + [C.c_void_p]
    L.rtm_last_error.restype = C.c_char_p


def _compare(L, NZ, NX, N2, seed, stream=None):
    """rel-L2 difference of the static-scratch update and the caller-scratch
    pair on one grid, both on `stream` (None: the legacy default stream)."""
    taoh, taoh2 = 1e-4, 5e-9
    u1, u0, u2, v, r1, w = _case(NZ, NX, N2, seed)
    ref2 = u2.clone()
    b = torch.zeros_like(u2)
    dummy = torch.zeros(1, device="cuda")
    sh = None if stream is None else C.c_void_p(stream.cuda_stream)
    torch.cuda.synchronize()
    args = [_vp(u1), _vp(u0), _vp(ref2), _vp(b), _vp(dummy), _vp(dummy), _vp(dummy), _vp(dummy),
            _vp(v), _vp(r1), _vp(w), NZ, NX, N2, 8, 3, taoh, taoh2, sh]
    assert L.rtm_k_Hybrid1(*args) == 0
    assert L.rtm_k_Hybrid2(*args) == 0
    got = u2.clone()
    torch.cuda.synchronize()
    rc = L.rtm_k_HybridStatic(_vp(u1), _vp(u0), _vp(got), _vp(v), _vp(r1), _vp(w), NZ, NX, N2,
                              taoh, taoh2, sh)
    assert rc == 0, L.rtm_last_error()
    torch.cuda.synchronize()
    return float((got - ref2).double().norm() / ref2.double().norm())


def test_static_scratch_matches_caller_scratch(product_lib, cuda_ok):
    L = capi.lib()
    _bind(L)
    for NZ, NX, N2, seed in ((461, 1261, 30, 1), (97, 131, 12, 2)):
        assert _compare(L, NZ, NX, N2, seed) <= TOL


def test_static_scratch_at_its_size_limit(product_lib, cuda_ok):
    L = capi.lib()
    _bind(L)
    NZ = NX = 4160
    N2 = 64  # 2*N2*(NZ+NX) - 4*N2^2 = 1,048,576 pad cells
    assert NZ * NX - (NZ - 2 * N2) * (NX - 2 * N2) == LIMIT
    assert _compare(L, NZ, NX, N2, 3) <= TOL


def test_static_scratch_on_a_side_stream(product_lib, cuda_ok):
    L = capi.lib()
    _bind(L)
    s = torch.cuda.Stream()
    assert _compare(L, 261, 461, 30, 4, stream=s) <= TOL


def test_static_scratch_rejects_oversized_pad(product_lib, cuda_ok):
    L = capi.lib()
    _bind(L)
    t = torch.zeros(1, device="cuda")
    # a 2000 x 2000 grid with a 200-cell pad has 1,440,000 pad cells
    rc = L.rtm_k_HybridStatic(*[_vp(t)] * 6, 2000, 2000, 200, 1e-4, 5e-9, None)
    assert rc == -1  # RTM_ERR_ARG
    assert b"fixed scratch" in L.rtm_last_error()
