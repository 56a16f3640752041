"""C-ABI library checks that need no GPU: it loads, exports every function
include/rtm_gb300.h declares, and its host-side preparation matches the
reference (golden fixtures) bit for bit."""
import os
import re

import numpy as np

from rtm_gpu_gb300 import capi, problem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def declared_functions():
    text = open(os.path.join(ROOT, "include", "rtm_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*?[\s\*]+(rtm_[A-Za-z0-9_]+)\s*\(",
                       text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(product_lib):
    names = declared_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(product_lib, n), n
    # one kernel-level entry point per reference kernel
    for k in capi.KERNEL_NAMES:
        assert "rtm_k_" + k in names


def test_prep_velocity_matches_reference(product_lib):
    G = dict(np.load(os.path.join(GOLD, "velocity_ricker.npz")))
    nx, nz = G["vin"].shape
    N2 = (G["v_flip0"].shape[0] - nz) // 2
    for flip in (0, 1):
        v, r1 = problem.prep_velocity(G["vin"], nz, nx, N2, np.float32(0.001), np.float32(10.0), flip)
        assert np.array_equal(v, G["v_flip%d" % flip])
        assert np.array_equal(r1, G["r1_flip%d" % flip])


def test_prep_wavelet_and_taylor_match_reference(product_lib):
    G = dict(np.load(os.path.join(GOLD, "velocity_ricker.npz")))
    for f0 in (20, 25):
        w = problem.prep_wavelet(len(G["ricker_t"]), 0.001, f0)
        assert np.array_equal(w, G["ricker_f%d" % f0])
    L = dict(np.load(os.path.join(GOLD, "lsm.npz")))
    for N in range(2, 22, 2):
        assert np.array_equal(problem.prep_taylor(N // 2), L["order_%d" % N])


def test_prep_bins_matches_oracle(product_lib):
    from oracle import oracle as orc
    rng = np.random.default_rng(3)
    v = rng.uniform(1512.3, 4480.7, (50, 70)).astype(np.float32)
    for dv in (1.0, 2.5, 10.0):
        a = problem.prep_bins(v, dv)
        b = orc.bin_velocity(v, dv)
        assert a[0] == b[0] and a[1] == b[1] and a[2] == b[2]
        assert np.array_equal(a[3], b[3])


def test_problem_constants_follow_reference_rounding():
    from util import small_problem
    p = small_problem(adaptive=False)
    f = np.float32
    assert p.tao2 == f(f(0.001) ** 2) or abs(p.tao2 - 1e-6) < 1e-12
    assert p.taoh == float(f(0.001) / f(10.0))
    assert p.NT2 == int(2.0 / float(f(25.0) * f(0.001))) + 1
    assert p.spike == float(f(float(p.wav[0]) / 2.0))
