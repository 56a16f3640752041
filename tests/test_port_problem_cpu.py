"""The oracle-port problem builder (used by bench.py's reference arm, which
must not load the product library) prepares the same problem as the
product's native preparation: padded model, bins, wavelet and Taylor table
bit for bit; an adaptive table equal to the oracle's funMandC restatement."""
import numpy as np

from oracle import oracle as orc
from oracle.port_problem import build_problem_port
from rtm_gpu_gb300.problem import build_problem, f32
from util import layered_model

KW = dict(N2=10, M=6, NT=64, h=12.5, tao=0.001, f0=25.0, compen=True, rec=(11, 10, 0, 1, 40))


def test_port_matches_product_prep_taylor(product_lib):
    vin = layered_model(30, 40, 1500.0, 3200.0, 9)
    a = build_problem_port(vin, adaptive=False, **KW)
    b = build_problem(vin, adaptive=False, **KW)
    for name in ("v", "r1", "w", "coef", "index", "length", "wav"):
        assert np.array_equal(getattr(a, name), getattr(b, name)), name
    assert (a.vmin, a.vmax, a.nvel) == (b.vmin, b.vmax, b.nvel)
    assert a.NT2 == b.NT2 and a.spike == b.spike


def test_port_adaptive_table_is_fun_m_and_c():
    vin = layered_model(30, 40, 1500.0, 1700.0, 3)
    a = build_problem_port(vin, adaptive=True, nthita=24, eps=1e-3, **KW)
    length, index, coef = orc.fun_m_and_c(24, KW["M"], 2, a.nvel, f32(KW["tao"]), f32(KW["h"]), 1.0,
                                          f32(1e-3), f32(2 * KW["f0"]), a.vmin, 1.0,
                                          orc.bin_velocity(a.v, 1.0)[3], 1.0)
    assert np.array_equal(a.length, length) and np.array_equal(a.index, index)
    assert np.array_equal(a.coef, coef)
