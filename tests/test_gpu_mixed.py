"""Mixed-precision boundary rings (BF16 / FP16 / scaled int16 with per-step
max-abs scaling; stencil and imaging stay FP32) against the FP64 oracle, on a small
case (80x160, 500 steps) whose random gathers put energy at every
wavenumber.  Errors are relative L2 on the interior cross-correlation (rel1)
and illumination (rel2) after one migration.  Target: NRMSE <= 1e-3 against
FP64 (the FP32 arithmetic alone accounts for ~3e-4 here); FP16 rings meet
it, BF16 rings (8-bit mantissa) land near 2e-3 here and are held to 5e-3;
int16 rings (fractions of each step's largest value) meet 1e-3.
(At full size with modelled gathers, one shot of the 401x1201 workload, the
finished image is within 7.7e-4 of FP64 for FP32 and FP16 rings and 7.0e-4
for BF16: tests/test_gpu_configs.py and the bench line's nrmse_vs_fp64.)"""
import numpy as np
import pytest

from oracle import oracle as orc
from rtm_gpu_gb300 import Engine, capi
from util import interior, rel_l2, small_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    p = small_problem(adaptive=False, M=8, N2=16, nz=80, nx=160, NT=500, vlo=1800, vhi=3200,
                      smooth=3.0)
    rng = np.random.default_rng(4)
    seis = (rng.standard_normal((p.nrec, p.NT)) * 1e-2).astype(np.float32)
    d1, d2 = orc.migrate(p, seis, precision="f64")
    return p, seis, d1, d2


@pytest.mark.parametrize("prec,tol", [(capi.RTM_RING_F32, 1e-3), (capi.RTM_RING_F16, 1e-3),
                                      (capi.RTM_RING_BF16, 5e-3), (capi.RTM_RING_I16, 1e-3)])
def test_ring_precision_vs_fp64(product_lib, cuda_ok, case, prec, tol):
    p, seis, d1, d2 = case
    with Engine(p, batch=2, ring_precision=prec) as e:
        g1, g2 = e.migrate([p.src_flat()] * 2, np.stack([seis, seis]))
    e1 = rel_l2(interior(p, g1[0]), interior(p, d1))
    e2 = rel_l2(interior(p, g2[0]), interior(p, d2))
    print("ring precision %d: image rel-L2 %.3e, illumination %.3e" % (prec, e1, e2))
    assert e1 <= tol and e2 <= tol
    assert np.array_equal(g1[0], g1[1])  # shots of a batch are independent


@pytest.mark.parametrize("prec", [capi.RTM_RING_BF16, capi.RTM_RING_I16])
def test_ring_bytes_halved(product_lib, cuda_ok, case, prec):
    p = case[0]
    with Engine(p, batch=1, ring_precision=capi.RTM_RING_F32) as a, \
            Engine(p, batch=1, ring_precision=prec) as b:
        ring32 = p.NT * 2 * p.M * (p.nz + p.nx) * 4
        assert a.device_bytes - b.device_bytes >= 0.45 * ring32


@pytest.mark.parametrize("prec", [capi.RTM_RING_F32, capi.RTM_RING_F16, capi.RTM_RING_BF16,
                                  capi.RTM_RING_I16])
def test_gathers_vs_fp64(product_lib, cuda_ok, case, prec):
    """Shot gathers of the forward run against the FP64 oracle for each ring
    storage precision (the rings enter only the backward run, so the
    gathers carry the FP32 arithmetic's error alone)."""
    p = case[0]
    ref = orc.model(p, precision="f64")
    with Engine(p, batch=1, ring_precision=prec) as e:
        g = e.model([p.src_flat()])[0]
    err = rel_l2(g, ref)
    print("ring precision %d: gather rel-L2 %.3e" % (prec, err))
    assert err <= 1e-3
