"""The reference's own GPU kernels under the restated launch sequence
(oracle/_ref/libref_gpu.so, the yardstick of the bench's reference arm and
of tests/test_gpu_configs.py) against the same kernels run on the CPU
(oracle/_ref/libref_rtm.so): the two builds differ only in multiply-add
contraction, so on small grids they agree to about 1e-6."""
import numpy as np
import pytest

from oracle import oracle as orc
from util import interior, rel_l2, small_problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("adaptive,compen,rec", [
    (True, True, None), (False, True, None), (True, False, None),
    (True, True, (8 + 5, 8 + 30, 2, 0, 20)),   # a well: the receiver-list rule
])
def test_reference_gpu_build_matches_its_cpu_build(cuda_ok, adaptive, compen, rec):
    p = small_problem(adaptive=adaptive, compen=compen, nz=60, nx=70, rec=rec)
    rng = np.random.default_rng(21)
    seis = (rng.standard_normal((p.nrec, p.NT)) * 1e-2).astype(np.float32)
    seis[:, ::4] = 0.0
    g1, g2, sec = orc.ref_gpu_migrate(p, seis)
    c1, c2 = orc.migrate(p, seis, use_ref=True)
    assert sec > 0
    assert rel_l2(interior(p, g1), interior(p, c1)) < 1e-4
    assert rel_l2(interior(p, g2), interior(p, c2)) < 1e-4
