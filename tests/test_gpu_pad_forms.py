"""The column-streaming pad update (k_pad_cols, the default) against the
per-cell one (k_pad, chosen by RTM_PAD_CELLS=1 when a context is created):
the same cells, formulas and outputs, so migrations, recorded gathers and
stacks agree to rounding (measured: bit for bit) -- with FP32 and FP16
rings, a receiver line and a well, and uneven windows (per-shot pad
tables)."""
import os

import numpy as np
import pytest

from rtm_gpu_gb300 import Engine, capi
from util import rel_l2, small_problem

pytestmark = pytest.mark.gpu


def _run(cells, fn):
    old = os.environ.get("RTM_PAD_CELLS")
    os.environ["RTM_PAD_CELLS"] = "1" if cells else "0"
    try:
        return fn()
    finally:
        if old is None:
            del os.environ["RTM_PAD_CELLS"]
        else:
            os.environ["RTM_PAD_CELLS"] = old


def _close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    print("bit-identical" if np.array_equal(a, b) else "rel-L2 %.3e" % rel_l2(a, b))
    assert rel_l2(a, b) < 1e-6


@pytest.mark.parametrize("ring", [capi.RTM_RING_F32, capi.RTM_RING_F16])
@pytest.mark.parametrize("rec", [None, (8 + 5, 8 + 30, 2, 0, 20)])
def test_pad_forms_agree(product_lib, cuda_ok, ring, rec):
    p = small_problem(nz=60, nx=70, rec=rec)
    srcs = [p.src_flat(p.N2 + 1, p.N2 + x) for x in (3, 35, 66)]
    rng = np.random.default_rng(2)
    seis = (rng.standard_normal((3, p.nrec, p.NT)) * 1e-2).astype(np.float32)

    def go():
        with Engine(p, batch=3, ring_precision=ring) as e:
            g = e.model(srcs)
            r1, r2 = e.migrate(srcs, seis)
        return g, r1, r2

    a, b = _run(False, go), _run(True, go)
    for x, y in zip(a, b):
        _close(x, y)


def test_pad_forms_agree_on_windows(product_lib, cuda_ok):
    N2 = 8
    p = small_problem(nz=50, nx=160, N2=N2, M=4, NT=150, rec=(N2 + 4, N2 + 70, 2, 0, 18))
    wins = [(0, 160), (30, 90), (55, 100), (12, 120)]
    srcs = [(N2 + 1) * (nx + 2 * N2) + N2 + nx // 2 for _, nx in wins]
    rng = np.random.default_rng(9)
    seis = (rng.standard_normal((4, p.nrec, p.NT)) * 1e-2).astype(np.float32)

    def go():
        with Engine(p, batch=4, ring_precision=capi.RTM_RING_F16) as e:
            return e.migrate_stack_windows(srcs, [w[0] for w in wins], [w[1] for w in wins], seis,
                                           1e-4, 4, True)

    a, b = _run(False, go), _run(True, go)
    for x, y in zip(a, b):
        _close(x, y)
