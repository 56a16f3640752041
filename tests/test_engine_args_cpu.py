"""Argument checks of the shot-level engine that run before any device work
(so they need no GPU): invalid problems, receivers outside the grid,
operators longer than the kernels support or than the pad."""
import ctypes as C
import dataclasses

import numpy as np
import pytest

from rtm_gpu_gb300 import capi
from util import small_problem


def create(p, batch=1):
    s = p.c_struct()
    h = C.c_void_p()
    rc = capi.lib().rtm_ctx_create(C.byref(h), C.byref(s), batch, None)
    if rc == 0:
        capi.lib().rtm_ctx_destroy(h)
    return rc, capi.lib().rtm_last_error().decode()


@pytest.fixture(scope="module")
def prob():
    return small_problem(adaptive=False)


def test_batch_must_be_positive(product_lib, prob):
    assert create(prob, batch=0)[0] == -1


def test_operator_longer_than_pad(product_lib, prob):
    rc, msg = create(dataclasses.replace(prob, M=prob.N2 + 1))
    assert rc == -1 and "invalid problem" in msg


def test_too_few_steps(product_lib, prob):
    assert create(dataclasses.replace(prob, NT=3))[0] == -1


def test_receiver_step_zero(product_lib, prob):
    rc, msg = create(dataclasses.replace(prob, rec=(prob.N2 + 1, prob.N2, 0, 0, 4)))
    assert rc == -1 and "receiver step" in msg


def test_receiver_outside_grid(product_lib, prob):
    rc, msg = create(dataclasses.replace(prob, rec=(prob.N2 + 1, prob.N2, 0, 3, prob.nx)))
    assert rc == -1 and "receiver outside" in msg


def test_bad_ring_precision(product_lib, prob):
    s = prob.c_struct()
    s.ring_precision = 7
    h = C.c_void_p()
    assert capi.lib().rtm_ctx_create(C.byref(h), C.byref(s), 1, None) == -1


def test_null_arguments(product_lib):
    h = C.c_void_p()
    assert capi.lib().rtm_ctx_create(C.byref(h), None, 1, None) == -1
    assert capi.lib().rtm_ctx_create(None, None, 1, None) == -1
    assert capi.lib().rtm_ctx_autotune(None, 1, None, None, None, 10, None) == -1
    assert capi.lib().rtm_ctx_set_kernel(None, 0, 0, 0) == -1


def test_snapshot_calls_need_a_context(product_lib):
    """rtm_ctx_set_snapshots / rtm_ctx_get_snapshots reject a null context
    before any device work."""
    lib = capi.lib()
    assert lib.rtm_ctx_set_snapshots(None, 4, capi.RTM_RING_F16) == capi.RTM_ERR_ARG
    e, p, b = C.c_int(), C.c_int(), C.c_size_t()
    assert lib.rtm_ctx_get_snapshots(None, C.byref(e), C.byref(p), C.byref(b)) == capi.RTM_ERR_ARG
