"""The reference's post-stack chain on the GPU against the oracle: depth to
time and back bit for bit, phase rotation within the last bit of FP64 (two
bins take atan from a different math library)."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as orc
from rtm_gpu_gb300 import capi

pytestmark = pytest.mark.gpu


def _traces(seed, ntr, nz):
    rng = np.random.default_rng(seed)
    v = np.sort((1800.0 + rng.uniform(0, 2600, (ntr, nz))).astype(np.float32), axis=1)
    img = rng.standard_normal((ntr, nz)).astype(np.float32)
    return v, img


def gpu_d2t(v, img, dz, dt):
    L = capi.lib()
    ntr, nz = img.shape
    nt = C.c_int()
    capi.check(L.rtm_depth_to_time(capi.fptr(v), capi.fptr(img), ntr, nz, dz, dt, None, 0, C.byref(nt), 0),
               "depth_to_time")
    out = np.zeros((ntr, nt.value), np.float32)
    capi.check(L.rtm_depth_to_time(capi.fptr(v), capi.fptr(img), ntr, nz, dz, dt, capi.fptr(out), out.size,
                                   C.byref(nt), 0), "depth_to_time")
    return out


def gpu_t2d(v, img, dt, dz):
    L = capi.lib()
    ntr, nt = img.shape
    nz = C.c_int()
    capi.check(L.rtm_time_to_depth(capi.fptr(v), v.shape[1], capi.fptr(img), ntr, nt, dt, dz, None, 0,
                                   C.byref(nz), 0), "time_to_depth")
    out = np.zeros((ntr, nz.value), np.float32)
    capi.check(L.rtm_time_to_depth(capi.fptr(v), v.shape[1], capi.fptr(img), ntr, nt, dt, dz, capi.fptr(out),
                                   out.size, C.byref(nz), 0), "time_to_depth")
    return out


def gpu_phase(d, angle):
    d = np.ascontiguousarray(d, np.float32)
    out = np.zeros_like(d)
    capi.check(capi.lib().rtm_phase_rotate(capi.fptr(d), capi.fptr(out), d.shape[0], d.shape[1], angle, 0),
               "phase_rotate")
    return out


@pytest.mark.parametrize("ntr,nz,dz,dt", [(48, 700, 5.0, 0.003), (301, 401, 12.5, 0.001), (7, 33, 10.0, 0.002)])
def test_depth_time_round_trip_bit_exact(product_lib, cuda_ok, ntr, nz, dz, dt):
    v, img = _traces(ntr + nz, ntr, nz)
    dz, dt = np.float32(dz), np.float32(dt)
    t = gpu_d2t(v, img, dz, dt)
    assert np.array_equal(t, orc.depth_to_time(v, img, dz, dt))
    d = gpu_t2d(v, t, dt, dz)
    assert np.array_equal(d, orc.time_to_depth(v, t, dt, dz))


@pytest.mark.parametrize("angle", [90.0, 37.5, -60.0, 0.0])
@pytest.mark.parametrize("nt", [533, 1024, 6700])
def test_phase_rotation(product_lib, cuda_ok, angle, nt):
    rng = np.random.default_rng(nt)
    d = rng.standard_normal((17, nt)).astype(np.float32)
    got = gpu_phase(d, angle)
    exp = orc.phase_rotate(d, angle)
    scale = np.abs(exp).max()
    assert np.abs(got - exp).max() <= 1e-6 * scale
    assert np.mean(got == exp) > 0.99


def test_phase_rotation_rejects_long_traces(product_lib, cuda_ok):
    d = np.zeros((1, 9000), np.float32)
    o = np.zeros_like(d)
    assert capi.lib().rtm_phase_rotate(capi.fptr(d), capi.fptr(o), 1, 9000, 90.0, 0) == -5
