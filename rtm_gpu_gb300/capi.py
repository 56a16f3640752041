"""ctypes binding of the engine's C ABI (include/rtm_gb300.h).

The library is the in-tree build rtm_gpu_gb300/_lib/librtm_gb300.so; loading
fails loudly when it is missing -- there is no other implementation to fall
back to.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _build

_lib = None

RTM_OK = 0
RTM_ERR_ARG, RTM_ERR_CUDA, RTM_ERR_NOMEM, RTM_ERR_DEVICE = -1, -2, -3, -4
RTM_DEVICE_PTRS = 1
RTM_NO_GRAPH = 2
RTM_RING_F32, RTM_RING_BF16, RTM_RING_F16, RTM_RING_I16 = 0, 1, 2, 3
RTM_KERNEL_TILED, RTM_KERNEL_PERSISTENT, RTM_KERNEL_SPLIT, RTM_KERNEL_X2, RTM_KERNEL_X2_SPLIT = 0, 1, 2, 3, 4

vp = C.c_void_p
fp = C.POINTER(C.c_float)
ip = C.POINTER(C.c_int)
I = C.c_int
F = C.c_float


class RtmProblem(C.Structure):
    """Mirror of struct rtm_problem."""

    _fields_ = [(n, C.c_int) for n in ("nz", "nx", "N2", "M", "NT", "NT2", "adaptive", "compen",
                                       "quirk", "nbins")] + \
        [(n, C.c_float) for n in ("tao2", "h2", "taoh", "taoh2", "vmin", "dv", "hzx2_1", "spike")] + \
        [("v", fp), ("r1", fp), ("w", fp), ("coef", fp), ("index", ip), ("wav", fp)] + \
        [(n, C.c_int) for n in ("rz0", "rx0", "rdz", "rdx", "nrec", "ring_precision")]


# argument lists of the kernel-level entry points (reference kernel.cu order)
_KSIG = {
    "Equal": [vp] * 6 + [I] * 4,
    "Add": [vp] * 5 + [vp, F, F, F, F, I, I, I, I, I, I, F, F],
    "Add_Con": [vp] * 5 + [F, F, I, I, I, I, I, I, F, F],
    "Hybrid1": [vp] * 11 + [I, I, I, I, I, F, F],
    "Hybrid2": [vp] * 11 + [I, I, I, I, I, F, F],
    "Hybrid3": [vp] * 11 + [I, I, I, I, I, F, F],
    "Deliver": [vp] * 3 + [I, I],
    "BKEqual": [vp] * 5 + [I] * 5,
    "BKAdd_EFF": [vp] * 5 + [vp, F, F, F, F, I, I, I, I, I, I, F, F],
    "BKAdd_EFF_Con": [vp] * 5 + [F, F, I, I, I, I, I, I, I, F, F],
    "Deliver_EFF": [vp] * 3 + [I, I, I],
    "BKAdd": [vp] * 5 + [vp, vp, F, F, F, F, I, I, I, I, I, I, I, I, F],
    "BKAdd_Con": [vp] * 5 + [vp, F, F, I, I, I, I, I, I, I, I, F],
    "BKHybrid1": [vp] * 7 + [I, I, I, F, F],
    "BKHybrid2": [vp] * 7 + [I, I, I, F, F],
    "Rel_NonCompen": [vp] * 4 + [I, I],
    "Rel_Compen": [vp] * 6 + [I, I],
}
KERNEL_NAMES = tuple(_KSIG)


def lib_path() -> str:
    return _build.LIB


def lib():
    """The loaded C-ABI library.  Raises if it has not been built."""
    global _lib
    if _lib is None:
        path = os.environ.get("RTM_GB300_LIB") or _build.LIB  # override: a library built elsewhere
        if not os.path.exists(path):
            raise RuntimeError(
                "rtm_gpu_gb300: native library %s is missing; run "
                "`python -c 'import __graft_entry__ as g; g.build()'` first" % path)
        L = C.CDLL(path)
        L.rtm_last_error.restype = C.c_char_p
        L.rtm_version.restype = C.c_int
        L.rtm_device_error.argtypes = [C.POINTER(C.c_uint)]
        for name, sig in _KSIG.items():
            f = getattr(L, "rtm_k_" + name)
            f.argtypes = sig + [vp]
            f.restype = C.c_int
        L.rtm_prep_velocity.argtypes = [fp, I, I, I, F, F, I, fp, fp]
        L.rtm_prep_bins.argtypes = [fp, C.c_long, F, fp, fp, ip, ip, I]
        L.rtm_prep_wavelet.argtypes = [fp, I, F, F]
        L.rtm_prep_taylor.argtypes = [I, fp]
        L.rtm_ctx_create.argtypes = [C.POINTER(vp), C.POINTER(RtmProblem), I, vp]
        L.rtm_ctx_destroy.argtypes = [vp]
        L.rtm_ctx_bytes.argtypes = [vp, C.POINTER(C.c_size_t)]
        L.rtm_model_batch.argtypes = [vp, I, ip, vp, I]
        L.rtm_migrate_batch.argtypes = [vp, I, ip, vp, vp, vp, I]
        L.rtm_migrate_stack.argtypes = [vp, I, ip, vp, F, I, I, vp, vp, vp, vp, I]
        L.rtm_migrate_stack_windows.argtypes = [vp, I, ip, ip, ip, vp, F, I, I, vp, vp, I]
        L.rtm_plain_migrate_shot.argtypes = [C.POINTER(RtmProblem), I, fp, fp, fp]
        L.rtm_ctx_timing.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_long)]
        L.rtm_ctx_set_timing.argtypes = [vp, I]
        L.rtm_ctx_launches.argtypes = [vp, C.POINTER(C.c_long), I]
        L.rtm_ctx_set_kernel.argtypes = [vp, I, I, I]
        L.rtm_ctx_get_kernel.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.rtm_ctx_set_snapshots.argtypes = [vp, I, I]
        L.rtm_ctx_get_snapshots.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_size_t)]
        L.rtm_ctx_autotune.argtypes = [vp, I, ip, ip, ip, I, C.POINTER(C.c_double)]
        L.rtm_resample.argtypes = [fp, I, I, C.c_float, fp, I, C.c_float, I]
        L.rtm_selftest_wait_timeout.argtypes = [C.c_uint, C.POINTER(C.c_uint)]
        L.rtm_run_config.argtypes = [C.c_char_p, I]
        L.rtm_depth_to_time.argtypes = [fp, fp, I, I, C.c_float, C.c_float, fp, C.c_long,
                                        C.POINTER(C.c_int), I]
        L.rtm_time_to_depth.argtypes = [fp, I, fp, I, I, C.c_float, C.c_float, fp, C.c_long,
                                        C.POINTER(C.c_int), I]
        L.rtm_phase_rotate.argtypes = [fp, fp, I, I, C.c_float, I]
        L.rtm_write_segy.argtypes = [C.c_char_p, C.c_char_p, fp, I, I, C.c_float, fp, fp, C.c_float,
                                     C.c_float, fp]
        _lib = L
    return _lib


def check(rc: int, what: str = "") -> None:
    if rc != RTM_OK:
        msg = lib().rtm_last_error().decode(errors="replace")
        raise RuntimeError("rtm %s failed (status %d): %s" % (what, rc, msg))


def fptr(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(fp)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(ip)
