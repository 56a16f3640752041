"""Shot-level engine: the Python face of rtm_ctx_* / rtm_model_batch /
rtm_migrate_batch / rtm_migrate_stack (include/rtm_gb300.h).

Host arrays are numpy; device arrays may be passed as torch CUDA tensors
(flags=RTM_DEVICE_PTRS is then set automatically).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .problem import Problem


def _ptr(a):
    """(pointer, is_device) of a numpy array or torch tensor."""
    if isinstance(a, np.ndarray):
        assert a.dtype == np.float32 and a.flags.c_contiguous
        return C.c_void_p(a.ctypes.data), False
    # torch tensor
    assert a.is_contiguous() and str(a.dtype) == "torch.float32"
    return C.c_void_p(a.data_ptr()), a.is_cuda


class Engine:
    """A context for one model grid; shots advance `batch` at a time."""

    def __init__(self, prob: Problem, batch: int = 1, ring_precision: int = capi.RTM_RING_F32,
                 stream: int = 0):
        self.prob = prob
        self.batch = batch
        self._p = prob.c_struct(ring_precision)
        h = C.c_void_p()
        capi.check(capi.lib().rtm_ctx_create(C.byref(h), C.byref(self._p), batch,
                                             C.c_void_p(stream)), "ctx_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            capi.lib().rtm_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def device_bytes(self) -> int:
        n = C.c_size_t()
        capi.check(capi.lib().rtm_ctx_bytes(self._h, C.byref(n)), "ctx_bytes")
        return int(n.value)

    def set_kernel(self, fwd: int, bwd: int | None = None, shots_per_launch: int = 0):
        """Stencil kernel form per phase (capi.RTM_KERNEL_TILED / _PERSISTENT /
        _SPLIT; the forward also _X2 / _X2_SPLIT) and shots per launch (0: the
        context's batch)."""
        bwd = fwd if bwd is None else bwd
        capi.check(capi.lib().rtm_ctx_set_kernel(self._h, fwd, bwd, shots_per_launch), "set_kernel")

    def kernel(self):
        f, b, n = C.c_int(), C.c_int(), C.c_int()
        capi.check(capi.lib().rtm_ctx_get_kernel(self._h, C.byref(f), C.byref(b), C.byref(n)),
                   "get_kernel")
        return {"fwd": f.value, "bwd": b.value, "shots_per_launch": n.value}

    def set_snapshots(self, every: int, precision: int = capi.RTM_RING_F16):
        """Source snapshots every `every` steps (0: off) in RTM_RING_* storage:
        the backward run then advances the receiver field alone and images at
        the snapshot steps (rtm_ctx_set_snapshots)."""
        capi.check(capi.lib().rtm_ctx_set_snapshots(self._h, int(every), int(precision)), "set_snapshots")

    def snapshots(self):
        e, p, b = C.c_int(), C.c_int(), C.c_size_t()
        capi.check(capi.lib().rtm_ctx_get_snapshots(self._h, C.byref(e), C.byref(p), C.byref(b)),
                   "get_snapshots")
        return {"every": e.value, "precision": p.value, "bytes": b.value}

    def autotune(self, src_cells, win_x0=None, win_nx=None, nsteps: int = 20) -> float:
        """Times the kernel forms and shots per launch on the first shots of
        a survey, keeps the fastest; returns its Gcell-updates/s."""
        src = self._src(src_cells)
        x0 = None if win_x0 is None else np.ascontiguousarray(win_x0, np.int32)
        wn = None if win_nx is None else np.ascontiguousarray(win_nx, np.int32)
        rate = C.c_double()
        capi.check(capi.lib().rtm_ctx_autotune(self._h, len(src), capi.iptr(src),
                                               None if x0 is None else capi.iptr(x0),
                                               None if wn is None else capi.iptr(wn), nsteps,
                                               C.byref(rate)), "autotune")
        return rate.value

    def set_timing(self, on: bool):
        capi.check(capi.lib().rtm_ctx_set_timing(self._h, int(on)), "set_timing")

    def timing(self):
        ms = (C.c_double * 3)()
        n = (C.c_long * 3)()
        capi.check(capi.lib().rtm_ctx_timing(self._h, ms, n), "ctx_timing")
        return {"fwd_ms": ms[0], "bwd_ms": ms[1], "pad_ms": ms[2], "fwd_n": n[0], "bwd_n": n[1],
                "pad_n": n[2]}

    def launches(self, reset: bool = False) -> int:
        n = C.c_long()
        capi.check(capi.lib().rtm_ctx_launches(self._h, C.byref(n), int(reset)), "ctx_launches")
        return int(n.value)

    @staticmethod
    def _src(src_cells) -> np.ndarray:
        return np.ascontiguousarray(src_cells, np.int32)

    def model(self, src_cells, out=None, graph: bool = True):
        """Receiver gathers [nshot, nrec, NT] of the forward runs."""
        src = self._src(src_cells)
        p = self.prob
        if out is None:
            out = np.zeros((len(src), p.nrec, p.NT), np.float32)
        ptr, dev = _ptr(out)
        flags = (capi.RTM_DEVICE_PTRS if dev else 0) | (0 if graph else capi.RTM_NO_GRAPH)
        capi.check(capi.lib().rtm_model_batch(self._h, len(src), capi.iptr(src), ptr, flags),
                   "model_batch")
        return out

    def migrate(self, src_cells, seis, rel1=None, rel2=None, graph: bool = True):
        """Full-grid rel1/rel2 [nshot, NZ, NX] of each shot."""
        src = self._src(src_cells)
        p = self.prob
        n = len(src)
        if rel1 is None:
            rel1 = np.zeros((n, p.NZ, p.NX), np.float32)
        if rel2 is None:
            rel2 = np.zeros((n, p.NZ, p.NX), np.float32)
        sp, sdev = _ptr(seis)
        p1, d1 = _ptr(rel1)
        p2, d2 = _ptr(rel2)
        assert sdev == d1 == d2, "mix of host and device buffers"
        flags = (capi.RTM_DEVICE_PTRS if sdev else 0) | (0 if graph else capi.RTM_NO_GRAPH)
        capi.check(capi.lib().rtm_migrate_batch(self._h, n, capi.iptr(src), sp, p1, p2, flags),
                   "migrate_batch")
        return rel1, rel2

    def migrate_stack(self, src_cells, seis, whitecoe: float, nrec_div: int, inorm: bool,
                      image=None, illum=None, ups=None, downs=None, graph: bool = True):
        """Stacked interior image and illumination [nz, nx] (Kahan over shots)."""
        src = self._src(src_cells)
        p = self.prob
        if image is None:
            image = np.zeros((p.nz, p.nx), np.float32)
        if illum is None:
            illum = np.zeros((p.nz, p.nx), np.float32)
        sp, sdev = _ptr(seis)
        ip_, idev = _ptr(image)
        lp, ldev = _ptr(illum)
        assert sdev == idev == ldev, "mix of host and device buffers"
        up = _ptr(ups)[0] if ups is not None else None
        dp = _ptr(downs)[0] if downs is not None else None
        flags = (capi.RTM_DEVICE_PTRS if sdev else 0) | (0 if graph else capi.RTM_NO_GRAPH)
        capi.check(capi.lib().rtm_migrate_stack(self._h, len(src), capi.iptr(src), sp,
                                                whitecoe, int(nrec_div), int(inorm), ip_, lp, up,
                                                dp, flags), "migrate_stack")
        return image, illum

    def migrate_stack_windows(self, src_cells, win_x0, win_nx, seis, whitecoe: float,
                              nrec_div: int, inorm: bool, image=None, illum=None,
                              graph: bool = True):
        """Stacked survey image [nz, nx] of shots with their own aperture
        windows (interior columns [win_x0[i], win_x0[i]+win_nx[i])); sources
        are flat cells of each shot's own padded grid."""
        src = self._src(src_cells)
        x0 = np.ascontiguousarray(win_x0, np.int32)
        wn = np.ascontiguousarray(win_nx, np.int32)
        p = self.prob
        if image is None:
            image = np.zeros((p.nz, p.nx), np.float32)
        if illum is None:
            illum = np.zeros((p.nz, p.nx), np.float32)
        sp, sdev = _ptr(seis)
        ip_, idev = _ptr(image)
        lp, ldev = _ptr(illum)
        assert sdev == idev == ldev, "mix of host and device buffers"
        flags = (capi.RTM_DEVICE_PTRS if sdev else 0) | (0 if graph else capi.RTM_NO_GRAPH)
        capi.check(capi.lib().rtm_migrate_stack_windows(self._h, len(src), capi.iptr(src),
                                                        capi.iptr(x0), capi.iptr(wn), sp, whitecoe,
                                                        int(nrec_div), int(inorm), ip_, lp, flags),
                   "migrate_stack_windows")
        return image, illum


def plain_migrate_shot(prob: Problem, src_cell: int, seis):
    """The reference's per-shot launch sequence on the drop-in kernels
    (rtm_plain_migrate_shot): full padded rel1, rel2 [NZ, NX]."""
    p = prob.c_struct()
    seis = np.ascontiguousarray(seis, np.float32)
    rel1 = np.zeros((prob.NZ, prob.NX), np.float32)
    rel2 = np.zeros_like(rel1)
    capi.check(capi.lib().rtm_plain_migrate_shot(C.byref(p), int(src_cell), capi.fptr(seis),
                                                 capi.fptr(rel1), capi.fptr(rel2)),
               "plain_migrate_shot")
    return rel1, rel2
