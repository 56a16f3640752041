"""ctypes front end of the CPU oracle (and of the reference's own CPU code).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and
the CPU-baseline leg of bench.py; the product package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_ref as _b

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


class Params(C.Structure):
    """Mirror of or_params (oracle/rtm_oracle.h)."""

    _fields_ = [(n, C.c_int) for n in (
        "NZ", "NX", "N2", "M", "NT", "NT2", "adaptive", "compen", "quirk", "r_u", "r_x",
        "s_l", "s_r", "s_z", "ds", "n", "nrec_list", "pad_")] + \
        [(n, C.c_float) for n in ("tao2", "h2", "taoh", "taoh2", "vmin", "dv", "hzx2_1", "spike")] + \
        [("rec_cells", C.POINTER(C.c_int))]


_lib = None
_ref = None
_refp = None
_refh = None
_refg = None


def lib():
    global _lib
    if _lib is None:
        path = _b.build_oracle()
        L = C.CDLL(path)
        for sfx, rp in (("f32", _f32p), ("f64", _f64p)):
            getattr(L, "or_migrate_" + sfx).argtypes = [C.POINTER(Params), _f32p, _f32p, _f32p,
                                                        _f32p, _i32p, _f32p, _f32p, rp, rp]
            getattr(L, "or_model_" + sfx).argtypes = [C.POINTER(Params), _f32p, _f32p, _f32p,
                                                      _f32p, _i32p, _f32p, rp]
            getattr(L, "or_hybrid1_" + sfx).argtypes = [rp, rp, rp, rp, _f32p, _f32p, C.c_int,
                                                        C.c_int, C.c_int, C.c_float, C.c_float,
                                                        C.c_int]
            getattr(L, "or_hybrid2_" + sfx).argtypes = [rp, rp, _f32p, C.c_int, C.c_int, C.c_int]
        L.or_ricker.restype = C.c_float
        L.or_ricker.argtypes = [C.c_float, C.c_float]
        L.or_wavelet_table.argtypes = [_f32p, C.c_int, C.c_float, C.c_float]
        L.or_pad_velocity.argtypes = [_f32p, _f32p, _f32p, C.c_int, C.c_int, C.c_int, C.c_float,
                                      C.c_float, C.c_int]
        L.or_bin_velocity.argtypes = [_f32p, C.c_long, C.c_float, C.POINTER(C.c_float),
                                      C.POINTER(C.c_float), C.c_void_p, C.c_int]
        L.or_finish_shot_f32.argtypes = [_f32p, _f32p, _f32p, C.c_int, C.c_int, C.c_int, C.c_float,
                                         C.c_float, _f32p, _f32p]
        L.or_finish_shot_f64.argtypes = [_f64p, _f64p, _f32p, C.c_int, C.c_int, C.c_int, C.c_float,
                                         C.c_float, _f64p, _f64p]
        L.or_stack_f32.argtypes = [_f32p, _f32p, C.c_int, C.c_long, C.c_int, C.c_int, C.c_int, _f32p,
                                   _f32p]
        L.or_stack_f64.argtypes = [_f64p, _f64p, C.c_int, C.c_long, C.c_int, C.c_int, _f64p, _f64p]
        L.ls_quad.restype = C.c_double
        L.ls_quad.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double]
        L.ls_coefs.argtypes = [_f64p, C.c_double, C.c_double, C.c_int, C.c_double]
        L.ls_min_len.restype = C.c_int
        L.ls_min_len.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_int, C.c_int, C.c_double, C.c_double]
        L.ls_len_passes.argtypes = [_f64p, C.c_int, C.c_double, _f64p, C.c_int, C.c_int, C.c_double,
                                    C.c_double, C.c_double]
        L.ls_fun_m_and_c.restype = C.c_int
        L.ls_fun_m_and_c.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                     C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                     _i32p, _i32p, _i32p, C.c_void_p, C.c_int, C.c_double]
        L.ls_taylor.argtypes = [C.c_int, _f32p]
        L.or_resample.argtypes = [C.c_int, C.c_float, _f32p, C.c_int, C.c_float, _f32p]
        L.or_d2t.restype = C.c_int
        L.or_d2t.argtypes = [_f32p, _f32p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_void_p, C.c_long]
        L.or_t2d.restype = C.c_int
        L.or_t2d.argtypes = [_f32p, C.c_int, _f32p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_void_p,
                             C.c_long]
        L.or_phase.argtypes = [_f32p, _f32p, C.c_int, C.c_int, C.c_float]
        L.rs_table.argtypes = [_f32p]
        L.or_set_threads.argtypes = [C.c_int]
        L.or_get_threads.restype = C.c_int
        _lib = L
    return _lib


def ref_available() -> bool:
    try:
        return "kernels" in _b.build_ref()
    except Exception:
        return False


def ref():
    """The reference's kernel bodies on the CPU (oracle/_ref/libref_rtm.so)."""
    global _ref
    if _ref is None:
        got = _b.build_ref()
        if "kernels" not in got:
            raise RuntimeError("reference kernel fragments unavailable (no checkout, no oracle/_ref)")
        L = C.CDLL(got["kernels"])
        L.ref_migrate.argtypes = [C.POINTER(Params), _f32p, _f32p, _f32p, _f32p, _i32p, _f32p,
                                  _f32p, _f32p, _f32p]
        L.ref_model.argtypes = [C.POINTER(Params), _f32p, _f32p, _f32p, _f32p, _i32p, _f32p, _f32p]
        L.ref_ricker.restype = C.c_float
        L.ref_ricker.argtypes = [C.c_float, C.c_float]
        _ref = L
    return _ref


def ref_gpu():
    """The reference's kernels on the GPU (oracle/_ref/libref_gpu.so)."""
    global _refg
    if _refg is None:
        L = C.CDLL(_b.build_ref_gpu())
        L.refgpu_migrate.restype = C.c_int
        L.refgpu_migrate.argtypes = [C.POINTER(Params), _f32p, _f32p, _f32p, _f32p, _i32p, C.c_int,
                                     C.c_int, _f32p, _f32p, _f32p, _f32p, C.POINTER(C.c_double)]
        _refg = L
    return _refg


def ref_gpu_migrate(prob, seis):
    """rel1, rel2 (full padded grid) and the wall-clock seconds of one shot on
    the reference's own GPU kernels with its per-shot launch sequence
    (kernel.cu:798-933).  Receivers other than the reference's surface line
    are injected by the line's rule after BKAdd, as the oracle's driver does."""
    P = make_params(prob, int(getattr(prob, "quirk", True)))
    rel1 = np.zeros(prob.NZ * prob.NX, np.float32)
    rel2 = np.zeros(prob.NZ * prob.NX, np.float32)
    sec = C.c_double()
    nvel = int(prob.nvel) if prob.adaptive else 0
    coef = np.ascontiguousarray(prob.coef, np.float32)
    rc = ref_gpu().refgpu_migrate(C.byref(P), prob.v.ravel(), prob.r1.ravel(), prob.w, coef,
                                  np.ascontiguousarray(prob.index, np.int32), nvel, int(coef.size),
                                  prob.wav, np.ascontiguousarray(seis, np.float32).ravel(), rel1,
                                  rel2, C.byref(sec))
    if rc != 0:
        raise RuntimeError("reference GPU migrate failed")
    return rel1.reshape(prob.NZ, prob.NX), rel2.reshape(prob.NZ, prob.NX), float(sec.value)


def ref_host():
    """LSMOrCon_rec_2D.cpp / GPU_velocity_real.cpp compiled from the checkout."""
    global _refh
    if _refh is None:
        got = _b.build_ref()
        if "host" not in got:
            raise RuntimeError("reference checkout unavailable")
        L = C.CDLL(got["host"])
        L.ref_order.argtypes = [C.c_int, _f32p]
        L.ref_cal2dfdcoe.argtypes = [_f64p, C.c_double, C.c_double, C.c_int, C.c_double]
        L.ref_callenfd.restype = C.c_int
        L.ref_callenfd.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                   C.c_double, C.c_int, C.c_int, C.c_double, C.c_double]
        L.ref_funMandC.restype = C.c_int
        L.ref_funMandC.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                   C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                   C.c_double, _i32p, _i32p, _i32p, _f32p, C.c_int, C.c_double]
        L.ref_velocity.argtypes = [C.c_char_p, _f32p, _f32p, _f32p, _f32p, _f32p, C.c_int, C.c_int,
                                   C.c_int, C.c_float, C.c_float, C.c_int]
        L.ref_resample.argtypes = [C.c_int, C.c_float, _f32p, C.c_int, C.c_float, _f32p]
        _refh = L
    return _refh


def ref_post():
    """DisToTimeAndTimeToDis1D.cpp / phase_correction_ricker_decon.cpp
    compiled from the checkout."""
    global _refp
    if _refp is None:
        got = _b.build_ref()
        if "post" not in got:
            raise RuntimeError("reference checkout unavailable")
        L = C.CDLL(got["post"])
        L.ref_d2t.restype = C.c_int
        L.ref_d2t.argtypes = [C.c_char_p, _f32p, _f32p, C.c_int, C.c_int, C.c_float, C.c_float,
                              C.c_float, _f32p, C.c_long]
        L.ref_t2d.restype = C.c_int
        L.ref_t2d.argtypes = [C.c_char_p, _f32p, _f32p, C.c_int, C.c_int, C.c_int, C.c_float,
                              C.c_float, C.c_float, _f32p, C.c_long]
        L.ref_phase_correction.argtypes = [_f32p, _f32p, C.c_int, C.c_int, C.c_float]
        _refp = L
    return _refp


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


def get_threads() -> int:
    return int(lib().or_get_threads())


# ---------------------------------------------------------------------------
# convenience wrappers (numpy in / numpy out)


def make_params(prob, quirk: int = 1, force_list: bool = False) -> Params:
    """or_params from a problem description (rtm_gpu_gb300.problem.Problem or
    any object with the same attributes).  A surface-line geometry uses the
    reference's line rule unless force_list; any other geometry is passed as
    an explicit receiver list."""
    P = Params()
    P.NZ, P.NX, P.N2, P.M = prob.NZ, prob.NX, prob.N2, prob.M
    P.NT, P.NT2 = prob.NT, prob.NT2
    P.adaptive = 1 if prob.adaptive else 0
    P.compen = 1 if prob.compen else 0
    P.quirk = quirk
    P.r_u, P.r_x = prob.src_cell
    if prob.rec_line is not None and not force_list:
        P.s_l, P.s_z, P.ds, P.n = prob.rec_line
        P.s_r = (P.n - 1) * P.ds + P.s_l
        P.nrec_list = 0
        P.rec_cells = C.POINTER(C.c_int)()
    else:
        P.s_l, P.s_r, P.s_z, P.ds, P.n = 1, 0, -1, 1, 0
        cells = np.ascontiguousarray(prob.rec_cells, dtype=np.int32)
        P._cells_keep = cells  # keep alive
        P.nrec_list = len(cells)
        P.rec_cells = cells.ctypes.data_as(C.POINTER(C.c_int))
    P.tao2, P.h2, P.taoh, P.taoh2 = prob.tao2, prob.h2, prob.taoh, prob.taoh2
    P.vmin, P.dv, P.hzx2_1, P.spike = prob.vmin, prob.dv, prob.hzx2_1, prob.spike
    return P


def migrate(prob, seis, precision: str = "f32", use_ref: bool = False, quirk: int = None,
            force_list: bool = False):
    """rel1, rel2 (full padded grid) of one shot. seis: [ntrace, NT] float32."""
    if quirk is None:
        quirk = int(getattr(prob, "quirk", True))
    P = make_params(prob, quirk, force_list)
    dt = np.float32 if precision == "f32" else np.float64
    rel1 = np.zeros(prob.NZ * prob.NX, dt)
    rel2 = np.zeros(prob.NZ * prob.NX, dt)
    args = (C.byref(P), prob.v.ravel(), prob.r1.ravel(), prob.w, prob.coef, prob.index, prob.wav,
            np.ascontiguousarray(seis, np.float32).ravel(), rel1, rel2)
    if use_ref:
        assert precision == "f32"
        rc = ref().ref_migrate(*args)
    else:
        rc = getattr(lib(), "or_migrate_" + precision)(*args)
    if rc != 0:
        raise RuntimeError("oracle migrate failed")
    return rel1.reshape(prob.NZ, prob.NX), rel2.reshape(prob.NZ, prob.NX)


def model(prob, precision: str = "f32", use_ref: bool = False):
    """Receiver recording [nrec, NT] of the forward run of one shot."""
    P = make_params(prob, int(getattr(prob, "quirk", True)))
    dt = np.float32 if precision == "f32" else np.float64
    rec = np.zeros(prob.nrec * prob.NT, dt)
    args = (C.byref(P), prob.v.ravel(), prob.r1.ravel(), prob.w, prob.coef, prob.index, prob.wav, rec)
    rc = ref().ref_model(*args) if use_ref else getattr(lib(), "or_model_" + precision)(*args)
    if rc != 0:
        raise RuntimeError("oracle model failed")
    return rec.reshape(prob.nrec, prob.NT)


def finish_shot(prob, rel1, rel2, whitecoe: float):
    """Per-shot (up, down) images, column-major interior [nx, nz]."""
    nz, nx = prob.nz, prob.nx
    if rel1.dtype == np.float64:
        up = np.zeros(nz * nx, np.float64)
        dn = np.zeros(nz * nx, np.float64)
        lib().or_finish_shot_f64(np.ascontiguousarray(rel1).ravel(), np.ascontiguousarray(rel2).ravel(),
                                 prob.v.ravel(), prob.NZ, prob.NX, prob.N2, prob.vmax, whitecoe, up, dn)
    else:
        up = np.zeros(nz * nx, np.float32)
        dn = np.zeros(nz * nx, np.float32)
        lib().or_finish_shot_f32(np.ascontiguousarray(rel1, np.float32).ravel(),
                                 np.ascontiguousarray(rel2, np.float32).ravel(), prob.v.ravel(),
                                 prob.NZ, prob.NX, prob.N2, prob.vmax, whitecoe, up, dn)
    return up.reshape(nx, nz), dn.reshape(nx, nz)


def stack(ups, downs, nrec: int, inorm: int, kahan: int = 0):
    ups = np.ascontiguousarray(ups)
    downs = np.ascontiguousarray(downs)
    nshot = ups.shape[0]
    ncell = int(np.prod(ups.shape[1:]))
    if ups.dtype == np.float64:
        img = np.zeros(ncell, np.float64)
        ill = np.zeros(ncell, np.float64)
        lib().or_stack_f64(ups.ravel(), downs.ravel(), nshot, ncell, nrec, inorm, img, ill)
    else:
        img = np.zeros(ncell, np.float32)
        ill = np.zeros(ncell, np.float32)
        lib().or_stack_f32(ups.astype(np.float32).ravel(), downs.astype(np.float32).ravel(), nshot,
                           ncell, nrec, inorm, kahan, img, ill)
    return img.reshape(ups.shape[1:]), ill.reshape(ups.shape[1:])


def wavelet_table(n: int, tao: float, f0: float) -> np.ndarray:
    wav = np.zeros(n, np.float32)
    lib().or_wavelet_table(wav, n, tao, f0)
    return wav


def pad_velocity(vin_colmajor, NZ, NX, N2, tao, h, choice=0):
    v = np.zeros(NZ * NX, np.float32)
    r1 = np.zeros(NZ * NX, np.float32)
    lib().or_pad_velocity(np.ascontiguousarray(vin_colmajor, np.float32).ravel(), v, r1, NZ, NX, N2,
                          tao, h, choice)
    return v.reshape(NZ, NX), r1.reshape(NZ, NX)


def bin_velocity(v, dv):
    v = np.ascontiguousarray(v, np.float32).ravel()
    vmin = C.c_float()
    vmax = C.c_float()
    nvel = lib().or_bin_velocity(v, v.size, dv, C.byref(vmin), C.byref(vmax), None, 0)
    need = np.zeros(nvel, np.int32)
    lib().or_bin_velocity(v, v.size, dv, C.byref(vmin), C.byref(vmax),
                          need.ctypes.data_as(C.c_void_p), nvel)
    return float(vmin.value), float(vmax.value), nvel, need


def fun_m_and_c(nthita, nfdmax, nfdmin, nvel, tao, h, df, eps, fmax, vmin, dv, need, hzx):
    need = np.ascontiguousarray(need, np.int32)
    length = np.zeros(nvel, np.int32)
    idx = np.zeros(nvel + 1, np.int32)
    nc = lib().ls_fun_m_and_c(nthita, nfdmax, nfdmin, nvel, tao, h, df, eps, fmax, vmin, dv, need,
                              length, idx, None, 0, hzx)
    if nc < 0:
        raise RuntimeError("coefficient design failed")
    c = np.zeros(nc, np.float32)
    nc2 = lib().ls_fun_m_and_c(nthita, nfdmax, nfdmin, nvel, tao, h, df, eps, fmax, vmin, dv, need,
                               length, idx, c.ctypes.data_as(C.c_void_p), nc, hzx)
    assert nc2 == nc
    return length, idx, c


def ls_coefs(r, bb, M, hzx=1.0):
    c = np.zeros(M + 1, np.float64)
    lib().ls_coefs(c, r, bb, M, hzx)
    return c


def resample(y, dxin, nxout, dxout):
    """Trace(s) y[..., nxin] resampled to nxout samples at dxout
    (Resample.cpp:193-225)."""
    y = np.ascontiguousarray(y, np.float32)
    flat = y.reshape(-1, y.shape[-1])
    out = np.zeros((flat.shape[0], nxout), np.float32)
    for i in range(flat.shape[0]):
        lib().or_resample(flat.shape[1], dxin, np.ascontiguousarray(flat[i]), nxout, dxout, out[i])
    return out.reshape(y.shape[:-1] + (nxout,))


def depth_to_time(v, img, dz, dt):
    """DisToTimeAndTimeToDis1D.cpp (D2T): traces [ntr][nz] -> [ntr][nt]."""
    v = np.ascontiguousarray(v, np.float32)
    img = np.ascontiguousarray(img, np.float32)
    ntr, nz = img.shape
    nt = lib().or_d2t(v, img, ntr, nz, dz, dt, None, 0)
    out = np.zeros((ntr, nt), np.float32)
    assert lib().or_d2t(v, img, ntr, nz, dz, dt, out.ctypes.data_as(C.c_void_p), out.size) == nt
    return out


def time_to_depth(v, img_t, dt, dz):
    """DisToTimeAndTimeToDis1D.cpp (T2D): v [ntr][nzv], traces [ntr][nt] ->
    [ntr][nz]."""
    v = np.ascontiguousarray(v, np.float32)
    img_t = np.ascontiguousarray(img_t, np.float32)
    ntr, nt = img_t.shape
    nz = lib().or_t2d(v, v.shape[1], img_t, ntr, nt, dt, dz, None, 0)
    out = np.zeros((ntr, nz), np.float32)
    assert lib().or_t2d(v, v.shape[1], img_t, ntr, nt, dt, dz, out.ctypes.data_as(C.c_void_p),
                        out.size) == nz
    return out


def phase_rotate(traces, angle):
    """phase_correction_ricker_decon.cpp (phase_correction) on [ntr][nt]."""
    d = np.ascontiguousarray(traces, np.float32)
    out = np.zeros_like(d)
    lib().or_phase(d, out, d.shape[0], d.shape[1], angle)
    return out


def resample_table():
    t = np.zeros(513 * 8, np.float32)
    lib().rs_table(t)
    return t.reshape(513, 8)


def taylor(M):
    c = np.zeros(M + 1, np.float32)
    lib().ls_taylor(2 * M, c)
    return c
