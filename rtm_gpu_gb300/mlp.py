"""Learned finite-difference coefficients (rtm_mlp_* in the C ABI).

The network maps (r = v*tao/h, band limit kmax*h, M) to c_1..c_M; it is
trained on the GPU on coefficient sets made by the GPU FP64 optimiser, and a
coefficient table built with it keeps the optimiser as fallback and judge of
the dispersion error.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import capi, coeffs
from .problem import f32

NI, NO = 3, 16
# dispersion measures (include/rtm_gb300.h): |v_FD/v - 1|, and the
# reference's (h/v) |v/v_FD - 1| that its operator-length test compares with eps
DISP_RELATIVE, DISP_REFERENCE = 0, 1


def _bind(L):
    if getattr(L, "_mlp_bound", False):
        return
    vp = C.c_void_p
    L.rtm_mlp_create.argtypes = [C.POINTER(vp), C.c_uint]
    L.rtm_mlp_destroy.argtypes = [vp]
    L.rtm_mlp_nparams.restype = C.c_int
    L.rtm_mlp_get_params.argtypes = [vp, capi.fp]
    L.rtm_mlp_set_params.argtypes = [vp, capi.fp]
    L.rtm_mlp_set_norm.argtypes = [vp, capi.fp]
    L.rtm_mlp_get_norm.argtypes = [vp, capi.fp]
    L.rtm_mlp_grad.argtypes = [vp, capi.fp, capi.fp, C.c_int, capi.fp, capi.fp]
    L.rtm_mlp_train.argtypes = [vp, capi.fp, capi.fp, C.c_int, C.c_int, C.c_int, C.c_float, capi.fp]
    L.rtm_mlp_predict.argtypes = [vp, capi.fp, C.c_int, capi.fp]
    dp = C.POINTER(C.c_double)
    L.rtm_disp_error_fp64.argtypes = [dp, C.c_int, capi.ip, dp, dp, C.c_int, C.c_int, C.c_int,
                                      C.c_double, C.c_int, C.c_double, dp]
    L.rtm_coeffs_mlp.argtypes = [vp, C.POINTER(coeffs.LsSettings), C.c_double, C.c_int, capi.ip,
                                 C.c_int, C.c_double, C.c_int, capi.ip, capi.ip, vp, C.c_int,
                                 C.POINTER(C.c_int), C.POINTER(C.c_int), dp, dp]
    L._mlp_bound = True


def training_set(n, seed=0, r_range=(0.05, 0.6), kh_range=(1.5, 2.9), m_range=(4, 10), hzx=1.0):
    """n samples (x [n,3] = (r, kh, M), c [n,16]) from the GPU FP64 optimiser."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(*r_range, n)
    kh = rng.uniform(*kh_range, n)
    M = rng.integers(m_range[0], m_range[1] + 1, n)
    c = coeffs.ls_coefs(r, kh, M, hzx)  # [n, 17]: c_0..c_16
    x = np.stack([r, kh, M.astype(np.float64)], 1).astype(np.float32)
    return x, np.ascontiguousarray(c[:, 1:17], np.float32)


def fit_norm(x, c=None):
    """Input mean/scale from the samples; outputs scaled by the size of the
    Taylor coefficients, c_l = (2 / l^2) * y_l.  The optimiser's own
    coefficients are a poor scale: where the band is narrow for M they grow
    large along directions that barely change the operator."""
    in_mean = x.mean(0)
    in_scale = x.std(0) + 1e-6
    out_mean = np.zeros(NO, np.float32)
    out_scale = (2.0 / np.arange(1, NO + 1) ** 2).astype(np.float32)
    return [a.astype(np.float32) for a in (in_mean, in_scale, out_mean, out_scale)]


def dispersion_error(c, M, r, bb, nk=64, nth=32, hzx=1.0, metric=DISP_RELATIVE, tao=0.0):
    """Largest dispersion error of coefficient sets c[n, >=M+1] (FP64, GPU):
    |v_FD/v - 1| (DISP_RELATIVE) or the reference's (h/v)|v/v_FD - 1| with
    h/v = tao/r (DISP_REFERENCE)."""
    L = capi.lib()
    _bind(L)
    c = np.ascontiguousarray(c, np.float64)
    M = np.ascontiguousarray(M, np.int32)
    r = np.ascontiguousarray(r, np.float64)
    bb = np.ascontiguousarray(bb, np.float64)
    err = np.zeros(len(r), np.float64)
    dp = C.POINTER(C.c_double)
    capi.check(L.rtm_disp_error_fp64(c.ctypes.data_as(dp), c.shape[1], capi.iptr(M),
                                     r.ctypes.data_as(dp), bb.ctypes.data_as(dp), len(r), nk, nth,
                                     hzx, int(metric), float(tao), err.ctypes.data_as(dp)),
               "disp_error_fp64")
    return err


class Mlp:
    def __init__(self, seed=0):
        L = capi.lib()
        _bind(L)
        h = C.c_void_p()
        capi.check(L.rtm_mlp_create(C.byref(h), seed), "mlp_create")
        self._h = h
        self.nparams = L.rtm_mlp_nparams()

    def close(self):
        if getattr(self, "_h", None):
            capi.lib().rtm_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self):
        p = np.zeros(self.nparams, np.float32)
        capi.check(capi.lib().rtm_mlp_get_params(self._h, capi.fptr(p)), "mlp_get_params")
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        capi.check(capi.lib().rtm_mlp_set_params(self._h, capi.fptr(p)), "mlp_set_params")

    @property
    def norm(self):
        n = np.zeros(2 * NI + 2 * NO, np.float32)
        capi.check(capi.lib().rtm_mlp_get_norm(self._h, capi.fptr(n)), "mlp_get_norm")
        return [n[:3], n[3:6], n[6:22], n[22:38]]

    @norm.setter
    def norm(self, parts):
        n = np.ascontiguousarray(np.concatenate([np.asarray(a, np.float32) for a in parts]))
        capi.check(capi.lib().rtm_mlp_set_norm(self._h, capi.fptr(n)), "mlp_set_norm")

    def grad(self, x, c):
        x = np.ascontiguousarray(x, np.float32)
        c = np.ascontiguousarray(c, np.float32)
        g = np.zeros(self.nparams, np.float32)
        loss = np.zeros(1, np.float32)
        capi.check(capi.lib().rtm_mlp_grad(self._h, capi.fptr(x), capi.fptr(c), len(x), capi.fptr(g),
                                           capi.fptr(loss)), "mlp_grad")
        return float(loss[0]), g

    def train(self, x, c, epochs=20, batch=512, lr=2e-3):
        x = np.ascontiguousarray(x, np.float32)
        c = np.ascontiguousarray(c, np.float32)
        loss = np.zeros(1, np.float32)
        capi.check(capi.lib().rtm_mlp_train(self._h, capi.fptr(x), capi.fptr(c), len(x), epochs,
                                            batch, lr, capi.fptr(loss)), "mlp_train")
        return float(loss[0])

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32)
        c = np.zeros((len(x), NO), np.float32)
        capi.check(capi.lib().rtm_mlp_predict(self._h, capi.fptr(x), len(x), capi.fptr(c)),
                   "mlp_predict")
        return c

    def table(self, *, M, tol, tao, h, fmax, df=1.0, nthita=1000, eps=1e-5, hzx=1.0, vmin, nvel,
              need, metric=DISP_REFERENCE):
        """(length, index, coef, info) of a coefficient table built with the
        network (length M everywhere), judged by the FP64 dispersion error in
        the measure `metric`; bins whose network set misses `tol` keep the
        lower-error set of the network's and the optimiser's."""
        L = capi.lib()
        s = coeffs.LsSettings(int(nthita), int(M), int(M), f32(tao), f32(h), f32(df), f32(eps),
                              f32(fmax), float(hzx))
        need = np.ascontiguousarray(need, np.int32)
        length = np.zeros(nvel, np.int32)
        index = np.zeros(nvel + 1, np.int32)
        nc, nfb = C.c_int(), C.c_int()
        dp = C.POINTER(C.c_double)
        en = np.zeros(nvel, np.float64)
        eu = np.zeros(nvel, np.float64)
        capi.check(L.rtm_coeffs_mlp(self._h, C.byref(s), float(vmin), nvel, capi.iptr(need), M, tol,
                                    int(metric), capi.iptr(length), capi.iptr(index), None, 0,
                                    C.byref(nc), C.byref(nfb), None, None), "coeffs_mlp")
        coef = np.zeros(nc.value, np.float32)
        t0 = time.perf_counter()
        capi.check(L.rtm_coeffs_mlp(self._h, C.byref(s), float(vmin), nvel, capi.iptr(need), M, tol,
                                    int(metric), capi.iptr(length), capi.iptr(index),
                                    C.c_void_p(coef.ctypes.data), nc.value, C.byref(nc),
                                    C.byref(nfb), en.ctypes.data_as(dp), eu.ctypes.data_as(dp)),
                   "coeffs_mlp")
        info = {"seconds": time.perf_counter() - t0, "fallback": nfb.value,
                "bins": int(need.sum()), "err_net": en, "err_used": eu}
        return length, index, coef, info


def train_default(n=200_000, epochs=30, seed=0, batch=512, lr=2e-3, **kw):
    """Network trained on n optimiser samples (default ranges: r in
    [0.05, 0.6], kh in [1.5, 2.9], M in 4..10; others through
    training_set's keywords)."""
    x, c = training_set(n, seed=seed, **kw)
    net = Mlp(seed)
    net.norm = fit_norm(x, c)
    loss = net.train(x, c, epochs=epochs, batch=batch, lr=lr)
    return net, loss
