"""Finite-difference coefficient tables: the FP64 GPU least-squares optimiser
(rtm_coeffs_optimise_fp64, LSMOrCon_rec_2D.cpp:22-524 on the GPU)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .problem import f32

KMAX = 16  # longest operator the GPU solver handles


class LsSettings(C.Structure):
    _fields_ = [("nthita", C.c_int), ("nfdmax", C.c_int), ("nfdmin", C.c_int),
                ("tao", C.c_double), ("h", C.c_double), ("df", C.c_double), ("eps", C.c_double),
                ("fmax", C.c_double), ("hzx", C.c_double)]


def _bind(L):
    if getattr(L, "_coeffs_bound", False):
        return
    L.rtm_coeffs_optimise_fp64.argtypes = [C.POINTER(LsSettings), C.c_double, C.c_double, C.c_int,
                                           capi.ip, capi.ip, capi.ip, C.c_void_p, C.c_int,
                                           C.POINTER(C.c_int)]
    L.rtm_ls_coefs_fp64.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double), capi.ip, C.c_int,
                                    C.c_double, C.POINTER(C.c_double)]
    L._coeffs_bound = True


def optimise_fp64(*, nthita, nfdmax, nfdmin, tao, h, df, eps, fmax, hzx, vmin, dv, nvel, need):
    """(length[nvel], index[nvel+1], coef[NC]) as funMandC builds them.  Float
    parameters are rounded to float32 first, as the reference reads them."""
    L = capi.lib()
    _bind(L)
    s = LsSettings(int(nthita), int(nfdmax), int(nfdmin), f32(tao), f32(h), f32(df), f32(eps),
                   f32(fmax), float(hzx))
    need = np.ascontiguousarray(need, np.int32)
    length = np.zeros(nvel, np.int32)
    index = np.zeros(nvel + 1, np.int32)
    nc = C.c_int()
    capi.check(L.rtm_coeffs_optimise_fp64(C.byref(s), float(vmin), float(dv), int(nvel),
                                          capi.iptr(need), capi.iptr(length), capi.iptr(index),
                                          None, 0, C.byref(nc)), "coeffs_optimise_fp64")
    coef = np.zeros(nc.value, np.float32)
    capi.check(L.rtm_coeffs_optimise_fp64(C.byref(s), float(vmin), float(dv), int(nvel),
                                          capi.iptr(need), capi.iptr(length), capi.iptr(index),
                                          C.c_void_p(coef.ctypes.data), nc.value, C.byref(nc)),
               "coeffs_optimise_fp64")
    return length, index, coef


def table_source(*, nfdmax, nfdmin, tao, h, fmax, df=1.0, nthita=1000, eps=1e-5):
    """coef_table callable for problem.build_problem backed by the GPU solver."""

    def make(vmin, dv, nvel, need, hzx):
        return optimise_fp64(nthita=nthita, nfdmax=nfdmax, nfdmin=nfdmin, tao=tao, h=h, df=df,
                             eps=eps, fmax=fmax, hzx=hzx, vmin=vmin, dv=dv, nvel=nvel, need=need)

    return make


def ls_coefs(r, bb, M, hzx=1.0):
    """c[n, KMAX+1] of CAL2DFDCOE_LSM for arrays of (r, bb, M) on the GPU."""
    L = capi.lib()
    _bind(L)
    r = np.ascontiguousarray(np.atleast_1d(r), np.float64)
    bb = np.ascontiguousarray(np.broadcast_to(bb, r.shape), np.float64)
    M = np.ascontiguousarray(np.broadcast_to(M, r.shape), np.int32)
    out = np.zeros((r.size, KMAX + 1), np.float64)
    dp = C.POINTER(C.c_double)
    capi.check(L.rtm_ls_coefs_fp64(r.ctypes.data_as(dp), bb.ctypes.data_as(dp), capi.iptr(M),
                                   r.size, float(hzx), out.ctypes.data_as(dp)), "ls_coefs_fp64")
    return out
