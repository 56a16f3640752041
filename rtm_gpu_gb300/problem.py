"""Host-side description of one RTM model grid and its acquisition geometry.

Mirrors the set-up part of the reference's main() (kernel.cu:542-753): grid
sizes with the absorbing pad, derived time/space constants, the padded
velocity (GPU_velocity_real.cpp:6-118), velocity bins (kernel.cu:704-742),
finite-difference coefficients (adaptive least-squares per velocity bin, or
Taylor), the Ricker wavelet table and the receiver geometry.

The numeric preparation runs in the native library (rtm_prep_* entry points);
adaptive coefficient tables come from the GPU FP64 optimiser
(rtm_gpu_gb300.coeffs) or are passed in.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional, Tuple

import numpy as np

from . import capi


def f32(x) -> float:
    """Round a Python float to float32 (the reference keeps these in float)."""
    return float(np.float32(x))


@dataclasses.dataclass
class Problem:
    nz: int
    nx: int
    N2: int
    M: int            # nfdmax: ring width and longest operator
    NT: int
    h: float
    hz: float
    tao: float
    f0: float
    adaptive: bool
    compen: bool
    v: np.ndarray     # (NZ, NX) float32
    r1: np.ndarray    # (NZ, NX) float32
    w: np.ndarray     # (N2+1,) float32
    vmin: float
    vmax: float
    dv: float
    nvel: int
    length: np.ndarray  # (nvel,) int32 operator length per bin (-1 unused)
    index: np.ndarray   # (nvel+1,) int32
    coef: np.ndarray    # float32 coefficient table
    wav: np.ndarray     # (NT+1,) float32
    rec: Tuple[int, int, int, int, int]  # (z0, x0, dz, dx, n) 0-based padded cells
    src_cell: Tuple[int, int] = (0, 0)   # current source (z, x)
    quirk: bool = True

    # ---- derived quantities, as the reference forms them (kernel.cu:613-626)
    @property
    def NZ(self) -> int:
        return self.nz + 2 * self.N2

    @property
    def NX(self) -> int:
        return self.nx + 2 * self.N2

    @property
    def tao2(self) -> float:
        return f32(math.pow(f32(self.tao), 2))

    @property
    def h2(self) -> float:
        return f32(1 / math.pow(f32(self.h), 2))

    @property
    def taoh(self) -> float:
        return f32(np.float32(self.tao) / np.float32(self.h))

    @property
    def taoh2(self) -> float:
        return f32(np.float32(self.tao2) * np.float32(self.h2) / np.float32(2))

    @property
    def hzx2_1(self) -> float:
        hzx = np.float32(self.hz) / np.float32(self.h)
        return f32(np.float32(1) / (hzx * hzx))

    @property
    def NT2(self) -> int:
        return int(2.0 / float(np.float32(self.f0) * np.float32(self.tao))) + 1

    @property
    def spike(self) -> float:
        return f32(float(self.wav[0]) / 2.0)

    @property
    def nrec(self) -> int:
        return self.rec[4]

    @property
    def rec_line(self) -> Optional[Tuple[int, int, int, int]]:
        """(s_l, s_z, ds, n) when the receivers form the reference's surface
        line, else None."""
        z0, x0, dz, dx, n = self.rec
        if dz == 0 and dx > 0:
            return (x0, z0, dx, n)
        return None

    @property
    def rec_cells(self) -> np.ndarray:
        z0, x0, dz, dx, n = self.rec
        j = np.arange(n)
        return ((z0 + j * dz) * self.NX + (x0 + j * dx)).astype(np.int32)

    def with_source(self, z: int, x: int) -> "Problem":
        return dataclasses.replace(self, src_cell=(int(z), int(x)))

    def src_flat(self, z: int = None, x: int = None) -> int:
        z = self.src_cell[0] if z is None else z
        x = self.src_cell[1] if x is None else x
        return int(z) * self.NX + int(x)

    def c_struct(self, ring_precision: int = capi.RTM_RING_F32) -> capi.RtmProblem:
        """rtm_problem block for rtm_ctx_create (keeps the arrays alive)."""
        p = capi.RtmProblem()
        p.nz, p.nx, p.N2, p.M, p.NT, p.NT2 = self.nz, self.nx, self.N2, self.M, self.NT, self.NT2
        p.adaptive, p.compen, p.quirk = int(self.adaptive), int(self.compen), int(self.quirk)
        p.nbins = self.nvel if self.adaptive else 0
        p.tao2, p.h2, p.taoh, p.taoh2 = self.tao2, self.h2, self.taoh, self.taoh2
        p.vmin, p.dv, p.hzx2_1, p.spike = self.vmin, self.dv, self.hzx2_1, self.spike
        self._keep = [np.ascontiguousarray(a) for a in (self.v, self.r1, self.w, self.coef, self.wav)]
        self._keep.append(np.ascontiguousarray(self.index, np.int32))
        p.v, p.r1, p.w, p.coef, p.wav = (capi.fptr(a) for a in self._keep[:5])
        p.index = capi.iptr(self._keep[5])
        p.rz0, p.rx0, p.rdz, p.rdx, p.nrec = self.rec
        p.ring_precision = ring_precision
        return p


# ---------------------------------------------------------------------------
# native preparation


def prep_velocity(vin_colmajor: np.ndarray, nz: int, nx: int, N2: int, tao: float, h: float,
                  flip: int = 0):
    L = capi.lib()
    vin = np.ascontiguousarray(vin_colmajor, np.float32).ravel()
    NZ, NX = nz + 2 * N2, nx + 2 * N2
    v = np.zeros(NZ * NX, np.float32)
    r1 = np.zeros(NZ * NX, np.float32)
    capi.check(L.rtm_prep_velocity(capi.fptr(vin), nz, nx, N2, tao, h, flip, capi.fptr(v),
                                   capi.fptr(r1)), "prep_velocity")
    return v.reshape(NZ, NX), r1.reshape(NZ, NX)


def prep_bins(v: np.ndarray, dv: float):
    import ctypes as C
    L = capi.lib()
    vv = np.ascontiguousarray(v, np.float32).ravel()
    vmin, vmax, nvel = C.c_float(), C.c_float(), C.c_int()
    capi.check(L.rtm_prep_bins(capi.fptr(vv), vv.size, dv, C.byref(vmin), C.byref(vmax),
                               C.byref(nvel), None, 0), "prep_bins")
    need = np.zeros(nvel.value, np.int32)
    capi.check(L.rtm_prep_bins(capi.fptr(vv), vv.size, dv, C.byref(vmin), C.byref(vmax),
                               C.byref(nvel), capi.iptr(need), need.size), "prep_bins")
    return float(vmin.value), float(vmax.value), int(nvel.value), need


def prep_wavelet(n: int, tao: float, f0: float) -> np.ndarray:
    wav = np.zeros(n, np.float32)
    capi.check(capi.lib().rtm_prep_wavelet(capi.fptr(wav), n, tao, f0), "prep_wavelet")
    return wav


def prep_taylor(M: int) -> np.ndarray:
    c = np.zeros(M + 1, np.float32)
    capi.check(capi.lib().rtm_prep_taylor(2 * M, capi.fptr(c)), "prep_taylor")
    return c


def build_problem(vin_rowmajor: np.ndarray, *, N2: int, M: int, NT: int, h: float, tao: float,
                  f0: float, hz: Optional[float] = None, adaptive: bool = True,
                  compen: bool = True, dv: float = 1.0, rec=(0, 0, 0, 1, 0), flip: int = 0,
                  coef_table=None, quirk: bool = True) -> Problem:
    """Problem from an interior model (nz, nx) in row-major order.

    coef_table: for adaptive=True, a callable (vmin, dv, nvel, need, hzx) ->
    (length, index, coef) -- normally rtm_gpu_gb300.coeffs.optimise_fp64 with
    the optimiser settings bound; ignored for Taylor coefficients."""
    vin = np.asarray(vin_rowmajor, np.float32)
    nz, nx = vin.shape
    hz = h if hz is None else hz
    v, r1 = prep_velocity(vin.T.copy(), nz, nx, N2, tao, h, flip)
    w = np.array([f32((1.0 * i) / (1.0 * N2)) for i in range(N2 + 1)], np.float32)
    vmin, vmax, nvel, need = prep_bins(v, dv)
    if adaptive:
        if coef_table is None:
            raise ValueError("adaptive coefficients need a coefficient table source")
        hzx = float(np.float32(hz) / np.float32(h))
        length, index, coef = coef_table(vmin, dv, nvel, need, hzx)
    else:
        coef = prep_taylor(M)
        length = np.full(nvel, M, np.int32)
        index = np.zeros(nvel + 1, np.int32)
    wav = prep_wavelet(NT + 1, tao, f0)
    return Problem(nz=nz, nx=nx, N2=N2, M=M, NT=NT, h=h, hz=hz, tao=tao, f0=f0,
                   adaptive=adaptive, compen=compen, v=v, r1=r1, w=w, vmin=vmin, vmax=vmax, dv=dv,
                   nvel=nvel, length=np.asarray(length, np.int32),
                   index=np.asarray(index, np.int32), coef=np.asarray(coef, np.float32), wav=wav,
                   rec=tuple(int(a) for a in rec), quirk=quirk)
