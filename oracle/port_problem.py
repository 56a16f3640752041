"""Problem set-up through the oracle's restatement of the reference's host code.

TEST INFRASTRUCTURE ONLY.  Used where a run must not touch the product
library: bench.py's reference arm, which times the reference's own CPU path
on a problem prepared the way the reference's main() prepares it
(kernel.cu:542-753): velocity padding (GPU_velocity_real.cpp:6-118), bins
(kernel.cu:704-742), the least-squares coefficient table with adaptive
operator length (funMandC, LSMOrCon_rec_2D.cpp:22-524) or Taylor
coefficients (order(), LSMOrCon_rec_2D.cpp:526-551), and the Ricker table
(kernel.cu:1261-1266).  Every routine is the oracle's bit-exact restatement
(pinned against the reference's own build by tests/test_oracle_pin.py).

The result is an rtm_gpu_gb300.problem.Problem (a plain dataclass; building
one does not load the product library).
"""
from __future__ import annotations

import numpy as np

from . import oracle as orc


def _f32(x) -> float:
    return float(np.float32(x))


def build_problem_port(vin_rowmajor, *, N2, M, NT, h, tao, f0, adaptive=True, compen=True,
                       rec=(0, 0, 0, 1, 0), dv=1.0, fmax=None, df=1.0, nthita=1000, eps=1e-5,
                       nfdmin=2, quirk=True):
    """Problem of an interior model (nz, nx) in row-major order; the
    optimiser's float settings are rounded to float32 as the reference reads
    them from its parameter file."""
    from rtm_gpu_gb300.problem import Problem

    vin = np.asarray(vin_rowmajor, np.float32)
    nz, nx = vin.shape
    NZ, NX = nz + 2 * N2, nx + 2 * N2
    v, r1 = orc.pad_velocity(vin.T.copy(), NZ, NX, N2, tao, h, 0)
    w = np.array([_f32((1.0 * i) / (1.0 * N2)) for i in range(N2 + 1)], np.float32)
    vmin, vmax, nvel, need = orc.bin_velocity(v, dv)
    if adaptive:
        fmax = 2.0 * f0 if fmax is None else fmax
        length, index, coef = orc.fun_m_and_c(nthita, M, nfdmin, nvel, _f32(tao), _f32(h), _f32(df),
                                              _f32(eps), _f32(fmax), vmin, dv, need, 1.0)
    else:
        coef = orc.taylor(M)
        length = np.full(nvel, M, np.int32)
        index = np.zeros(nvel + 1, np.int32)
    wav = orc.wavelet_table(NT + 1, tao, f0)
    return Problem(nz=nz, nx=nx, N2=N2, M=M, NT=NT, h=h, hz=h, tao=tao, f0=f0, adaptive=adaptive,
                   compen=compen, v=v, r1=r1, w=w, vmin=vmin, vmax=vmax, dv=dv, nvel=nvel,
                   length=np.asarray(length, np.int32), index=np.asarray(index, np.int32),
                   coef=np.asarray(coef, np.float32), wav=wav, rec=tuple(int(a) for a in rec),
                   quirk=quirk)


def window_problem(p, xa, nx):
    """The problem p restricted to the aperture window of interior columns
    [xa, xa+nx): the window's interior model padded by edge extension as the
    reference pads a model it reads (GPU_velocity_real.cpp:20-80), the same
    coefficient table and wavelet, receivers shifted into the window."""
    import dataclasses

    N2 = p.N2
    vin = p.v[N2:p.NZ - N2, N2 + xa:N2 + xa + nx]
    v, r1 = orc.pad_velocity(vin.T.copy(), p.nz + 2 * N2, nx + 2 * N2, N2, np.float32(p.tao),
                             np.float32(p.h), 0)
    z0, x0, dz, dx, n = p.rec
    return dataclasses.replace(p, nx=nx, v=v, r1=r1, rec=(z0, x0 - xa, dz, dx, n))
