"""Shared helpers of the test suite: small seeded problems and comparisons.

Adaptive coefficient tables of the CPU tests come from the oracle's FP64
optimiser (the tests are the oracle's user); the GPU tests check the
product's own GPU optimiser against the same oracle separately.
"""
from __future__ import annotations

import numpy as np

from oracle import oracle as orc
from rtm_gpu_gb300.problem import build_problem, f32

# optimiser settings small enough for CPU tests (the reference's own file
# uses nthita=1000, eps=1e-5; the algorithm is the same)
LS_SMALL = dict(nthita=24, nfdmin=2, df=1.0, eps=1e-3)


def oracle_table(nfdmax, tao, h, fmax, nthita=24, nfdmin=2, df=1.0, eps=1e-3):
    """coef_table callable for build_problem backed by the CPU oracle."""

    def make(vmin, dv, nvel, need, hzx):
        return orc.fun_m_and_c(nthita, nfdmax, nfdmin, nvel, f32(tao), f32(h), df, eps, fmax,
                               vmin, dv, need, hzx)

    return make


def layered_model(nz, nx, vlo, vhi, seed, nlayer=4, smooth=0.0):
    """Seeded layered model (row-major [nz, nx]) with a dipping interface and
    a Gaussian anomaly; optional Gaussian smoothing (sigma in cells)."""
    rng = np.random.default_rng(seed)
    vel = np.sort(rng.uniform(vlo, vhi, nlayer)).astype(np.float64)
    z = np.arange(nz)[:, None]
    x = np.arange(nx)[None, :]
    bounds = np.sort(rng.uniform(0.15, 0.9, nlayer - 1)) * nz
    dip = rng.uniform(-0.15, 0.15)
    v = np.full((nz, nx), vel[0])
    for i, b in enumerate(bounds):
        v = np.where(z >= b + dip * (x - nx / 2), vel[i + 1], v)
    cz, cx = rng.uniform(0.3, 0.7) * nz, rng.uniform(0.3, 0.7) * nx
    sig = max(2.0, 0.1 * min(nz, nx))
    v += rng.choice([-1, 1]) * 0.1 * (vhi - vlo) * np.exp(-((z - cz) ** 2 + (x - cx) ** 2) / (2 * sig * sig))
    if smooth > 0:
        from scipy.ndimage import gaussian_filter
        v = gaussian_filter(v, smooth, mode="nearest")
    return np.clip(v, vlo, vhi).astype(np.float32)


def small_problem(adaptive=True, compen=True, nz=40, nx=56, N2=8, M=4, NT=160, seed=1,
                  vlo=1500.0, vhi=1800.0, smooth=0.0, rec=None, hz=None, quirk=True, f0=25.0,
                  h=10.0, tao=0.001):
    vin = layered_model(nz, nx, vlo, vhi, seed, smooth=smooth)
    if rec is None:
        rec = (N2 + 1, N2, 0, 2, (nx + 1) // 2)   # surface line every other column
    fmax = 2.0 * f0
    prob = build_problem(vin, N2=N2, M=M, NT=NT, h=h, tao=tao, f0=f0, hz=hz, adaptive=adaptive,
                         compen=compen, rec=rec, quirk=quirk,
                         coef_table=oracle_table(M, tao, h, fmax) if adaptive else None)
    return prob.with_source(N2 + 2, N2 + nx // 2)


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm((a - b).ravel())
    n = np.linalg.norm(b.ravel())
    return float(d / n) if n > 0 else float(d)


def interior(prob, g):
    """Interior [.., nz, nx] part of full padded grids."""
    N2 = prob.N2
    return g[..., N2:prob.NZ - N2, N2:prob.NX - N2]
