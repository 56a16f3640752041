"""Seeded synthetic velocity models and acquisition geometries for the
benchmark configurations (there is no field data on the GPU machine; these stand
in for the reference's missing gathers with the stated shapes and value
ranges).

c1: 201x401, 5 flat layers U(1500,4500) sorted + Gaussian anomaly (+-300 m/s,
    sigma 15 cells); 20 Hz source at (2,200); 401 surface receivers at z=2.
c2: 401x1201, 12 random-dip layers 1500-5500 m/s, two normal faults (5-15
    cell throw), a low-velocity lens; 64 surface shots, full-spread receivers.
c3: c2's model, 128 sources with apertures of 300-1201 columns, 300 well
    receivers at x=600, z=50..349.
c5: 1201x4001, 1500-6000 m/s with smooth gradients and 4500 m/s salt bodies.
Coordinates follow the reference's 1-based interior convention (an index i
is padded cell i + N2 - 1).
"""
from __future__ import annotations

import numpy as np


def _smooth(v: np.ndarray, sigma: float) -> np.ndarray:
    if sigma <= 0:
        return v
    from scipy.ndimage import gaussian_filter

    return gaussian_filter(v.astype(np.float64), sigma, mode="nearest").astype(np.float32)


def model_c1(seed: int = 1235):
    rng = np.random.default_rng(seed)
    nz, nx = 201, 401
    vel = np.sort(rng.uniform(1500, 4500, 5))
    bounds = np.sort(rng.choice(np.arange(20, nz - 10), 4, replace=False))
    z = np.arange(nz)[:, None] * np.ones((1, nx))
    v = np.full((nz, nx), vel[0])
    for i, b in enumerate(bounds):
        v[z >= b] = vel[i + 1]
    cz, cx = rng.uniform(40, nz - 40), rng.uniform(60, nx - 60)
    amp = rng.choice([-300.0, 300.0])
    zz, xx = np.mgrid[0:nz, 0:nx]
    v = v + amp * np.exp(-((zz - cz) ** 2 + (xx - cx) ** 2) / (2 * 15.0 ** 2))
    return v.astype(np.float32)


def model_c2(seed: int = 1236, nz: int = 401, nx: int = 1201):
    rng = np.random.default_rng(seed)
    zz, xx = np.mgrid[0:nz, 0:nx].astype(np.float64)
    vel = np.sort(rng.uniform(1500, 5500, 12))
    depth = np.sort(rng.uniform(0.04, 0.95, 11)) * nz
    dips = rng.uniform(-0.12, 0.12, 11)
    # two normal faults: dipping planes; the hanging wall is shifted down
    faults = []
    for _ in range(2):
        x0 = rng.uniform(0.2, 0.8) * nx
        slope = rng.uniform(0.5, 1.2) * rng.choice([-1, 1])
        throw = rng.uniform(5, 15)
        faults.append((x0, slope, throw))
    shift = np.zeros_like(zz)
    for x0, slope, throw in faults:
        hang = (xx - x0) > slope * zz * 0.3
        shift += np.where(hang, throw, 0.0)
    zeff = zz - shift
    v = np.full((nz, nx), vel[0])
    for i in range(11):
        iface = depth[i] + dips[i] * (xx - nx / 2)
        v = np.where(zeff >= iface, vel[i + 1], v)
    # low-velocity lens
    cz, cx = rng.uniform(0.3, 0.6) * nz, rng.uniform(0.3, 0.7) * nx
    a, b = rng.uniform(30, 60), rng.uniform(8, 20)
    lens = ((xx - cx) / a) ** 2 + ((zz - cz) / b) ** 2 <= 1.0
    v = np.where(lens, np.maximum(1500.0, v - 800.0), v)
    return np.clip(v, 1500, 5500).astype(np.float32)


def model_c5(seed: int = 1239, nz: int = 1201, nx: int = 4001):
    rng = np.random.default_rng(seed)
    zz, xx = np.mgrid[0:nz, 0:nx].astype(np.float32)
    v = 1500.0 + 3500.0 * (zz / nz) ** 0.8 + 300.0 * np.sin(xx / nx * 2 * np.pi * rng.uniform(1, 3))
    for _ in range(3):
        cz, cx = rng.uniform(0.3, 0.8) * nz, rng.uniform(0.1, 0.9) * nx
        a, b = rng.uniform(150, 500), rng.uniform(60, 200)
        body = ((xx - cx) / a) ** 2 + ((zz - cz) / b) ** 2 <= 1.0
        v = np.where(body, 4500.0, v)
    return np.clip(v, 1500, 6000).astype(np.float32)


def smooth_model(v: np.ndarray, sigma: float = 10.0) -> np.ndarray:
    return _smooth(v, sigma)


def surface_shots(nx: int, nshot: int, N2: int, z1: int = 2):
    """Source cells (z, x) of nshot shots spaced evenly along the surface."""
    xs = np.linspace(1, nx, nshot).round().astype(int)
    return [(z1 + N2 - 1, int(x) + N2 - 1) for x in xs]


def full_spread(nx: int, N2: int, z1: int = 2):
    """Receiver line (z0, x0, dz, dx, n) covering every interior column."""
    return (z1 + N2 - 1, N2, 0, 1, nx)
