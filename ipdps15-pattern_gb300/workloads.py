"""Seeded synthetic inputs with the shapes of the benchmark configurations.

No public dataset exists for this path (the reference's moldyn input files are
not part of its tree), so the configurations are generated: uniform-random
boxes, miniMD's FCC lattice, and Maxwell-distributed velocities.
"""
from __future__ import annotations

import math

import numpy as np


def random_box(n: int, density: float, seed: int):
    """n float32 positions uniform in a periodic cube of side (n/density)^(1/3)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    side = np.float32((n / density) ** (1.0 / 3.0))
    pos = (rng.random((n, 3), dtype=np.float32) * side).astype(np.float32)
    pos[pos >= side] = 0.0
    return pos, float(side)


def density_for_neighbours(neighbours: float, cutoff: float) -> float:
    """Density at which a sphere of radius `cutoff` holds `neighbours` others."""
    return neighbours / (4.0 / 3.0 * math.pi * cutoff ** 3)


def fcc_lattice(nx: int, ny: int, nz: int, rho: float):
    """miniMD's FCC lattice (4 nx ny nz atoms at reduced density rho) and the box side.

    Lattice constant (4/rho)^(1/3); sites on the half-lattice grid with
    i + j + k even, z outermost, as miniMD/setup.cpp:61-122 enumerates them.
    """
    alat = (4.0 / rho) ** (1.0 / 3.0)
    i = np.arange(2 * nx)
    j = np.arange(2 * ny)
    k = np.arange(2 * nz)
    kk, jj, ii = np.meshgrid(k, j, i, indexing="ij")
    keep = (ii + jj + kk) % 2 == 0
    pos = np.stack([ii[keep], jj[keep], kk[keep]], axis=1).astype(np.float64) * (0.5 * alat)
    if not (nx == ny == nz):
        raise ValueError("a cubic box is expected")
    return pos, nx * alat


def maxwell_velocities(n: int, temperature: float, seed: int, mass: float = 1.0):
    """Gaussian velocities at `temperature` (k_B = 1), zero total momentum,
    rescaled so that sum(m v^2) / (3n - 3) equals the temperature exactly."""
    rng = np.random.Generator(np.random.PCG64(seed))
    v = rng.normal(0.0, math.sqrt(temperature / mass), (n, 3))
    v -= v.mean(axis=0)
    t = mass * (v * v).sum() / (3 * n - 3)
    v *= math.sqrt(temperature / t)
    return v
