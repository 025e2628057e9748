"""Synthetic point clouds for the benchmark workloads and parity tests.

Arrays use the reference's memory layout: a Julia `T[d, N]` column-major coordinate
matrix is a C-contiguous numpy array of shape (N, d) (point-major).  Lattice points are
1-based like `CartesianIndices` (test/point_cloud.jl:19), first dimension fastest.
Randomness comes from numpy's PCG64 `default_rng(seed)`; the reference's Julia RNG
streams cannot be reproduced here, so the clouds have the reference's shapes, sizes and
noise distributions but not its exact values.
"""
from __future__ import annotations

import math

import numpy as np


def lattice(n_per_dim, spacing=1.0, origin=1.0, dtype=np.float64) -> np.ndarray:
    """Points origin + spacing * (i_1 - 1, ..., i_d - 1), first index fastest."""
    n_per_dim = tuple(int(n) for n in n_per_dim)
    axes = [origin + spacing * np.arange(n, dtype=np.float64) for n in n_per_dim]
    grids = np.meshgrid(*axes, indexing="ij")
    # Column-major point order: the first dimension varies fastest.
    pts = np.stack([g.reshape(-1, order="F") for g in grids], axis=1)
    return np.ascontiguousarray(pts, dtype=dtype)


def perturbed_lattice(n_per_dim, noise=0.25, spacing=1.0, origin=1.0, seed=1,
                      dtype=np.float64) -> np.ndarray:
    """Lattice perturbed by uniform noise in [-noise, noise] per coordinate (in FP64, then
    rounded to `dtype`)."""
    rng = np.random.default_rng(seed)
    pts = lattice(n_per_dim, spacing, origin, np.float64)
    pts += rng.uniform(-noise, noise, size=pts.shape)
    return np.ascontiguousarray(pts, dtype=dtype)


def reference_test_cloud(n_per_dim, search_radius, seed=1) -> np.ndarray:
    """The structure of test/point_cloud.jl:4-58: lattice + 0.05 normal noise applied
    twice, then sorted by the cells (floor(x / r) + 1) of the perturbed points, sorted
    lexicographically with the first cell coordinate most significant (sortperm of
    SVectors)."""
    rng = np.random.default_rng(seed)
    pts = lattice(n_per_dim, 1.0, 1.0, np.float64)
    pts += 0.05 * rng.standard_normal(pts.shape)
    pts += 0.05 * rng.standard_normal(pts.shape)
    cells = np.floor(pts / search_radius).astype(np.int64) + 1
    order = np.lexsort(tuple(cells[:, k] for k in reversed(range(cells.shape[1]))))
    return np.ascontiguousarray(pts[order])


# ------------------------------------------------------------------ workload configs

def wcsph_cloud(n_side=200, seed=1, dtype=np.float32):
    """3D lattice n_side^3, spacing 1, uniform noise [-0.25, 0.25]; velocities N(0, 0.1^2);
    a displacement N(0, 0.05^2) for the update! step.  Returns (x, v, dx)."""
    rng = np.random.default_rng(seed)
    x = lattice((n_side,) * 3, 1.0, 1.0, np.float64)
    x += rng.uniform(-0.25, 0.25, size=x.shape)
    v = rng.normal(0.0, 0.1, size=x.shape)
    dx = rng.normal(0.0, 0.05, size=x.shape)
    return (np.ascontiguousarray(x, dtype=dtype), np.ascontiguousarray(v, dtype=dtype),
            np.ascontiguousarray(dx, dtype=dtype))


def periodic_nbody_cloud(n_side=4096, seed=1, dtype=np.float32):
    """2D periodic box [0, n_side)^2: points at (i + 0.5) + U[-0.3, 0.3], masses U[0.5, 1.5]."""
    rng = np.random.default_rng(seed)
    x = lattice((n_side, n_side), 1.0, 0.5, np.float64)
    x += rng.uniform(-0.3, 0.3, size=x.shape)
    m = rng.uniform(0.5, 1.5, size=x.shape[0])
    return np.ascontiguousarray(x, dtype=dtype), np.ascontiguousarray(m, dtype=dtype)


def batched_clouds(n_clouds=512, n_min=1000, n_max=200000, r_min=2.0, r_max=3.5, seed=1,
                   dtype=np.float32):
    """Many independent 3D clouds: N log-uniform in [n_min, n_max], each a perturbed cubic
    lattice of side round(N^(1/3)) (so the realised count is side^3), spacing 1, noise
    U[-0.25, 0.25]; radius U[r_min, r_max]; box [-1, side + 1]^3 (the lattice 1..side with a
    margin of 1, as for the 200^3 workload).  Returns a list of
    dicts with x, v, dx, radius, min_corner, max_corner."""
    rng = np.random.default_rng(seed)
    clouds = []
    for _ in range(n_clouds):
        n = math.exp(rng.uniform(math.log(n_min), math.log(n_max)))
        side = max(2, int(round(n ** (1.0 / 3.0))))
        r = float(rng.uniform(r_min, r_max))
        x = lattice((side,) * 3, 1.0, 1.0, np.float64)
        x += rng.uniform(-0.25, 0.25, size=x.shape)
        v = rng.normal(0.0, 0.1, size=x.shape)
        dx = rng.normal(0.0, 0.05, size=x.shape)
        clouds.append({
            "x": np.ascontiguousarray(x, dtype=dtype),
            "v": np.ascontiguousarray(v, dtype=dtype),
            "dx": np.ascontiguousarray(dx, dtype=dtype),
            "radius": r,
            "min_corner": [-1.0, -1.0, -1.0],
            "max_corner": [side + 1.0] * 3,
        })
    return clouds


# Physical constants of the WCSPH workload (Wendland C2 with h = 1.5 so that the
# support 2h equals the search radius 3; Tait EOS c0 = 10, rho0 = 1, gamma = 7;
# Monaghan viscosity alpha = 0.02, beta = 0 as in the reference's SPH benchmark).
WCSPH = dict(mass=1.0, h=1.5, c0=10.0, rho0=1.0, gamma_exp=7.0, alpha=0.02, eps_visc=0.01)
