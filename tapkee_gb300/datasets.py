"""Seeded synthetic manifolds for the local-neighborhood operator.

The reference ships no dataset for this stage (its examples' data submodule is
not part of the library); these generators produce the Swiss-roll / S-curve /
cluster-curve inputs used by the tests and the benchmark, from numpy's PCG64
with fixed seeds so every run sees the same points.

All generators return points-major arrays (N x D, one point per row), which is
the memory layout of the reference's D x N column-major feature matrix.
"""
from __future__ import annotations

import numpy as np


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def swiss_roll(n: int, seed: int = 0, noise: float = 0.05) -> np.ndarray:
    """Swiss roll in R^3: u1,u2 ~ U(0,1), t = 3pi/2 (1 + 2 u1), h = 10 u2,
    x = (t cos t, h, t sin t) + N(0, noise^2). float64, n x 3."""
    rng = _rng(seed)
    u1 = rng.random(n)
    u2 = rng.random(n)
    t = 1.5 * np.pi * (1.0 + 2.0 * u1)
    h = 10.0 * u2
    X = np.stack([t * np.cos(t), h, t * np.sin(t)], axis=1)
    return X + rng.normal(0.0, noise, size=(n, 3))


def orthonormal_lift(d_in: int, d_out: int, seed: int) -> np.ndarray:
    """Random orthonormal map R^d_in -> R^d_out (QR of a Gaussian), d_out x d_in."""
    rng = _rng(seed)
    Q, _ = np.linalg.qr(rng.normal(size=(d_out, d_in)))
    return Q


def lifted_swiss_roll(n: int = 200_000, d: int = 64, seed: int = 1, noise: float = 0.01,
                      roll_noise: float = 0.05, dtype=np.float32) -> np.ndarray:
    """The Swiss roll lifted to R^d by a seeded orthonormal 3->d map plus
    isotropic N(0, noise^2) noise (the N=200k, D=64 LLE workload)."""
    X3 = swiss_roll(n, seed=seed, noise=roll_noise)
    Q = orthonormal_lift(3, d, seed + 1000)
    rng = _rng(seed + 2000)
    X = X3 @ Q.T + rng.normal(0.0, noise, size=(n, d))
    return X.astype(dtype)


def s_curve(n: int, seed: int = 3) -> np.ndarray:
    """S-curve in R^3: u,v ~ U(0,1), s = 3pi(u - 1/2),
    x = (sin s, 2v, sign(s)(cos s - 1))."""
    rng = _rng(seed)
    u = rng.random(n)
    v = rng.random(n)
    s = 3.0 * np.pi * (u - 0.5)
    return np.stack([np.sin(s), 2.0 * v, np.sign(s) * (np.cos(s) - 1.0)], axis=1)


def lifted_s_curve(n: int = 50_000, d: int = 32, seed: int = 3, noise: float = 0.02,
                   dtype=np.float32) -> np.ndarray:
    """The S-curve lifted to R^d by a seeded orthonormal map plus N(0, noise^2)
    (the N=50k, D=32, k=20 LTSA workload)."""
    X3 = s_curve(n, seed=seed)
    Q = orthonormal_lift(3, d, seed + 1000)
    rng = _rng(seed + 2000)
    X = X3 @ Q.T + rng.normal(0.0, noise, size=(n, d))
    return X.astype(dtype)


def cluster_curve(n: int = 20_000, d: int = 128, n_clusters: int = 10, sigma: float = 0.3,
                  seed: int = 5, dtype=np.float32) -> np.ndarray:
    """n points from n_clusters Gaussian clusters (std sigma) whose centres lie
    on a seeded random smooth 1-D curve in R^d."""
    rng = _rng(seed)
    a = rng.normal(size=(3, d))
    s = np.linspace(0.0, 1.0, n_clusters)
    centres = (np.outer(np.sin(np.pi * s), a[0]) + np.outer(np.cos(np.pi * s), a[1])
               + np.outer(s, a[2])) * 3.0
    lab = rng.integers(0, n_clusters, size=n)
    X = centres[lab] + rng.normal(0.0, sigma, size=(n, d))
    return X.astype(dtype)


def batch_problems(count: int = 256, seed: int = 7, n_range=(500, 20_000),
                   dims=(3, 16, 64, 128), ks=(8, 12, 16, 24, 32)):
    """Specs of independent uneven LLE problems: (N, D, k, seed) with
    N ~ U[n_range], D from dims, k from ks, per-problem seed = seed + i."""
    rng = _rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        D = int(rng.choice(dims))
        k = int(rng.choice(ks))
        out.append((n, D, k, seed + 1 + i))
    return out


def batch_problem_data(n: int, d: int, seed: int, dtype=np.float32) -> np.ndarray:
    """One noisy Swiss roll lifted to R^d (d=3: the plain roll)."""
    if d == 3:
        return swiss_roll(n, seed=seed).astype(dtype)
    return lifted_swiss_roll(n, d, seed=seed, dtype=dtype)
