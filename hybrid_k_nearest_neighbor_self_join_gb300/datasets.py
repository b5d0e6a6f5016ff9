"""Seeded synthetic datasets with the shapes of the benchmark configurations.

The reference measures on the Gaia DR2 25M-point RA/Dec catalogue
(README.md:34-37, 61), which is not available here; `sky_like` stands in for
it with the same size, 2-D shape, coordinate ranges and skew (a Gaussian band
around the equator plus dense clumps).  All generators use numpy's PCG64
(`np.random.default_rng(seed)`), so every run sees identical points.
"""
from __future__ import annotations

import numpy as np


def uniform(n: int = 100_000, d: int = 2, seed: int = 0, dtype=np.float32) -> np.ndarray:
    """i.i.d. uniform points in [0,1)^d (configuration 1: 100k x 2-D, k=8, BETA=0)."""
    rng = np.random.default_rng(seed)
    return rng.random((n, d), dtype=np.float64).astype(dtype)


def _sky_base(rng, m: int) -> np.ndarray:
    x = rng.uniform(0.0, 360.0, m)
    band = rng.random(m) < 0.7
    y = np.where(band, np.clip(rng.normal(0.0, 8.0, m), -90.0, 90.0), rng.uniform(-90.0, 90.0, m))
    return np.stack([x, y], axis=1)


def sky_like(n: int = 25_000_000, seed: int = 1, n_clumps: int = 200, clump_frac: float = 0.001,
             clump_sd: float = 0.2, dtype=np.float32) -> np.ndarray:
    """Sky-like 2-D skew (configuration 2: 25M x 2-D, k=64, BETA=0.025).

    x ~ U[0,360); y: 70% N(0, 8^2) clipped to [-90,90], 30% U[-90,90];
    n_clumps Gaussian clumps of sd clump_sd each holding clump_frac of the
    points, centred by the same x/y law.  Rows are shuffled.
    """
    rng = np.random.default_rng(seed)
    per = int(round(n * clump_frac))
    n_cl = per * n_clumps
    base = _sky_base(rng, n - n_cl)
    centres = _sky_base(rng, n_clumps)
    cl = np.repeat(centres, per, axis=0) + rng.normal(0.0, clump_sd, (n_cl, 2))
    cl[:, 1] = np.clip(cl[:, 1], -90.0, 90.0)
    pts = np.concatenate([base, cl]).astype(dtype)
    return np.ascontiguousarray(pts[rng.permutation(n)])


def gmm(n: int, d: int, n_comp: int, uniform_frac: float, seed: int, sd_lo: float = 0.005,
        sd_hi: float = 0.1, dtype=np.float64) -> np.ndarray:
    """Mixture of n_comp anisotropic Gaussians (axis sd log-uniform in
    [sd_lo, sd_hi], centres uniform in [0,1]^d) plus a uniform background."""
    rng = np.random.default_rng(seed)
    n_u = int(round(n * uniform_frac))
    n_g = n - n_u
    centres = rng.random((n_comp, d))
    sds = np.exp(rng.uniform(np.log(sd_lo), np.log(sd_hi), (n_comp, d)))
    lab = rng.integers(0, n_comp, n_g)
    pts = np.empty((n, d), dtype=dtype)
    pts[:n_g] = (centres[lab] + rng.standard_normal((n_g, d)) * sds[lab]).astype(dtype)
    pts[n_g:] = rng.random((n_u, d)).astype(dtype)
    return np.ascontiguousarray(pts[rng.permutation(n)])


def gmm6d(n: int = 10_000_000, seed: int = 2) -> np.ndarray:
    """Configuration 3: 10M x 6-D float64, 100 Gaussians + 10% uniform, k=16, BETA=0.05."""
    return gmm(n, 6, 100, 0.10, seed, dtype=np.float64)


def heldout4d(n: int = 5_000_000, seed: int = 3) -> np.ndarray:
    """Configuration 4: 5M x 4-D float32, 50-component mixture + 20% uniform, k=128."""
    return gmm(n, 4, 50, 0.20, seed, dtype=np.float32)


def batched_sets(n_sets: int = 512, seed: int = 4, n_lo: int = 2_000, n_hi: int = 500_000):
    """Configuration 5: independent float32 sets, sizes log-uniform in
    [n_lo, n_hi], d in {2,3,4,6,8}, 1-20 Gaussian components plus 5-30%
    uniform, k in {8, 32}; set i uses seed + 1 + i.  Yields (points, k)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(n_lo), np.log(n_hi), n_sets)).astype(np.int64)
    dims = rng.choice([2, 3, 4, 6, 8], n_sets)
    comps = rng.integers(1, 21, n_sets)
    ufrac = rng.uniform(0.05, 0.30, n_sets)
    ks = rng.choice([8, 32], n_sets)
    for i in range(n_sets):
        pts = gmm(int(sizes[i]), int(dims[i]), int(comps[i]), float(ufrac[i]), seed + 1 + i,
                  dtype=np.float32)
        yield pts, int(ks[i])


# name -> (generator, k, BETA, NUMINDEXEDDIM)
CONFIGS = {
    "uniform2d_100k": (lambda: uniform(100_000, 2, 0), 8, 0.0, 2),
    "sky2d_25m": (lambda: sky_like(25_000_000, 1), 64, 0.025, 2),
    "gmm6d_10m": (lambda: gmm6d(10_000_000, 2), 16, 0.05, 6),
    "heldout4d_5m": (lambda: heldout4d(5_000_000, 3), 128, 0.05, 4),
}
