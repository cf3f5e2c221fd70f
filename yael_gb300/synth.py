"""Seeded synthetic workloads with the shapes and value distributions of the
benchmark configurations (there is no network for real datasets).

All generators are deterministic in (seed, sizes) and return float32 arrays in
yael's layout (one vector per row, C-contiguous).
"""
from __future__ import annotations

import numpy as np


def sift_like(n, d=128, seed=0, zero_frac=0.30, sigma=40.0):
    """SIFT-like integer descriptors: each value is 0 with probability
    ``zero_frac``, else min(floor(|N(0, sigma)|), 255)."""
    rng = np.random.default_rng(seed)
    out = np.empty((n, d), dtype=np.float32)
    step = max(1, (1 << 24) // max(d, 1))
    for s in range(0, n, step):
        e = min(n, s + step)
        g = rng.standard_normal((e - s, d), dtype=np.float32)
        v = np.minimum(np.floor(np.abs(g) * sigma), 255.0)
        v[rng.random((e - s, d), dtype=np.float32) < zero_frac] = 0.0
        out[s:e] = v
    return out


def gaussian_mixture(n, d, ncomp, sigma, seed=0, weights=None, centre_scale=1.0):
    """Points drawn from a mixture of isotropic Gaussians: centres ~ N(0, 1)
    per coordinate, component chosen by ``weights`` (uniform by default),
    within-component standard deviation ``sigma``.  Returns (points, labels,
    centres)."""
    rng = np.random.default_rng(seed)
    centres = (rng.standard_normal((ncomp, d), dtype=np.float32) * centre_scale).astype(np.float32)
    if weights is None:
        lab = rng.integers(0, ncomp, n)
    else:
        p = np.asarray(weights, dtype=np.float64)
        lab = rng.choice(ncomp, size=n, p=p / p.sum())
    out = np.empty((n, d), dtype=np.float32)
    step = max(1, (1 << 24) // max(d, 1))
    for s in range(0, n, step):
        e = min(n, s + step)
        out[s:e] = centres[lab[s:e]] + sigma * rng.standard_normal((e - s, d), dtype=np.float32)
    return out, lab.astype(np.int32), centres


def zipf_weights(k, a=1.1):
    r = np.arange(1, k + 1, dtype=np.float64)
    w = r ** (-a)
    return w / w.sum()


def unit_gaussian(n, d, seed=0):
    """N(0, 1) rows normalised to unit L2 norm."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, d), dtype=np.float32)
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    return x.astype(np.float32)


def uneven_pairs(npairs=512, d=128, seed=0, nq_range=(1, 8192), nb_range=(10_000, 2_000_000)):
    """(nq, nb) sizes of the batched uneven k-NN workload: both log-uniform."""
    rng = np.random.default_rng(seed)
    lq = rng.uniform(np.log(nq_range[0]), np.log(nq_range[1]), npairs)
    lb = rng.uniform(np.log(nb_range[0]), np.log(nb_range[1]), npairs)
    return np.floor(np.exp(lq)).astype(np.int64), np.floor(np.exp(lb)).astype(np.int64)
