"""Golden fixtures of L1 and chi2 k-means (KMEANS_L1 / KMEANS_CHI2,
yael/kmeans.c:213-330) from the reference library compiled from its own
sources (oracle/_ref, see make_golden.py).  Writes tests/golden/kmeans_l1.npz
and tests/golden/kmeans_chi2.npz; needs the reference tree."""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from _util import ORACLE_DIR, REF_LIB, reference  # noqa: E402
from make_golden import run_kmeans  # noqa: E402

QUIET_RANDOM = 0x10000 | 0x80000 | 4
L1, CHI2 = 0x200000, 0x400000


def main():
    if not os.path.exists(REF_LIB):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "ref"], check=True)
    r = reference()
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    rng = np.random.default_rng(20261204)
    # L1: a Gaussian mixture (d = 16: the reference's SSE form of the L1 distance)
    cent = rng.standard_normal((15, 16)) * 3
    v = (cent[rng.integers(0, 15, 3000)] + rng.standard_normal((3000, 16))).astype(np.float32)
    out = run_kmeans(r, v, 12, 8, QUIET_RANDOM | L1, 9, 1)
    np.savez_compressed(os.path.join(HERE, "kmeans_l1.npz"), v=v, k=12, niter=8, seed=9,
                        flags=QUIET_RANDOM | L1, **out)
    # chi2: non-negative histogram-like rows (d = 12: the double form)
    hist = rng.gamma(0.7, 1.0, (2000, 12)) * rng.integers(0, 3, (2000, 1))
    v = (hist / np.maximum(hist.sum(1, keepdims=True), 1e-6)).astype(np.float32)
    out = run_kmeans(r, v, 10, 6, QUIET_RANDOM | CHI2, 3, 1)
    np.savez_compressed(os.path.join(HERE, "kmeans_chi2.npz"), v=v, k=10, niter=6, seed=3,
                        flags=QUIET_RANDOM | CHI2, **out)
    print("wrote kmeans_l1.npz, kmeans_chi2.npz")


if __name__ == "__main__":
    main()
