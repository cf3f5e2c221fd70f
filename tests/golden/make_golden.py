"""Generate the golden fixtures from the reference itself.

The reference has no known-answer tests, so its own outputs are the golden
vectors: this script runs yael's C library compiled from its own sources
(``make -C oracle ref`` -> oracle/_ref/libyael_ref.so, BLAS from the numpy /
scipy OpenBLAS through oracle/blas_shim.c) on small seeded inputs and stores
inputs and outputs in ``tests/golden/*.npz``.  It needs the reference tree, so
it runs only where that exists; the fixtures are committed.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from _util import (ORACLE_DIR, REF_LIB, oracle, ptr, reference,  # noqa: E402
                   srand48)


def run_knn(r, b, q, k, nt=4, dt=2):
    nq, d = q.shape
    idx = np.empty((nq, k), np.int32)
    dis = np.empty((nq, k), np.float32)
    r.knn_full_thread(dt, nq, b.shape[0], d, k, ptr(b), ptr(q), None, ptr(idx), ptr(dis), nt)
    return idx, dis


def run_kmeans(r, v, k, niter, flags, seed, redo):
    n, d = v.shape
    C = np.zeros((k, d), np.float32)
    dis = np.empty(n, np.float32)
    assign = np.empty(n, np.int32)
    nassign = np.empty(k, np.int32)
    qerr = r.kmeans(d, n, k, niter, ptr(v), flags, seed, redo, ptr(C), ptr(dis), ptr(assign),
                    ptr(nassign))
    return dict(C=C, dis=dis, assign=assign, nassign=nassign, qerr=np.float32(qerr))


def main():
    if not os.path.exists(REF_LIB):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "ref"], check=True)
    r = reference()
    blas = oracle().oracle_blas_name().decode()
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    quiet = 0x10000 | 0x80000 | 4

    rng = np.random.default_rng(20240601)
    # 1. integer data with many exact ties
    b = rng.integers(0, 16, (3000, 24)).astype(np.float32)
    q = rng.integers(0, 16, (60, 24)).astype(np.float32)
    out = dict(b=b, q=q, blas=blas)
    for k in (1, 5, 37):
        i, d = run_knn(r, b, q, k)
        out[f"idx_k{k}"] = i
        out[f"dis_k{k}"] = d
    np.savez_compressed(os.path.join(HERE, "knn_int.npz"), **out)

    # 2. float data
    b = rng.standard_normal((4000, 40)).astype(np.float32)
    q = rng.standard_normal((60, 40)).astype(np.float32)
    i, d = run_knn(r, b, q, 10)
    i1, d1 = run_knn(r, b, q, 1)
    i16, d16 = run_knn(r, b, q, 7, dt=16)
    np.savez_compressed(os.path.join(HERE, "knn_float.npz"), b=b, q=q, idx_k10=i, dis_k10=d,
                        idx_k1=i1, dis_k1=d1, idx_dot_k7=i16, dis_dot_k7=d16, blas=blas)

    # 3. k-means on separated clusters
    centres = rng.standard_normal((20, 16)).astype(np.float32) * 3
    lab = rng.integers(0, 20, 3000)
    v = (centres[lab] + 0.1 * rng.standard_normal((3000, 16))).astype(np.float32)
    res = run_kmeans(r, v, 20, 12, quiet, 1234, 1)
    np.savez_compressed(os.path.join(HERE, "kmeans_sep.npz"), v=v, k=20, niter=12, flags=quiet,
                        seed=1234, redo=1, blas=blas, **res)

    # 4. duplicated points: random init picks duplicates -> empty clusters -> splits
    v = rng.integers(0, 3, (600, 4)).astype(np.float32)
    res = run_kmeans(r, v, 40, 20, quiet, 77, 1)
    np.savez_compressed(os.path.join(HERE, "kmeans_empty.npz"), v=v, k=40, niter=20, flags=quiet,
                        seed=77, redo=1, blas=blas, **res)

    # 5. several runs, best kept
    v = rng.standard_normal((2000, 8)).astype(np.float32)
    res = run_kmeans(r, v, 10, 10, quiet, 5, 3)
    np.savez_compressed(os.path.join(HERE, "kmeans_redo.npz"), v=v, k=10, niter=10, flags=quiet,
                        seed=5, redo=3, blas=blas, **res)

    # 5b. k-means++ initialisation (KMEANS_INIT_BERKELEY), integer data so the
    #     distances feeding the sampling are exact whatever the BLAS
    v = rng.integers(0, 20, (3000, 12)).astype(np.float32)
    fl = 0x10000 | 0x20000 | 4
    res = run_kmeans(r, v, 30, 8, fl, 99, 1)
    np.savez_compressed(os.path.join(HERE, "kmeans_pp.npz"), v=v, k=30, niter=8, flags=fl,
                        seed=99, redo=1, blas=blas, **res)

    # 6. hierarchical k-means, seeds from lrand48 after srand48(42)
    centres = rng.standard_normal((64, 8)).astype(np.float32) * 2
    lab = rng.integers(0, 64, 4000)
    v = (centres[lab] + 0.2 * rng.standard_normal((4000, 8))).astype(np.float32)
    srand48(42)
    assign_p = ctypes.POINTER(ctypes.c_int)()
    h = r.hkm_learn(4000, 8, 2, 4, ptr(v), 8, 4, 0, ctypes.byref(assign_p))

    class Hkm(ctypes.Structure):
        _fields_ = [("nlevel", ctypes.c_int), ("bf", ctypes.c_int), ("k", ctypes.c_int),
                    ("d", ctypes.c_int), ("centroids", ctypes.POINTER(ctypes.POINTER(ctypes.c_float)))]

    hk = Hkm.from_address(h)
    lv0 = np.ctypeslib.as_array(hk.centroids[0], shape=(4 * 8,)).copy().reshape(4, 8)
    lv1 = np.ctypeslib.as_array(hk.centroids[1], shape=(16 * 8,)).copy().reshape(16, 8)
    assign = np.ctypeslib.as_array(assign_p, shape=(4000,)).copy()
    np.savez_compressed(os.path.join(HERE, "hkm.npz"), v=v, nlevel=2, bf=4, niter=8, srand=42,
                        level0=lv0, level1=lv1, assign=assign, blas=blas)

    # 7. cross distances
    a = rng.standard_normal((70, 33)).astype(np.float32)
    bb = rng.standard_normal((50, 33)).astype(np.float32)
    dist = np.empty((50, 70), np.float32)
    r.compute_cross_distances(33, 70, 50, ptr(a), ptr(bb), ptr(dist))
    np.savez_compressed(os.path.join(HERE, "cross.npz"), a=a, b=bb, dist2=dist, blas=blas)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
