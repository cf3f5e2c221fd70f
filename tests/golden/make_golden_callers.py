"""Golden fixtures of the path's callers from the reference library compiled
from its own sources (oracle/_ref, see make_golden.py): k-means LSH
(yael/kmlsh.c: kmlsh_ann_fvec), Gaussian mixtures (yael/gmm.c: gmm_learn,
gmm_compute_p) and VLAD (yael/vlad.c: vlad_compute).  Writes
tests/golden/{kmlsh,gmm,vlad}.npz; needs the reference tree.  Each file
records the BLAS the reference was linked with (the sgemm summation order
decides the last bits of float results)."""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from _util import ORACLE_DIR, REF_LIB, oracle, ptr, reference, srand48  # noqa: E402

P = ctypes.c_void_p
I = ctypes.c_int


class Gmm(ctypes.Structure):
    _fields_ = [("d", I), ("k", I), ("w", ctypes.POINTER(ctypes.c_float)),
                ("mu", ctypes.POINTER(ctypes.c_float)), ("sigma", ctypes.POINTER(ctypes.c_float))]


def main():
    if not os.path.exists(REF_LIB):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "ref"], check=True)
    r = reference()
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    blas = oracle().oracle_blas_name().decode()
    rng = np.random.default_rng(20261205)

    # k-means LSH: clustered float rows, 3 partitions, k = 10, one thread
    cent = rng.standard_normal((30, 16)) * 3
    vb = (cent[rng.integers(0, 30, 1500)] + rng.standard_normal((1500, 16))).astype(np.float32)
    vq = (cent[rng.integers(0, 30, 120)] + rng.standard_normal((120, 16))).astype(np.float32)
    r.kmlsh_ann_fvec.restype = P
    r.kmlsh_ann_fvec.argtypes = [P, I, P, I, I, I, I, I]
    r.nnlist_delete.argtypes = [P]
    srand48(4242)
    lp = r.kmlsh_ann_fvec(ptr(vb), 1500, ptr(vq), 120, 16, 10, 3, 1)
    raw = ctypes.cast(lp, ctypes.POINTER(ctypes.c_long))
    idx = np.ctypeslib.as_array(ctypes.cast(raw[2], ctypes.POINTER(ctypes.c_int)),
                                shape=(1200,)).reshape(120, 10).copy()
    dis = np.ctypeslib.as_array(ctypes.cast(raw[3], ctypes.POINTER(ctypes.c_float)),
                                shape=(1200,)).reshape(120, 10).copy()
    r.nnlist_delete(lp)
    np.savez_compressed(os.path.join(HERE, "kmlsh.npz"), vb=vb, vq=vq, k=10, nhash=3,
                        srand48=4242, idx=idx, dis=dis, blas=blas)

    # Gaussian mixtures: gmm_learn (GMM_FLAGS_W, 6 iterations) and the
    # posteriors of the learned mixture
    cent = rng.standard_normal((5, 8))
    v = (cent[rng.integers(0, 5, 2000)] + 0.9 * rng.standard_normal((2000, 8))).astype(np.float32)
    r.gmm_learn.restype = P
    r.gmm_learn.argtypes = [I, I, I, I, P, I, I, I, I]
    r.gmm_delete.argtypes = [P]
    r.gmm_compute_p.argtypes = [I, P, P, P, I]
    gp = r.gmm_learn(8, 2000, 5, 6, ptr(v), 1, 17, 1, 1)
    g = ctypes.cast(gp, ctypes.POINTER(Gmm)).contents
    w = np.ctypeslib.as_array(g.w, shape=(5,)).copy()
    mu = np.ctypeslib.as_array(g.mu, shape=(40,)).reshape(5, 8).copy()
    sigma = np.ctypeslib.as_array(g.sigma, shape=(40,)).reshape(5, 8).copy()
    p = np.empty((2000, 5), np.float32)
    r.gmm_compute_p(2000, ptr(v), gp, ptr(p), 1)
    r.gmm_delete(gp)
    np.savez_compressed(os.path.join(HERE, "gmm.npz"), v=v, k=5, niter=6, seed=17, flags=1,
                        w=w, mu=mu, sigma=sigma, p=p, blas=blas)

    # VLAD: descriptors against 24 centroids
    C = (rng.standard_normal((24, 16)) * 3).astype(np.float32)
    x = (C[rng.integers(0, 24, 1200)] + 0.5 * rng.standard_normal((1200, 16))).astype(np.float32)
    r.vlad_compute.argtypes = [I, I, P, I, P, P]
    desc = np.zeros((24, 16), np.float32)
    r.vlad_compute(24, 16, ptr(C), 1200, ptr(x), ptr(desc))
    np.savez_compressed(os.path.join(HERE, "vlad.npz"), C=C, v=x, desc=desc, blas=blas)


if __name__ == "__main__":
    main()
