"""Shared test helpers: loading the oracle (test infrastructure) and the
reference build, and tie-aware comparison of k-NN results."""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle.so")
REF_LIB = os.path.join(ORACLE_DIR, "_ref", "libyael_ref.so")
GOLDEN = os.path.join(ROOT, "tests", "golden")

P = ctypes.c_void_p
I = ctypes.c_int
L = ctypes.c_long
F = ctypes.c_float
D = ctypes.c_double

_oracle = None
_ref = None
_libc = ctypes.CDLL(None)
_libc.srand48.argtypes = [ctypes.c_long]


def srand48(seed):
    _libc.srand48(seed)


def read_bytes(path):
    """The contents of a file (path as str, bytes or PathLike), closed after reading."""
    with open(path, "rb") as f:
        return f.read()


def read_text(path):
    with open(path) as f:
        return f.read()


def write_text(path, text):
    with open(path, "w") as f:
        f.write(text)


def build_oracle():
    if not os.path.exists(ORACLE_LIB) or any(
            os.path.getmtime(os.path.join(ORACLE_DIR, f)) > os.path.getmtime(ORACLE_LIB)
            for f in ("yael_oracle.c", "yael_oracle.h", "blas_shim.c")):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    return ORACLE_LIB


def oracle():
    global _oracle
    if _oracle is None:
        build_oracle()
        o = ctypes.CDLL(ORACLE_LIB, mode=ctypes.RTLD_LOCAL)
        o.orc_knn_exact.argtypes = [I, I, I, I, P, P, P, P, P, I]
        o.orc_knn_port.argtypes = [I, I, I, I, I, P, P, P, P, P, I]
        o.orc_cross_distances_port.argtypes = [I, I, I, P, I, P, I, P, I]
        o.orc_cross_distances_exact.argtypes = [I, I, I, P, P, P]
        o.orc_kmeans.argtypes = [I, I, I, I, P, I, L, I, P, P, P, P, I, P]
        o.orc_kmeans.restype = F
        o.orc_kmeans_step_exact.argtypes = [I, I, I, P, P, P, P, P, P, I]
        o.orc_fixed_shift.argtypes = [L, L, P]
        o.orc_fixed_shift.restype = I
        o.orc_reassign_empty.argtypes = [I, I, P, P, ctypes.c_uint]
        o.orc_reassign_empty.restype = I
        o.orc_hkm_learn.argtypes = [I, I, I, I, P, I, P, P, I]
        o.orc_hkm_learn.restype = I
        o.orc_hkm_quantize.argtypes = [I, I, I, P, I, P, P, I]
        o.orc_gaussrand_r.argtypes = [ctypes.POINTER(ctypes.c_uint)]
        o.orc_gaussrand_r.restype = D
        o.orc_random_init.argtypes = [I, I, ctypes.c_uint, P]
        o.oracle_blas_name.restype = ctypes.c_char_p
        o.orc_assign_check.argtypes = [I, I, I, P, P, P, I, P]
        o.orc_assign_check.restype = L
        o.orc_objective64.argtypes = [I, I, P, P, P, I]
        o.orc_knn_check.argtypes = [I, I, I, I, P, P, P, I, P]
        o.orc_knn_check.restype = L
        o.orc_objective64.restype = D
        _oracle = o
    return _oracle


def reference():
    """The reference library compiled from its own sources, or None."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB):
        r = ctypes.CDLL(REF_LIB, mode=ctypes.RTLD_LOCAL)
        r.knn_full_thread.argtypes = [I, I, I, I, I, P, P, P, P, P, I]
        r.kmeans.argtypes = [I, I, I, I, P, I, L, I, P, P, P, P]
        r.kmeans.restype = F
        r.hkm_learn.argtypes = [I, I, I, I, P, I, I, I, ctypes.POINTER(ctypes.POINTER(I))]
        r.hkm_learn.restype = ctypes.c_void_p
        r.compute_cross_distances.argtypes = [I, I, I, P, P, P]
        _ref = r
    return _ref


def ptr(a):
    return None if a is None else a.ctypes.data


# ---------------------------------------------------------------------------
# oracle wrappers


def knn_exact(b, q, k, nt=8):
    nb, d = b.shape
    nq = q.shape[0]
    idx = np.empty((nq, k), np.int32)
    dis = np.empty((nq, k), np.float32)
    d64 = np.empty((nq, k), np.float64)
    oracle().orc_knn_exact(nq, nb, d, k, ptr(b), ptr(q), ptr(idx), ptr(dis), ptr(d64), nt)
    return idx, dis, d64


def knn_port(b, q, k, nt=8, distance_type=2, w=None):
    nb, d = b.shape
    nq = q.shape[0]
    idx = np.empty((nq, k), np.int32)
    dis = np.empty((nq, k), np.float32)
    oracle().orc_knn_port(distance_type, nq, nb, d, k, ptr(b), ptr(q), ptr(w), ptr(idx), ptr(dis), nt)
    return idx, dis


def assign_mismatches(v, C, assign, nt=8):
    """Points whose assignment is not the oracle's FP64 nearest centroid (ties
    to the lowest index), and the first of them (-1 if none)."""
    n, d = v.shape
    first = ctypes.c_long(-1)
    bad = oracle().orc_assign_check(d, n, C.shape[0], ptr(v), ptr(C), ptr(assign), nt,
                                    ctypes.byref(first))
    return int(bad), int(first.value)


def knn_mismatches(b, q, idx, nt=8):
    """Queries whose k ids differ from the oracle's FP64 (distance, id) order,
    and the first of them (-1 if none)."""
    nb, d = b.shape
    nq, k = idx.shape
    first = ctypes.c_long(-1)
    bad = oracle().orc_knn_check(d, nq, nb, k, ptr(b), ptr(q), ptr(np.ascontiguousarray(idx)),
                                 nt, ctypes.byref(first))
    return int(bad), int(first.value)


def objective64(v, C, assign, nt=8):
    """FP64 sum of the points' distances to their assigned centroids."""
    n, d = v.shape
    return float(oracle().orc_objective64(d, n, ptr(v), ptr(C), ptr(assign), nt))


def exact_dist64(b, q, idx):
    """FP64 distances of the listed pairs."""
    qq = q.astype(np.float64)[:, None, :]
    bb = b.astype(np.float64)[np.maximum(idx, 0)]
    return ((qq - bb) ** 2).sum(-1)


# ---------------------------------------------------------------------------
# tie-aware comparison


def check_knn_ties(idx, dis64_of_idx, ref_idx, ref_d64, atol=0.0):
    """idx must equal the canonical (FP64 distance, id) order ref_idx, except
    where FP64 distances tie (within atol): then ids may permute inside an
    equal-distance group and the k-th position may hold any tied id.  Returns
    the number of exact mismatches (0 for parity)."""
    bad = 0
    for r in range(idx.shape[0]):
        a, ra = idx[r], ref_idx[r]
        if np.array_equal(a, ra):
            continue
        da, dr = dis64_of_idx[r], ref_d64[r]
        if not np.allclose(da, dr, rtol=0, atol=atol):
            bad += 1
            continue
        # same multiset of distances; ids must agree on strictly-inside groups
        kth = dr[-1]
        inside = dr < kth - atol
        if set(a[inside]) != set(ra[inside]):
            bad += 1
    return bad
