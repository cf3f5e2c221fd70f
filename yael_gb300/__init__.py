"""GB300 (sm_103a) implementation of yael's distance-GEMM path.

The product is the C-ABI library ``libyael_gb300.so`` (declared in
``include/yael_gpu.h``): exact k-NN, cross distances, k-means and hierarchical
k-means with yael's own symbol names and conventions.  This module loads it
with ctypes and mirrors the reference's numpy front end (yael/ynumpy.py:46-130:
``knn``, ``cross_distances``, ``kmeans``) on top of it.

There is no CPU fallback: if the library (or a GPU) is missing, calls raise.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libyael_gb300.so")

_lib = None
_lock = threading.Lock()

c_int, c_long, c_float, c_double = ctypes.c_int, ctypes.c_long, ctypes.c_float, ctypes.c_double
P = ctypes.c_void_p

# kmeans flag bits (yael/kmeans.h:11-18)
KMEANS_QUIET = 0x10000
KMEANS_INIT_BERKELEY = 0x20000
KMEANS_NORMALIZE_CENTS = 0x40000
KMEANS_INIT_RANDOM = 0x80000
KMEANS_INIT_USER = 0x100000
KMEANS_L1 = 0x200000
KMEANS_CHI2 = 0x400000

PREC_ENV, PREC_FP32, PREC_BF16, PREC_BF16X3 = -1, 0, 1, 2


class KnnPair(ctypes.Structure):
    _fields_ = [("nq", c_int), ("nb", c_int), ("q", P), ("b", P), ("assign", P), ("dis", P)]


class KmeansOpts(ctypes.Structure):
    _fields_ = [("precision", c_int), ("device_ptrs", c_int), ("stream", P), ("status", c_int),
                ("iterations", c_long), ("n_fallback", c_long), ("n_second", c_long),
                ("ms_assign", c_float),
                ("ms_update", c_float), ("n_band", c_long)]


class Hkm(ctypes.Structure):
    _fields_ = [("nlevel", c_int), ("bf", c_int), ("k", c_int), ("d", c_int),
                ("centroids", ctypes.POINTER(ctypes.POINTER(c_float)))]


class KnnOpts(ctypes.Structure):
    _fields_ = [("precision", c_int), ("metric", c_int), ("device_ptrs", c_int),
                ("stream", P), ("n_fallback", c_int), ("n_candidates", c_int),
                ("exact_class", c_int), ("timing", c_int), ("ms_scan", c_float),
                ("ms_sample", c_float), ("ms_rerank", c_float), ("scan_launches", c_int),
                ("n_second", c_int), ("n_band", c_int), ("ms_second", c_float)]


# name -> (restype, argtypes); every symbol of include/yael_gpu.h
SIGNATURES = {
    "knn_full": (None, [c_int, c_int, c_int, c_int, c_int, P, P, P, P, P]),
    "knn_full_thread": (None, [c_int, c_int, c_int, c_int, c_int, P, P, P, P, P, c_int]),
    "nn": (c_double, [c_int, c_int, c_int, P, P, P]),
    "nn_thread": (c_double, [c_int, c_int, c_int, P, P, P, c_int]),
    "knn": (P, [c_int, c_int, c_int, c_int, P, P, P]),
    "knn_thread": (P, [c_int, c_int, c_int, c_int, P, P, P, c_int]),
    "knn_reorder_shortlist": (None, [c_int, c_int, c_int, c_int, P, P, P, P]),
    "knn_recompute_exact_dists": (None, [c_int, c_int, c_int, c_int, P, P, c_int, P, P, P]),
    "compute_cross_distances": (None, [c_int, c_int, c_int, P, P, P]),
    "compute_cross_distances_nonpacked": (None, [c_int, c_int, c_int, P, c_int, P, c_int, P, c_int]),
    "compute_cross_distances_thread": (None, [c_int, c_int, c_int, P, P, P, c_int]),
    "compute_cross_distances_alt": (None, [c_int, c_int, c_int, c_int, P, P, P]),
    "compute_cross_distances_alt_nonpacked": (None, [c_int, c_int, c_int, c_int, P, c_int, P, c_int, P, c_int]),
    "compute_cross_distances_alt_thread": (None, [c_int, c_int, c_int, c_int, P, P, P, c_int]),
    "compute_distances_1": (None, [c_int, c_int, P, P, P]),
    "compute_distances_1_nonpacked": (None, [c_int, c_int, P, P, c_int, P]),
    "compute_distances_1_thread": (None, [c_int, c_int, P, P, P, c_int]),
    "compute_distances_1_nonpacked_thread": (None, [c_int, c_int, P, P, c_int, P, c_int]),
    "yael_gpu_knn_ex": (c_int, [c_int, c_int, c_int, c_int, P, P, P, P, ctypes.POINTER(KnnOpts)]),
    "yael_gpu_knn_batch": (c_int, [c_int, P, c_int, c_int, P]),
    "yael_gpu_last_error": (ctypes.c_char_p, []),
    "kmeans": (c_float, [c_int, c_int, c_int, c_int, P, c_int, c_long, c_int, P, P, P, P]),
    "clustering_kmeans": (P, [c_int, c_int, P, c_int, c_int, c_double]),
    "clustering_kmeans_assign": (P, [c_int, c_int, P, c_int, c_int, c_double, P]),
    "clustering_kmeans_assign_with_score": (P, [c_int, c_int, P, c_int, c_int, c_double, c_int, P, P]),
    "hkm_learn": (P, [c_int, c_int, c_int, c_int, P, c_int, c_int, c_int, P]),
    "hkm_delete": (None, [P]),
    "hkm_quantize": (None, [P, c_int, P, P]),
    "hkm_write": (None, [ctypes.c_char_p, P]),
    "hkm_read": (P, [ctypes.c_char_p]),
    "vlad_compute": (None, [c_int, c_int, P, c_int, P, P]),
    "vlad_compute_weighted": (None, [c_int, c_int, P, c_int, P, P, P]),
    "vlad_compute_subsets": (None, [c_int, c_int, P, c_int, P, c_int, P, P, P]),
    "bof_compute": (None, [c_int, c_int, P, c_int, P, P]),
    "bof_compute_ma": (None, [c_int, c_int, P, c_int, P, P, c_int, c_float, c_int]),
    "bof_compute_subsets": (None, [c_int, c_int, P, c_int, P, c_int, P, P, P]),
    "gmm_learn": (P, [c_int, c_int, c_int, c_int, P, c_int, c_int, c_int, c_int]),
    "gmm_print": (None, [P]),
    "gmm_delete": (None, [P]),
    "gmm_compute_p": (None, [c_int, P, P, P, c_int]),
    "gmm_compute_p_thread": (None, [c_int, P, P, P, c_int, c_int]),
    "gmm_fisher": (None, [c_int, P, P, c_int, P]),
    "gmm_fisher_from_posteriors": (None, [c_int, P, P, c_int, P, P]),
    "gmm_fisher_sizeof": (ctypes.c_size_t, [P, c_int]),
    "gmm_fisher_spatial": (None, [c_int, c_int, c_int, P, P, P, P]),
    "gmm_write": (None, [P, P]),
    "gmm_read": (P, [P]),
    "nnlist_new": (P, [c_int, c_int]),
    "nnlist_new_noalloc": (P, [c_int, c_int]),
    "nnlist_delete": (None, [P]),
    "nnlist_addn": (None, [P, c_int, c_int, P, P]),
    "kmlsh_new": (P, [c_int, c_int, c_int]),
    "kmlsh_delete": (None, [P]),
    "kmlsh_learn_xvec": (None, [P, c_int, c_int, P, c_int, c_int]),
    "kmlsh_new_learn_bvec": (P, [c_int, c_int, c_int, c_int, c_int, P, c_int]),
    "kmlsh_new_learn_fvec": (P, [c_int, c_int, c_int, c_int, c_int, P, c_int]),
    "kmlsh_match_xvec": (P, [P, P, P, c_int, P, P, c_int, c_int, c_int, c_int]),
    "kmlsh_match_bvec": (P, [P, P, P, c_int, P, P, c_int, c_int, c_int]),
    "kmlsh_match_fvec": (P, [P, P, P, c_int, P, P, c_int, c_int, c_int]),
    "kmlsh_ann_xvec": (P, [P, c_int, P, c_int, c_int, c_int, c_int, c_int, c_int]),
    "kmlsh_ann_bvec": (P, [P, c_int, P, c_int, c_int, c_int, c_int, c_int]),
    "kmlsh_ann_fvec": (P, [P, c_int, P, c_int, c_int, c_int, c_int, c_int]),
    "kmlsh_idx_new": (P, [P, c_int]),
    "kmlsh_idx_delete": (None, [P]),
    "kmlsh_idx_new_compile_xvec": (P, [P, P, c_int, c_int, c_int]),
    "kmlsh_idx_new_compile_bvec": (P, [P, P, c_int, c_int]),
    "kmlsh_idx_new_compile_fvec": (P, [P, P, c_int, c_int]),
    "kmlsh_idx_get_nvec": (c_int, [P, c_int, c_int]),
    "kmlsh_idx_get_maxincell": (c_int, [P, c_int]),
    "kmlsh_idx_get_vecids": (P, [P, c_int, c_int]),
    "kmeans_cohash_xvec": (None, [P, c_int, P, c_int, P, P, c_int, c_int]),
    "kmeans_cohash_bvec": (None, [P, c_int, P, c_int, P, P, c_int]),
    "kmeans_cohash_fvec": (None, [P, c_int, P, c_int, P, P, c_int]),
    "kmlsh_write": (None, [ctypes.c_char_p, P]),
    "kmlsh_read": (None, [ctypes.c_char_p, P]),
    "kmlsh_idx_write": (None, [ctypes.c_char_p, P]),
    "kmlsh_idx_read": (None, [ctypes.c_char_p, P]),
    "fvec_fwrite": (c_int, [P, P, c_int]),
    "ivec_fwrite": (c_int, [P, P, c_int]),
    "bvec_fwrite": (c_int, [P, P, c_int]),
    "fvecs_fwrite": (c_int, [P, c_int, c_int, P]),
    "ivecs_fwrite": (c_int, [P, c_int, c_int, P]),
    "bvecs_fwrite": (c_int, [P, c_int, c_int, P]),
    "fvecs_write": (c_int, [ctypes.c_char_p, c_int, c_int, P]),
    "ivecs_write": (c_int, [ctypes.c_char_p, c_int, c_int, P]),
    "bvecs_write": (c_int, [ctypes.c_char_p, c_int, c_int, P]),
    "fvecs_fsize": (ctypes.c_long, [ctypes.c_char_p, P, P]),
    "ivecs_fsize": (ctypes.c_long, [ctypes.c_char_p, P, P]),
    "bvecs_fsize": (ctypes.c_long, [ctypes.c_char_p, P, P]),
    "fvecs_new_read": (c_int, [ctypes.c_char_p, P, P]),
    "fvecs_new_fread_max": (c_int, [P, P, P, ctypes.c_long]),
    "ivecs_new_read": (c_int, [ctypes.c_char_p, P, P]),
    "ivecs_new_fread_max": (c_int, [P, P, P, ctypes.c_long]),
    "bvecs_new_read": (c_int, [ctypes.c_char_p, P, P]),
    "b2fvecs_new_read": (c_int, [ctypes.c_char_p, P, P]),
    "fvecs_read": (c_int, [ctypes.c_char_p, c_int, c_int, P]),
    "b2fvecs_read": (c_int, [ctypes.c_char_p, c_int, c_int, P]),
    "fvec_fread": (c_int, [P, P, c_int]),
    "ivec_fread": (c_int, [P, P, c_int]),
    "bvec_fread": (c_int, [P, P, c_int]),
    "fvecs_fread": (ctypes.c_long, [P, P, ctypes.c_long, c_int]),
    "ivecs_fread": (ctypes.c_long, [P, P, ctypes.c_long, c_int]),
    "bvecs_fread": (ctypes.c_long, [P, P, ctypes.c_long, c_int]),
    "fvec_fwrite_raw": (c_int, [P, P, ctypes.c_long]),
    "ivec_fwrite_raw": (c_int, [P, P, ctypes.c_long]),
    "bvec_fwrite_raw": (c_int, [P, P, ctypes.c_long]),
    "fvec_write_raw": (c_int, [ctypes.c_char_p, P, ctypes.c_long]),
    "ivec_write_raw": (c_int, [ctypes.c_char_p, P, ctypes.c_long]),
    "bvec_write_raw": (c_int, [ctypes.c_char_p, P, ctypes.c_long]),
    "fvec_fread_raw": (c_int, [P, P, ctypes.c_long]),
    "ivec_fread_raw": (c_int, [P, P, ctypes.c_long]),
    "bvec_fread_raw": (c_int, [P, P, ctypes.c_long]),
    "fvec_new_fread_raw": (P, [P, ctypes.c_long]),
    "ivec_new_fread_raw": (P, [P, ctypes.c_long]),
    "bvec_new_fread_raw": (P, [P, ctypes.c_long]),
    "fvec_new_read_raw": (P, [ctypes.c_char_p, ctypes.c_long]),
    "ivec_new_read_raw": (P, [ctypes.c_char_p, ctypes.c_long]),
    "bvec_new_read_raw": (P, [ctypes.c_char_p, ctypes.c_long]),
    "ivecs_write_txt": (c_int, [ctypes.c_char_p, c_int, c_int, P]),
    "fvecs_write_txt": (c_int, [ctypes.c_char_p, c_int, c_int, P]),
    "fvecs_read_txt": (c_int, [ctypes.c_char_p, c_int, c_int, P]),
    "hkm_get_centroids": (P, [P, c_int, c_int]),
    "yael_gpu_kmeans_ex": (c_float, [c_int, c_int, c_int, c_int, P, c_int, c_long, c_int, P, P, P, P, ctypes.c_void_p]),
    "yael_gpu_hkm_learn_ex": (c_int, [c_int, c_int, c_int, c_int, P, c_int, c_int, P, P, P, P]),
    "yael_gpu_knn_noalloc": (c_int, [c_int, c_int, c_int, c_int, P, P, P, P, P]),
    "yael_gpu_version": (c_int, []),
    "yael_gpu_launch_count": (c_long, []),
}


def lib() -> ctypes.CDLL:
    """Load libyael_gb300.so (built by ``yael_gb300.build.build()``)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with "
                    "`python -c 'import __graft_entry__ as g; g.build()'`")
            L = ctypes.CDLL(LIB_PATH, mode=ctypes.RTLD_LOCAL)
            for name, (res, args) in SIGNATURES.items():
                if hasattr(L, name):
                    f = getattr(L, name)
                    f.restype = res
                    f.argtypes = args
            _lib = L
    return _lib


def last_error() -> str:
    m = lib().yael_gpu_last_error()
    return m.decode() if m else ""


def _f32(x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    return x


def _ptr(a):
    return a.ctypes.data if a is not None else None


# ---------------------------------------------------------------------------
# numpy front end mirroring yael/ynumpy.py


def knn(queries, base, nnn=1, distance_type=2, nt=1, precision=None, stats=False):
    """k nearest neighbours of each query row among the base rows.

    Same contract as ynumpy.knn (yael/ynumpy.py:46-67): returns (idx, dis) of
    shape (nq, nnn), int32 / float32, ordered by increasing distance with ties
    by increasing base index.  ``precision`` ("fp32" | "bf16" | None = the
    YAEL_GPU_PRECISION environment variable) picks the distance pass.
    """
    base = _f32(base)
    queries = _f32(queries)
    nb, d = base.shape
    nq, d2 = queries.shape
    assert d == d2, "base and queries must have the same dimension"
    idx = np.empty((nq, nnn), dtype=np.int32)
    dis = np.empty((nq, nnn), dtype=np.float32)
    prec = {None: PREC_ENV, "fp32": PREC_FP32, "bf16": PREC_BF16, "bf16x3": PREC_BF16X3}[precision]
    opts = KnnOpts(prec, distance_type, 0, None, 0, 0, 0, 0, 0, 0, 0, 0, 0)
    rc = lib().yael_gpu_knn_ex(nq, nb, d, nnn, _ptr(base), _ptr(queries), _ptr(idx), _ptr(dis),
                               ctypes.byref(opts))
    if rc != 0:
        raise RuntimeError(f"yael_gpu_knn_ex failed ({rc}): {last_error()}")
    if stats:
        return idx, dis, {"n_fallback": opts.n_fallback, "n_candidates": opts.n_candidates,
                          "exact_class": opts.exact_class, "n_second": opts.n_second,
                          "n_band": opts.n_band, "ms_second": opts.ms_second}
    return idx, dis


def knn_batch(pairs, nnn=1, distance_type=2, precision=None, stats=False):
    """Exact k-NN for many independent (queries, base) pairs in one call
    (yael_gpu_knn_batch); pairs = [(queries, base), ...] float32 arrays with the
    same d.  Returns [(idx, dis), ...] as knn() would for each pair."""
    arrays = []
    descs = (KnnPair * len(pairs))()
    d = None
    for i, (q, b) in enumerate(pairs):
        q = np.ascontiguousarray(q, dtype=np.float32)
        b = np.ascontiguousarray(b, dtype=np.float32)
        if d is None:
            d = q.shape[1]
        if q.shape[1] != d or b.shape[1] != d:
            raise ValueError("knn_batch: every pair must have the same d")
        idx = np.empty((q.shape[0], nnn), dtype=np.int32)
        dis = np.empty((q.shape[0], nnn), dtype=np.float32)
        arrays.append((q, b, idx, dis))
        descs[i] = KnnPair(q.shape[0], b.shape[0], _ptr(q), _ptr(b), _ptr(idx), _ptr(dis))
    prec = {None: PREC_ENV, "fp32": PREC_FP32, "bf16": PREC_BF16, "bf16x3": PREC_BF16X3}[precision]
    opts = KnnOpts(prec, distance_type, 0, None, 0, 0, 0, 0, 0, 0, 0, 0, 0)
    rc = lib().yael_gpu_knn_batch(len(pairs), ctypes.cast(descs, P), d or 1, nnn,
                                  ctypes.byref(opts))
    if rc != 0:
        raise RuntimeError(f"yael_gpu_knn_batch failed ({rc}): {last_error()}")
    out = [(a[2], a[3]) for a in arrays]
    if stats:
        return out, {"n_fallback": opts.n_fallback, "n_band": opts.n_band,
                     "n_second": opts.n_second, "exact_class": opts.exact_class}
    return out


def cross_distances(a, b, distance_type=12):
    """dis[j, i] = distance(a_i, b_j) (yael/ynumpy.py:69-84)."""
    a = _f32(a)
    b = _f32(b)
    na, d = a.shape
    nb, d2 = b.shape
    assert d == d2
    dis = np.empty((nb, na), dtype=np.float32)
    lib().compute_cross_distances_alt_nonpacked(distance_type, d, na, nb, _ptr(a), d, _ptr(b), d,
                                                _ptr(dis), na)
    return dis


def kmeans(v, k, distance_type=2, nt=1, niter=30, seed=0, redo=1, verbose=True,
           normalize=False, init="random", output="centroids", precision=None,
           stats=False):
    """k-means with the contract of ynumpy.kmeans (yael/ynumpy.py:87-130)."""
    v = _f32(v)
    n, d = v.shape
    centroids = np.zeros((k, d), dtype=np.float32)
    dis = np.empty(n, dtype=np.float32)
    assign = np.empty(n, dtype=np.int32)
    nassign = np.empty(k, dtype=np.int32)
    flags = nt
    if not verbose:
        flags |= KMEANS_QUIET
    if distance_type == 1:
        flags |= KMEANS_L1
    elif distance_type == 3:
        flags |= KMEANS_CHI2
    if init == "random":
        flags |= KMEANS_INIT_RANDOM
    elif init == "kmeans++":
        flags |= KMEANS_INIT_BERKELEY
    if normalize:
        flags |= KMEANS_NORMALIZE_CENTS
    prec = {None: PREC_ENV, "fp32": PREC_FP32, "bf16": PREC_BF16, "bf16x3": PREC_BF16X3}[precision]
    opts = KmeansOpts(prec, 0, None, 0, 0, 0, 0, 0, 0)
    qerr = lib().yael_gpu_kmeans_ex(d, n, k, niter, _ptr(v), flags, seed, redo, _ptr(centroids),
                                    _ptr(dis), _ptr(assign), _ptr(nassign), ctypes.byref(opts))
    if opts.status != 0:
        raise RuntimeError(f"kmeans failed: {last_error()}")
    if qerr < 0:
        raise RuntimeError("kmeans: clustering failed. Is dataset diverse enough?")
    res = centroids if output == "centroids" else (centroids, qerr, dis, assign, nassign)
    if stats:
        return res, {"iterations": opts.iterations, "n_fallback": opts.n_fallback,
                     "n_second": opts.n_second, "n_band": opts.n_band,
                     "ms_assign": opts.ms_assign, "ms_update": opts.ms_update}
    return res


def hkm(v, nlevel, bf, niter=15, small_nodes=False):
    """Hierarchical k-means: (list of per-level centroid arrays, leaf assignment)."""
    v = _f32(v)
    n, d = v.shape
    sizes = [bf ** (l + 1) for l in range(nlevel)]
    cent = np.empty(sum(sizes) * d, dtype=np.float32)
    assign = np.empty(n, dtype=np.int32)
    rc = lib().yael_gpu_hkm_learn_ex(n, d, nlevel, bf, _ptr(v), niter, int(small_nodes),
                                     _ptr(cent), _ptr(assign), None, None)
    if rc != 0:
        raise RuntimeError(f"hkm failed: {last_error()}")
    out, o = [], 0
    for s in sizes:
        out.append(cent[o:o + s * d].reshape(s, d))
        o += s * d
    return out, assign
