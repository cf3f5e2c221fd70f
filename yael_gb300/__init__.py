"""GB300 (sm_103a) implementation of yael's distance-GEMM path.

The product is the C-ABI library ``libyael_gb300.so`` (declared in
``include/yael_gpu.h``): exact k-NN, cross distances, k-means and hierarchical
k-means, and their callers (VLAD / bag-of-features, Gaussian mixtures and
Fisher vectors, k-means LSH) and vector files, with yael's own symbol names
and conventions.  This module loads it with ctypes and mirrors the reference's
numpy front end on top of it (yael/ynumpy.py:46-130, 158-369: ``knn``,
``cross_distances``, ``kmeans``, the ``fvecs`` / ``ivecs`` / ``bvecs``
helpers, ``gmm_learn``, ``gmm_read``, ``fisher``, ``vlad``).

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

PREC_ENV, PREC_FP32, PREC_BF16, PREC_BF16X3, PREC_FP16 = -1, 0, 1, 2, 3


class KnnPair(ctypes.Structure):
    _fields_ = [("nq", c_int), ("nb", c_int), ("q", P), ("b", P), ("assign", P), ("dis", P)]


class KmeansOpts(ctypes.Structure):
    _fields_ = [("precision", c_int), ("device_ptrs", c_int), ("stream", P), ("status", c_int),
                ("iterations", c_long), ("n_fallback", c_long), ("n_second", c_long),
                ("ms_assign", c_float),
                ("ms_update", c_float), ("n_band", c_long), ("prec_used", c_int),
                ("n_probe", c_int), ("probe_rows", P), ("probe_iters", c_int),
                ("probe_assign", P), ("probe_centroids", P), ("probe_qerr", P),
                ("wait_limit_us", c_int)]


class CallStats(ctypes.Structure):
    _fields_ = [("instance_iterations", c_long), ("point_iterations", c_long),
                ("level_iterations", c_long), ("ms_assign", c_float), ("ms_update", c_float),
                ("prec_used", c_int)]


class Hkm(ctypes.Structure):
    _fields_ = [("nlevel", c_int), ("bf", c_int), ("k", c_int), ("d", c_int),
                ("centroids", ctypes.POINTER(ctypes.POINTER(c_float)))]


class KnnOpts(ctypes.Structure):
    _fields_ = [("precision", c_int), ("metric", c_int), ("device_ptrs", c_int),
                ("stream", P), ("n_fallback", c_int), ("n_candidates", c_int),
                ("exact_class", c_int), ("timing", c_int), ("ms_scan", c_float),
                ("ms_sample", c_float), ("ms_rerank", c_float), ("scan_launches", c_int),
                ("n_second", c_int), ("n_band", c_int), ("ms_second", c_float),
                ("wait_limit_us", c_int)]


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
    "yael_gpu_last_stats": (c_int, [P]),
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
    prec = {None: PREC_ENV, "fp32": PREC_FP32, "bf16": PREC_BF16, "bf16x3": PREC_BF16X3,
            "fp16": PREC_FP16}[precision]
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
    prec = {None: PREC_ENV, "fp32": PREC_FP32, "bf16": PREC_BF16, "bf16x3": PREC_BF16X3,
            "fp16": PREC_FP16}[precision]
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
    prec = {None: PREC_ENV, "fp32": PREC_FP32, "bf16": PREC_BF16, "bf16x3": PREC_BF16X3,
            "fp16": PREC_FP16}[precision]
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


class Gmm(ctypes.Structure):
    """gmm_t (yael/gmm.h:19-25)."""
    _fields_ = [("d", c_int), ("k", c_int), ("w", ctypes.POINTER(c_float)),
                ("mu", ctypes.POINTER(c_float)), ("sigma", ctypes.POINTER(c_float))]


GMM_FLAGS_W, GMM_FLAGS_NO_NORM, GMM_FLAGS_1SIGMA = 1, 2, 4
GMM_FLAGS_SIGMA, GMM_FLAGS_MU, GMM_FLAGS_PURE_KMEANS = 8, 16, 32

_libc_handle = None


def _libc():
    global _libc_handle
    if _libc_handle is None:
        c = ctypes.CDLL(None)
        c.fopen.restype = P
        c.fopen.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        c.fdopen.restype = P
        c.fdopen.argtypes = [c_int, ctypes.c_char_p]
        c.fclose.argtypes = [P]
        c.free.argtypes = [P]
        _libc_handle = c
    return _libc_handle


def _fopen(filename, mode):
    fh = _libc().fopen(os.fsencode(filename), mode.encode())
    if not fh:
        raise IOError(f"cannot open {filename}")
    return fh


def _take(p, n, ctype, dtype):
    """copy n elements of a malloc'd C array into numpy, then free it"""
    a = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctype)), shape=(n,)).astype(dtype) \
        if n > 0 else np.zeros(0, dtype)
    _libc().free(p)
    return a


def _rows(a, dtype, name):
    a = np.ascontiguousarray(a, dtype=dtype)
    if a.ndim != 2:
        raise ValueError(f"{name}: expected a 2-D array")
    return a


def fvecs_fsize(filename):
    """(n, d) of a .fvecs file (yael/ynumpy.py:158-163)."""
    d, n = c_int(), c_int()
    lib().fvecs_fsize(os.fsencode(filename), ctypes.byref(d), ctypes.byref(n))
    if n.value < 0 and d.value < 0:
        raise IOError("fvecs_fsize: cannot read " + str(filename))
    return n.value, d.value


def fvecs_read(filename, nmax=-1, c_contiguous=True):
    """The vectors of a .fvecs file as an (n, d) float32 array
    (yael/ynumpy.py:165-186): all of them, or at most nmax."""
    if nmax < 0:
        fv = np.fromfile(filename, dtype=np.float32)
        if fv.size == 0:
            return np.zeros((0, 0))
        dim = int(fv.view(np.int32)[0])
        assert dim > 0
        fv = fv.reshape(-1, 1 + dim)
        if not (fv.view(np.int32)[:, 0] == dim).all():
            raise IOError("non-uniform vector sizes in " + str(filename))
        fv = fv[:, 1:]
        return fv.copy() if c_contiguous else fv
    fh = _fopen(filename, "r")
    d, out = c_int(), P()
    n = lib().fvecs_new_fread_max(fh, ctypes.byref(d), ctypes.byref(out), nmax)
    _libc().fclose(fh)
    if n == -1:
        raise IOError("could not read " + str(filename))
    dd = d.value if n > 0 else 0
    return _take(out, n * dd, c_float, np.float32).reshape(n, dd)


def ivecs_read(filename):
    """The vectors of a .ivecs file as an (n, d) int32 array
    (yael/ynumpy.py:188-196)."""
    d, out = c_int(), P()
    n = lib().ivecs_new_read(os.fsencode(filename), ctypes.byref(d), ctypes.byref(out))
    if n == -1:
        raise IOError("could not read " + str(filename))
    dd = d.value if n > 0 else 0
    return _take(out, n * dd, c_int, np.int32).reshape(n, dd)


def fvecs_write(filename, matrix):
    """yael/ynumpy.py:200-205"""
    m = _rows(matrix, np.float32, "fvecs_write")
    n, d = m.shape
    if lib().fvecs_write(os.fsencode(filename), d, n, _ptr(m)) != n:
        raise IOError("write error " + str(filename))


def fvecs_fwrite(f, matrix):
    """Append the rows of matrix to the open binary file f (yael/ynumpy.py:208-213)."""
    m = _rows(matrix, np.float32, "fvecs_fwrite")
    n, d = m.shape
    f.flush()
    fh = _libc().fdopen(os.dup(f.fileno()), b"ab")
    if not fh:
        raise IOError("fvecs_fwrite: cannot write to the file")
    ret = lib().fvecs_fwrite(fh, d, n, _ptr(m))
    _libc().fclose(fh)
    if ret != n:
        raise IOError("write error")


def bvecs_write(filename, matrix):
    """yael/ynumpy.py:216-221"""
    m = _rows(matrix, np.uint8, "bvecs_write")
    n, d = m.shape
    if lib().bvecs_write(os.fsencode(filename), d, n, _ptr(m)) != n:
        raise IOError("write error " + str(filename))


def ivecs_write(filename, matrix):
    """The rows of an int32 matrix as an .ivecs file (yael/ynumpy.py:225-226
    leaves this unimplemented; yael/vector.c:1524-1535 writes the format)."""
    m = _rows(matrix, np.int32, "ivecs_write")
    n, d = m.shape
    if lib().ivecs_write(os.fsencode(filename), d, n, _ptr(m)) != n:
        raise IOError("write error " + str(filename))


def _gmm_to_numpy(gp):
    """(w, mu, sigma) copies of a gmm_t (yael/ynumpy.py:268-275)."""
    g = ctypes.cast(gp, ctypes.POINTER(Gmm)).contents
    k, d = g.k, g.d
    w = np.ctypeslib.as_array(g.w, shape=(k,)).copy()
    mu = np.ctypeslib.as_array(g.mu, shape=(k * d,)).reshape(k, d).copy()
    sigma = np.ctypeslib.as_array(g.sigma, shape=(k * d,)).reshape(k, d).copy()
    return w, mu, sigma


def _numpy_to_gmm(gmm_npy):
    """A gmm_t over the arrays of (w, mu, sigma) (yael/ynumpy.py:283-300);
    returns it with the float32 arrays it points into (keep them alive)."""
    w, mu, sigma = (np.ascontiguousarray(a, dtype=np.float32) for a in gmm_npy)
    k, d = mu.shape
    assert sigma.shape == mu.shape and w.shape == (k,)
    fp = ctypes.POINTER(c_float)
    g = Gmm(d, k, w.ctypes.data_as(fp), mu.ctypes.data_as(fp), sigma.ctypes.data_as(fp))
    return g, (w, mu, sigma)


def gmm_learn(v, k, nt=1, niter=30, seed=0, redo=1, use_weights=True):
    """A diagonal Gaussian mixture of k components: (w, mu, sigma)
    (yael/ynumpy.py:303-320)."""
    v = _f32(v)
    n, d = v.shape
    flags = GMM_FLAGS_W if use_weights else 0
    gp = lib().gmm_learn(d, n, k, niter, _ptr(v), nt, seed, redo, flags)
    try:
        return _gmm_to_numpy(gp)
    finally:
        lib().gmm_delete(gp)


def gmm_read(filename):
    """(w, mu, sigma) of a file written by gmm_write (yael/ynumpy.py:323-329)."""
    fh = _fopen(filename, "r")
    gp = lib().gmm_read(fh)
    _libc().fclose(fh)
    try:
        return _gmm_to_numpy(gp)
    finally:
        lib().gmm_delete(gp)


def fisher(gmm_npy, v, include="mu"):
    """The Fisher vector of the rows of v under the mixture (w, mu, sigma),
    with the gradients named in include ('mu', 'sigma', 'w')
    (yael/ynumpy.py:332-353)."""
    v = _f32(v)
    n, d = v.shape
    g, keep = _numpy_to_gmm(gmm_npy)
    assert d == g.d
    flags = 0
    if "mu" in include:
        flags |= GMM_FLAGS_MU
    if "sigma" in include:
        flags |= GMM_FLAGS_SIGMA
    if "w" in include:
        flags |= GMM_FLAGS_W
    out = np.zeros(lib().gmm_fisher_sizeof(ctypes.byref(g), flags), dtype=np.float32)
    lib().gmm_fisher(n, _ptr(v), ctypes.byref(g), flags, _ptr(out))
    return out


def vlad(centroids, v):
    """The VLAD descriptor (k, d) of the rows of v (yael/ynumpy.py:356-369)."""
    v = _f32(v)
    n, d = v.shape
    c = _f32(centroids)
    k, d2 = c.shape
    assert d2 == d
    out = np.zeros((k, d), dtype=np.float32)
    lib().vlad_compute(k, d, _ptr(c), n, _ptr(v), _ptr(out))
    return out


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
