"""VLAD and bag-of-features descriptors (yael/vlad.c): a numpy restatement
(exact nearest centroid by the FP64 oracle, then the reference's float32
additions in point / list order) is pinned against the reference library
compiled here (CPU), and the GPU library must equal it bit for bit (GPU)."""
import ctypes

import numpy as np
import pytest

import yael_gb300 as yg
from _util import knn_exact, reference

P = ctypes.c_void_p
I = ctypes.c_int


def ptr(a):
    return None if a is None else a.ctypes.data_as(P)


def data(seed, n=1500, k=40, d=24):
    """Well-separated clusters: every nearest centroid is unambiguous, so an
    FP32 sgemm-based search (the reference's nn) picks the FP64 one too."""
    rng = np.random.default_rng(seed)
    C = (rng.standard_normal((k, d)) * 4).astype(np.float32)
    lab = rng.integers(0, k, n)
    v = (C[lab] + 0.3 * rng.standard_normal((n, d))).astype(np.float32)
    w = rng.uniform(0.5, 2.0, n).astype(np.float32)
    sub_idx = rng.integers(0, n, 900).astype(np.int32)  # list order, with repeats
    sub_end = np.array([200, 200, 650, 900], np.int32)  # one empty subset
    return C, v, w, sub_idx, sub_end


def vlad_np(C, v, assign, w=None, idx=None, ends=None):
    k, d = C.shape
    if idx is None:
        idx, ends = np.arange(v.shape[0], dtype=np.int32), np.array([v.shape[0]], np.int32)
    out = np.zeros((len(ends), k, d), np.float32)
    b = 0
    for s, e in enumerate(ends):
        for i in idx[b:e]:
            a = assign[i]
            r = (v[i] - C[a]).astype(np.float32)
            if w is not None:
                r = (r * w[i]).astype(np.float32)
            out[s, a] = out[s, a] + r
        b = e
    return out


def bof_np(k, assign, idx=None, ends=None):
    if idx is None:
        return np.bincount(assign.ravel(), minlength=k).astype(np.int32)
    out, b = np.zeros((len(ends), k), np.float32), 0
    for s, e in enumerate(ends):
        out[s] = np.bincount(assign[idx[b:e]], minlength=k)
        b = e
    return out


def run_all(L, C, v, w, sub_idx, sub_end, ma=3):
    k, d = C.shape
    n = v.shape[0]
    vl = np.zeros((k, d), np.float32)
    L.vlad_compute(k, d, ptr(C), n, ptr(v), ptr(vl))
    vw = np.zeros((k, d), np.float32)
    L.vlad_compute_weighted(k, d, ptr(C), n, ptr(v), ptr(w), ptr(vw))
    vs = np.zeros((len(sub_end), k, d), np.float32)
    L.vlad_compute_subsets(k, d, ptr(C), n, ptr(v), len(sub_end), ptr(sub_idx), ptr(sub_end),
                           ptr(vs))
    bf = np.zeros(k, np.int32)
    L.bof_compute(k, d, ptr(C), n, ptr(v), ptr(bf))
    bm = np.zeros(k, np.int32)
    L.bof_compute_ma(k, d, ptr(C), n, ptr(v), ptr(bm), ma, ctypes.c_float(1.0), 1)
    bs = np.zeros((len(sub_end), k), np.float32)
    L.bof_compute_subsets(k, d, ptr(C), n, ptr(v), len(sub_end), ptr(sub_idx), ptr(sub_end),
                          ptr(bs))
    return vl, vw, vs, bf, bm, bs


def expected(C, v, w, sub_idx, sub_end, ma=3):
    k = C.shape[0]
    a1 = knn_exact(C, v, 1)[0][:, 0]
    am = knn_exact(C, v, ma)[0]
    return (vlad_np(C, v, a1)[0], vlad_np(C, v, a1, w)[0], vlad_np(C, v, a1, None, sub_idx, sub_end),
            bof_np(k, a1), bof_np(k, am), bof_np(k, a1, sub_idx, sub_end))


def test_restatement_pinned_to_reference():
    R = reference()
    if R is None:
        pytest.skip("reference library not built here (oracle/_ref)")
    for name, (res, args) in yg.SIGNATURES.items():
        if name.startswith(("vlad_", "bof_")):
            getattr(R, name).restype = res
            getattr(R, name).argtypes = args
    C, v, w, si, se = data(5)
    got = run_all(R, C, v, w, si, se)
    for g, e in zip(got, expected(C, v, w, si, se)):
        np.testing.assert_array_equal(g, e)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [5, 6])
def test_gpu_descriptors_bit_identical(seed):
    C, v, w, si, se = data(seed)
    got = run_all(yg.lib(), C, v, w, si, se)
    for g, e in zip(got, expected(C, v, w, si, se)):
        np.testing.assert_array_equal(g, e)


def test_numpy_front_end_plumbing(monkeypatch):
    """ynumpy.vlad (yael/ynumpy.py:356-369) over the reference library (same C
    ABI) returns what a direct vlad_compute call into it returns."""
    R = reference()
    if R is None:
        pytest.skip("reference library not built here (oracle/_ref)")
    res, args = yg.SIGNATURES["vlad_compute"]
    R.vlad_compute.restype = res
    R.vlad_compute.argtypes = args
    C, v, w, si, se = data(7)
    k, d = C.shape
    exp = np.zeros((k, d), np.float32)
    R.vlad_compute(k, d, ptr(C), v.shape[0], ptr(v), ptr(exp))
    monkeypatch.setattr(yg, "_lib", R)
    np.testing.assert_array_equal(yg.vlad(C, v), exp)


@pytest.mark.parametrize("nt", [1, 3])
def test_oracle_port_bit_identical_to_reference(nt):
    """The oracle's C restatement of vlad_compute (the reference's sgemm-based
    nearest centroid, float sums in vector order) equals the reference library
    bit for bit; it is the timed CPU baseline."""
    from _util import oracle
    R = reference()
    if R is None:
        pytest.skip("reference library not built here (oracle/_ref)")
    res, args = yg.SIGNATURES["vlad_compute"]
    R.vlad_compute.restype = res
    R.vlad_compute.argtypes = args
    o = oracle()
    o.orc_vlad_compute.argtypes = [I, I, P, I, P, P, I]
    C, v, w, si, se = data(9)
    k, d = C.shape
    exp = np.zeros((k, d), np.float32)
    R.vlad_compute(k, d, ptr(C), v.shape[0], ptr(v), ptr(exp))
    got = np.zeros((k, d), np.float32)
    o.orc_vlad_compute(k, d, ptr(C), v.shape[0], ptr(v), ptr(got), nt)
    np.testing.assert_array_equal(got, exp)
