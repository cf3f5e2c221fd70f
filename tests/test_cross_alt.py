"""compute_cross_distances_alt distance types 1-6 (yael/nn.c:164-350): a numpy
restatement of the reference's arithmetic (float SSE lanes for L1 / chi2 when
d % 4 == 0, double sums of float terms otherwise) is pinned against the
reference library compiled here (CPU); the GPU library must equal it bit for
bit (GPU)."""
import ctypes

import numpy as np
import pytest

import yael_gb300 as yg
from _util import reference

P = ctypes.c_void_p
I = ctypes.c_int
f32, f64 = np.float32, np.float64


def ptr(a):
    return a.ctypes.data_as(P)


def operands(seed, na, nb, d):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((na, d)).astype(f32)
    b = rng.standard_normal((nb, d)).astype(f32)
    a[:, ::5] = 0.0           # zeros: chi2 / histogram-intersection edge terms
    b[:, ::7] = 0.0
    b[: min(na, nb) // 2, 1] = a[: min(na, nb) // 2, 1]      # equal coordinates
    b[: min(na, nb) // 3, 2] = -a[: min(na, nb) // 3, 2]     # a + b == 0
    return a, b


def restate(t, a, b):
    """dist[j, i] of the reference for type t."""
    na, d = a.shape
    A = a[:, None, :]
    B = b[None, :, :]
    with np.errstate(divide="ignore", invalid="ignore"):
        if t in (1, 3) and d % 4 == 0:
            lanes = [np.zeros((na, b.shape[0]), f32) for _ in range(4)]
            for k in range(d):
                av, bv = A[:, :, k], B[:, :, k]
                df = (av - bv).astype(f32)
                if t == 1:
                    term = np.abs(df)
                else:
                    term = np.where(av != bv, (df * df).astype(f32) / (av + bv).astype(f32), f32(0))
                lanes[k % 4] = (lanes[k % 4] + term.astype(f32)).astype(f32)
            out = (((lanes[0] + lanes[1]).astype(f32) + lanes[2]).astype(f32) + lanes[3]).astype(f32)
            return out.T
        s = np.zeros((na, b.shape[0]), f64)
        for k in range(d):
            av, bv = A[:, :, k], B[:, :, k]
            df = (av - bv).astype(f32).astype(f64)
            if t == 1:
                s = s + np.abs(df)
            elif t == 2:
                s = s + df * df
            elif t == 3:
                sm = (av + bv).astype(f32)
                s = s + np.where(sm != 0, (df * df) / sm.astype(f64), 0.0)
            elif t == 4:
                den = np.abs((av + bv).astype(f32))
                s = s + np.where(den != 0, (df * df) / den.astype(f64), 0.0)
            elif t == 5:
                s = s + np.where(av < bv, av, bv).astype(f64)
            else:
                s = s + (av * bv).astype(f32).astype(f64)
        return s.astype(f32).T


def run(L, t, a, b, ldd_extra=0):
    na, d = a.shape
    nb = b.shape[0]
    out = np.full((nb, na + ldd_extra), -1.0, f32)
    L.compute_cross_distances_alt_nonpacked(t, d, na, nb, ptr(a), d, ptr(b), d, ptr(out),
                                            na + ldd_extra)
    return out[:, :na]


CASES = [(t, d) for t in range(1, 7) for d in (16, 13)]


def test_restatement_pinned_to_reference():
    R = reference()
    if R is None:
        pytest.skip("reference library not built here (oracle/_ref)")
    res, args = yg.SIGNATURES["compute_cross_distances_alt_nonpacked"]
    R.compute_cross_distances_alt_nonpacked.restype = res
    R.compute_cross_distances_alt_nonpacked.argtypes = args
    for t, d in CASES:
        a, b = operands(t * 100 + d, 37, 29, d)
        np.testing.assert_array_equal(run(R, t, a, b), restate(t, a, b), err_msg=f"type {t} d {d}")


@pytest.mark.gpu
@pytest.mark.parametrize("t,d", CASES + [(1, 64), (3, 128), (2, 96), (6, 5)])
def test_gpu_alt_types_bit_identical(t, d):
    a, b = operands(t * 100 + d + 1, 70, 45, d)
    np.testing.assert_array_equal(run(yg.lib(), t, a, b, ldd_extra=3), restate(t, a, b))


def knn_restate(t, base, queries, k):
    """k smallest (value, index) of the reference's distances (base as the
    first operand); NaN never taken; k = 1 takes only values below 1e30."""
    dist = restate(t, base, queries)  # [query, base row]
    nq, nb = dist.shape
    idx = np.full((nq, k), -1, np.int32)
    dis = np.full((nq, k), np.nan, f32)
    for q in range(nq):
        row = dist[q]
        ok = ~np.isnan(row)
        if k == 1:
            ok &= row < f32(1e30)
        cand = np.nonzero(ok)[0]
        order = cand[np.lexsort((cand, row[cand]))][:k]
        idx[q, :len(order)] = order
        dis[q, :len(order)] = row[order]
        if k == 1 and len(order) == 0:
            dis[q, 0] = f32(1e30)
    return idx, dis


KNN_CASES = [(t, d, k) for t in (1, 3, 4, 5, 6) for d in (16, 13) for k in (1, 5)]


def knn_call(L, t, base, queries, k, nt=1):
    nq, d = queries.shape
    idx = np.zeros((nq, k), np.int32)
    dis = np.zeros((nq, k), f32)
    L.knn_full_thread(t, nq, base.shape[0], d, k, ptr(base), ptr(queries), None, ptr(idx),
                      ptr(dis), nt)
    return idx, dis


def test_knn_restatement_pinned_to_reference():
    R = reference()
    if R is None:
        pytest.skip("reference library not built here (oracle/_ref)")
    for t, d, k in KNN_CASES:
        rng = np.random.default_rng(t * 1000 + d * 10 + k)
        base = rng.standard_normal((300, d)).astype(f32)
        queries = rng.standard_normal((20, d)).astype(f32)
        gi, gd = knn_call(R, t, base, queries, k)
        ei, ed = knn_restate(t, base, queries, k)
        np.testing.assert_array_equal(gi, ei, err_msg=f"type {t} d {d} k {k}")
        np.testing.assert_array_equal(gd, ed, err_msg=f"type {t} d {d} k {k}")


@pytest.mark.gpu
@pytest.mark.parametrize("t,d,k", KNN_CASES)
def test_gpu_knn_alt_types(t, d, k):
    rng = np.random.default_rng(t * 1000 + d * 10 + k + 1)
    base = rng.standard_normal((2000, d)).astype(f32)
    queries = rng.standard_normal((50, d)).astype(f32)
    gi, gd = knn_call(yg.lib(), t, base, queries, k)
    ei, ed = knn_restate(t, base, queries, k)
    np.testing.assert_array_equal(gi, ei)
    np.testing.assert_array_equal(gd, ed)


def test_oracle_port_bit_identical_to_reference():
    """The oracle's C restatement of the _alt dispatch, and of knn_full_thread
    over it (blocked, heap, nt query slices), equal the reference library bit
    for bit for every distance type; they are the timed CPU baselines."""
    from _util import oracle
    R = reference()
    if R is None:
        pytest.skip("reference library not built here (oracle/_ref)")
    res, args = yg.SIGNATURES["compute_cross_distances_alt_nonpacked"]
    R.compute_cross_distances_alt_nonpacked.restype = res
    R.compute_cross_distances_alt_nonpacked.argtypes = args
    o = oracle()
    o.orc_cross_distances_alt.argtypes = [I, I, I, I, P, I, P, I, P, I]
    for t in (1, 2, 3, 4, 5, 6, 12, 16):
        for d in (16, 13):
            a, b = operands(t * 10 + d, 300, 270, d)  # more than one 256-row block
            exp = np.full((270, 300), -1.0, f32)
            R.compute_cross_distances_alt_nonpacked(t, d, 300, 270, ptr(a), d, ptr(b), d,
                                                    ptr(exp), 300)
            got = np.full((270, 300), -1.0, f32)
            o.orc_cross_distances_alt(t, d, 300, 270, ptr(a), d, ptr(b), d, ptr(got), 300)
            np.testing.assert_array_equal(got, exp, err_msg=f"type {t} d {d}")
    for t in (1, 3, 4, 5, 6):
        for k, nt in ((1, 1), (5, 1), (5, 3)):
            rng = np.random.default_rng(t * 100 + k + nt)
            base = rng.standard_normal((600, 16)).astype(f32)
            queries = rng.standard_normal((40, 16)).astype(f32)
            gi, gd = knn_call(R, t, base, queries, k, nt)
            ei = np.zeros((40, k), np.int32)
            ed = np.zeros((40, k), f32)
            o.orc_knn_port(t, 40, 600, 16, k, ptr(base), ptr(queries), None, ptr(ei), ptr(ed), nt)
            np.testing.assert_array_equal(ei, gi, err_msg=f"type {t} k {k} nt {nt}")
            np.testing.assert_array_equal(ed, gd, err_msg=f"type {t} k {k} nt {nt}")
