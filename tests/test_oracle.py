"""The oracle (C restatement) pinned against the reference's own outputs
(tests/golden, generated by running the compiled reference) and against a
numpy FP64 brute force.  CPU only."""
import ctypes
import os

import numpy as np
import pytest

from _util import (GOLDEN, check_knn_ties, exact_dist64, knn_exact, knn_port, oracle, ptr,
                   reference, srand48)
from yael_gb300 import synth


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def same_blas(g):
    return str(g["blas"]) == oracle().oracle_blas_name().decode()


@pytest.mark.parametrize("k", [1, 5, 37])
def test_port_knn_matches_reference_int(k):
    g = load("knn_int.npz")
    idx, dis = knn_port(g["b"], g["q"], k, nt=4)
    # integer data: every distance is exact, so the port is bit-exact whatever the BLAS
    np.testing.assert_array_equal(dis, g[f"dis_k{k}"])
    np.testing.assert_array_equal(idx, g[f"idx_k{k}"])


def test_port_knn_matches_reference_float():
    g = load("knn_float.npz")
    idx, dis = knn_port(g["b"], g["q"], 10, nt=4)
    if same_blas(g):
        np.testing.assert_array_equal(idx, g["idx_k10"])
        np.testing.assert_array_equal(dis, g["dis_k10"])
    else:
        assert (idx == g["idx_k10"]).mean() > 0.99
    idx, dis = knn_port(g["b"], g["q"], 7, nt=4, distance_type=16)
    if same_blas(g):
        np.testing.assert_array_equal(idx, g["idx_dot_k7"])


def test_exact_knn_vs_numpy():
    rng = np.random.default_rng(3)
    b = rng.standard_normal((700, 19)).astype(np.float32)
    q = rng.standard_normal((40, 19)).astype(np.float32)
    idx, dis, d64 = knn_exact(b, q, 13)
    full = ((q.astype(np.float64)[:, None] - b.astype(np.float64)[None]) ** 2).sum(-1)
    order = np.lexsort((np.broadcast_to(np.arange(700), full.shape), full), axis=1)[:, :13]
    np.testing.assert_array_equal(idx, order)
    np.testing.assert_allclose(d64, np.take_along_axis(full, order, 1), rtol=1e-12)


def test_reference_equals_exact_modulo_ties():
    """The reference's k>1 order among equal distances is heap-history
    dependent; modulo those ties it is the canonical (distance, id) order."""
    g = load("knn_int.npz")
    for k in (1, 5, 37):
        ridx = g[f"idx_k{k}"]
        idx, dis, d64 = knn_exact(g["b"], g["q"], k)
        np.testing.assert_array_equal(dis, g[f"dis_k{k}"])
        assert check_knn_ties(ridx, exact_dist64(g["b"], g["q"], ridx), idx, d64) == 0
        if k == 1:  # the k=1 path is strict '<' over increasing ids: lowest id wins
            np.testing.assert_array_equal(ridx, idx)


I = ctypes.c_int
P = ctypes.c_void_p


def run_kmeans(v, k, niter, flags, seed, redo, mode):
    n, d = v.shape
    C = np.zeros((k, d), np.float32)
    dis = np.empty(n, np.float32)
    assign = np.empty(n, np.int32)
    nassign = np.empty(k, np.int32)
    q = oracle().orc_kmeans(d, n, k, niter, ptr(v), flags, seed, redo, ptr(C), ptr(dis),
                            ptr(assign), ptr(nassign), mode, None)
    return dict(C=C, dis=dis, assign=assign, nassign=nassign, qerr=np.float32(q))


@pytest.mark.parametrize("name", ["kmeans_sep.npz", "kmeans_empty.npz", "kmeans_redo.npz",
                                  "kmeans_pp.npz"])
def test_port_kmeans_matches_reference(name):
    g = load(name)
    r = run_kmeans(g["v"], int(g["k"]), int(g["niter"]), int(g["flags"]), int(g["seed"]),
                   int(g["redo"]), 0)
    if same_blas(g):
        for key in ("C", "dis", "assign", "nassign"):
            np.testing.assert_array_equal(r[key], g[key], err_msg=key)
        assert r["qerr"] == g["qerr"]
    else:
        np.testing.assert_array_equal(r["assign"], g["assign"])
        np.testing.assert_allclose(r["C"], g["C"], rtol=1e-5, atol=1e-5)


def test_exact_kmeans_close_to_reference():
    """ORC_EXACT (FP64 assignment, exact fixed-point sums) and the reference
    (FP32 expanded-form distances) part ways only at near ties: two centroids
    inside one true cluster whose FP64 gap is below the FP32 rounding of the
    expanded form.  The objective agrees closely."""
    g = load("kmeans_sep.npz")
    r = run_kmeans(g["v"], 20, 12, int(g["flags"]), int(g["seed"]), 1, 1)
    assert (r["assign"] == g["assign"]).mean() > 0.995
    np.testing.assert_allclose(r["qerr"], g["qerr"], rtol=1e-4)


def test_exact_kmeans_runs_split_path():
    """Duplicated points: the random init picks duplicates, clusters empty out
    and are split with the reference's RNG stream.  After a split the two
    centroids differ by ~1e-7 relative, so later FP32 and FP64 assignments
    legitimately part ways; the port follows the reference bit for bit (see
    test_port_kmeans_matches_reference), the exact mode must stay valid."""
    g = load("kmeans_empty.npz")
    r = run_kmeans(g["v"], int(g["k"]), int(g["niter"]), int(g["flags"]), int(g["seed"]), 1, 1)
    assert r["qerr"] > 0 and np.isfinite(r["C"]).all()
    assert r["nassign"].sum() == 600 and (r["assign"] >= 0).all()


def test_exact_kmeans_step_vs_numpy():
    rng = np.random.default_rng(11)
    v = rng.standard_normal((1500, 12)).astype(np.float32)
    c = v[rng.choice(1500, 25, replace=False)].copy()
    o = oracle()
    S = o.orc_fixed_shift(1500, 12, ptr(v))
    assign = np.empty(1500, np.int32)
    dis = np.empty(1500, np.float32)
    nassign = np.empty(25, np.int32)
    cout = np.empty_like(c)
    o.orc_kmeans_step_exact(12, 1500, 25, ptr(v), ptr(c), ptr(assign), ptr(dis), ptr(nassign),
                            ptr(cout), S)
    d64 = ((v.astype(np.float64)[:, None] - c.astype(np.float64)[None]) ** 2).sum(-1)
    np.testing.assert_array_equal(assign, d64.argmin(1))
    np.testing.assert_array_equal(dis, d64.min(1).astype(np.float32))
    fx = np.rint(v.astype(np.float64) * 2.0 ** S).astype(np.int64)
    for j in range(25):
        m = assign == j
        sums = fx[m].sum(0)
        ref = (sums.astype(np.float64) * 2.0 ** -S * (1.0 / m.sum())).astype(np.float32)
        np.testing.assert_array_equal(cout[j], ref)


def test_port_hkm_matches_reference():
    g = load("hkm.npz")
    v = g["v"]
    n, d = v.shape
    bf, nl = int(g["bf"]), int(g["nlevel"])
    cent = np.zeros((bf + bf * bf) * d, np.float32)
    assign = np.empty(n, np.int32)
    srand48(int(g["srand"]))
    rc = oracle().orc_hkm_learn(n, d, nl, bf, ptr(v), int(g["niter"]), ptr(cent), ptr(assign), 0)
    assert rc == 0
    np.testing.assert_array_equal(assign, g["assign"])
    if same_blas(g):
        np.testing.assert_array_equal(cent[:bf * d].reshape(bf, d), g["level0"])
        np.testing.assert_array_equal(cent[bf * d:].reshape(bf * bf, d), g["level1"])


def test_port_cross_distances_matches_reference():
    g = load("cross.npz")
    a, b = g["a"], g["b"]
    out = np.empty((b.shape[0], a.shape[0]), np.float32)
    oracle().orc_cross_distances_port(a.shape[1], a.shape[0], b.shape[0], ptr(a), a.shape[1],
                                      ptr(b), b.shape[1], ptr(out), a.shape[0])
    if same_blas(g):
        np.testing.assert_array_equal(out, g["dist2"])
    else:
        np.testing.assert_allclose(out, g["dist2"], rtol=1e-5, atol=1e-4)


def test_random_init_is_partial_fisher_yates():
    sel = np.empty(5, np.int32)
    oracle().orc_random_init(10, 5, 123, ptr(sel))
    assert len(set(sel.tolist())) == 5 and sel.min() >= 0 and sel.max() < 10


@pytest.mark.parametrize("name", ["kmeans_l1", "kmeans_chi2"])
def test_port_kmeans_l1_chi2_matches_reference(name):
    """The oracle's port of KMEANS_L1 / KMEANS_CHI2 (L1 / chi2 assignment
    through its knn_full port, medians / chi2 minimisers over the cluster
    columns in the reference's order) reproduces the reference's own outputs
    bit for bit; with three threads it equals the reference library called
    directly."""
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    v = g["v"]
    k, niter, flags, seed = int(g["k"]), int(g["niter"]), int(g["flags"]), int(g["seed"])
    r = run_kmeans(v, k, niter, flags, seed, 1, 0)
    for key in ("C", "dis", "assign", "nassign"):
        np.testing.assert_array_equal(r[key], g[key], err_msg=key)
    assert r["qerr"] == g["qerr"]
    R = reference()
    if R is None:
        return
    R.kmeans.restype = ctypes.c_float
    R.kmeans.argtypes = [I, I, I, I, P, I, ctypes.c_long, I, P, P, P, P]
    n, d = v.shape
    flags3 = (flags & ~0xffff) | 3
    C = np.zeros((k, d), np.float32)
    dis = np.empty(n, np.float32)
    assign = np.empty(n, np.int32)
    nassign = np.empty(k, np.int32)
    R.kmeans(d, n, k, niter, ptr(v), flags3, seed, 1, ptr(C), ptr(dis), ptr(assign), ptr(nassign))
    r3 = run_kmeans(v, k, niter, flags3, seed, 1, 0)
    for key, val in (("C", C), ("dis", dis), ("assign", assign), ("nassign", nassign)):
        np.testing.assert_array_equal(r3[key], val, err_msg=key)


def test_callers_port_matches_reference_fixtures():
    """The oracle's C restatements of the callers reproduce the reference's own
    outputs stored in tests/golden (make_golden_callers.py): k-means LSH lists
    slot for slot, the learned mixture and its posteriors, the VLAD descriptor
    -- bit for bit under the BLAS the fixtures were made with."""
    o = oracle()
    g = load("kmlsh.npz")
    vb, vq, k, nhash = g["vb"], g["vq"], int(g["k"]), int(g["nhash"])
    o.orc_kmlsh_ann.argtypes = [P, I, P, I, I, I, I, I, I, I, P, P]
    idx = np.empty((vq.shape[0], k), np.int32)
    dis = np.empty((vq.shape[0], k), np.float32)
    srand48(int(g["srand48"]))
    o.orc_kmlsh_ann(ptr(vb), vb.shape[0], ptr(vq), vq.shape[0], vb.shape[1], k, nhash, 0, 0, 1,
                    ptr(idx), ptr(dis))
    exact = same_blas(g)
    if exact:
        np.testing.assert_array_equal(idx, g["idx"])
        np.testing.assert_array_equal(dis, g["dis"])
    else:
        assert (idx == g["idx"]).mean() > 0.99
    g = load("gmm.npz")
    v, k = g["v"], int(g["k"])
    n, d = v.shape
    o.orc_gmm_learn.argtypes = [I] * 4 + [P] + [I] * 4 + [P, P, P, P]
    o.orc_gmm_compute_p.argtypes = [I, P, I, I, P, P, P, P, I, I]
    w, mu, sg = np.empty(k, np.float32), np.empty((k, d), np.float32), np.empty((k, d), np.float32)
    assert o.orc_gmm_learn(d, n, k, int(g["niter"]), ptr(v), 1, int(g["seed"]), 1, int(g["flags"]),
                           ptr(w), ptr(mu), ptr(sg), None) == 0
    p = np.empty((n, k), np.float32)
    o.orc_gmm_compute_p(n, ptr(v), d, k, ptr(w), ptr(mu), ptr(sg), ptr(p), 1, 1)
    for got, key in ((w, "w"), (mu, "mu"), (sg, "sigma"), (p, "p")):
        if exact:
            np.testing.assert_array_equal(got, g[key], err_msg=key)
        else:
            np.testing.assert_allclose(got, g[key], rtol=1e-4, atol=1e-5, err_msg=key)
    g = load("vlad.npz")
    C, v = g["C"], g["v"]
    o.orc_vlad_compute.argtypes = [I, I, P, I, P, P, I]
    desc = np.empty_like(g["desc"])
    o.orc_vlad_compute(C.shape[0], C.shape[1], ptr(C), v.shape[0], ptr(v), ptr(desc), 1)
    if exact:
        np.testing.assert_array_equal(desc, g["desc"])
    else:
        np.testing.assert_allclose(desc, g["desc"], rtol=1e-5, atol=1e-4)


def test_assign_check_and_objective_vs_numpy():
    """The sampled FP64 checker used at the benchmarked sizes agrees with a
    numpy FP64 brute force: no false alarms on the exact argmin (duplicate
    centroids tie to the lowest index, a NaN row maps to -1), every planted
    error found, and the FP64 objective equal to numpy's sum."""
    from _util import assign_mismatches, objective64
    v, _, _ = synth.gaussian_mixture(6000, 24, 40, 0.2, seed=13)
    C = np.ascontiguousarray(v[::37][:120]).copy()
    C[9] = C[4]
    v[17] = np.nan
    d64 = ((v.astype(np.float64)[:, None, :] - C.astype(np.float64)[None]) ** 2).sum(-1)
    a = np.where(np.isnan(d64).all(1), -1, np.argmin(np.nan_to_num(d64, nan=np.inf), 1))
    a = a.astype(np.int32)
    assert assign_mismatches(v, C, a) == (0, -1)
    planted = a.copy()
    planted[[5, 2000, 5999]] = (planted[[5, 2000, 5999]] + 1) % C.shape[0]
    assert assign_mismatches(v, C, planted) == (3, 5)
    ok = a >= 0
    ref = float(d64[np.nonzero(ok)[0], a[ok]].sum())
    assert abs(objective64(v, C, a) - ref) <= 1e-12 * ref


def test_knn_check_vs_exact():
    """The screened k-NN checker used at the benchmarked sizes agrees with the
    FP64 brute force (float data with exact duplicate rows, integer ties, a
    NaN base row) and finds planted errors."""
    from _util import knn_mismatches
    rng = np.random.default_rng(3)
    b = rng.standard_normal((3000, 40)).astype(np.float32)
    b[100:110] = b[7]
    q = rng.standard_normal((60, 40)).astype(np.float32)
    q[5] = b[7]
    for k in (1, 12):
        idx, _, _ = knn_exact(b, q, k)
        assert knn_mismatches(b, q, idx) == (0, -1)
        bad = idx.copy()
        bad[[4, 33], -1] = (bad[[4, 33], -1] + 1) % 3000
        assert knn_mismatches(b, q, bad) == (2, 4)
    bi = rng.integers(0, 4, (500, 8)).astype(np.float32)
    qi = rng.integers(0, 4, (30, 8)).astype(np.float32)
    idx, _, _ = knn_exact(bi, qi, 20)
    assert knn_mismatches(bi, qi, idx) == (0, -1)
    bi[3, 2] = np.nan
    idx, _, _ = knn_exact(bi, qi, 20)
    assert knn_mismatches(bi, qi, idx) == (0, -1)
