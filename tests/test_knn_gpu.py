"""Exact k-NN parity on the GPU, through the C ABI.

The oracle is the FP64 brute force (canonical order: distance, then base id);
the reference's own outputs (tests/golden) are checked modulo its
heap-history tie order.  Every distance pass is covered: the plain FP32
CUDA-core path, the BF16 and FP16 tensor-core paths with exact re-rank and
the 3xBF16 split.
"""
import ctypes
import os

import numpy as np
import pytest

import yael_gb300 as yg
from _util import GOLDEN, check_knn_ties, exact_dist64, knn_exact, knn_port, ptr
from yael_gb300 import synth

pytestmark = pytest.mark.gpu
PRECS = ["fp32", "bf16"]
NT = os.cpu_count() or 8


def gpu_knn(b, q, k, prec, dt=2):
    idx, dis, st = yg.knn(q, b, nnn=k, distance_type=dt, precision=prec, stats=True)
    return idx, dis, st


def assert_exact(b, q, k, prec, rtol=2e-6):
    idx, dis, st = gpu_knn(b, q, k, prec)
    ridx, rdis, r64 = knn_exact(b, q, k, NT)
    mism = np.nonzero((idx != ridx).any(1))[0]
    if len(mism):
        # only FP64-exact ties may differ (equal distance, different id order is impossible
        # with ties by id, so any mismatch is an error unless distances tie exactly)
        d_gpu = exact_dist64(b, q, idx)
        bad = check_knn_ties(idx, d_gpu, ridx, r64)
        assert bad == 0, f"{prec}: {len(mism)} rows differ, first {mism[:5]}"
    np.testing.assert_allclose(dis, rdis, rtol=rtol, atol=1e-6 * max(1.0, float(np.abs(rdis).max())))
    return st


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("k", [1, 5, 37])
def test_golden_integer_ties(prec, k):
    g = np.load(os.path.join(GOLDEN, "knn_int.npz"))
    b, q = g["b"], g["q"]
    idx, dis, st = gpu_knn(b, q, k, prec)
    ridx, rdis, r64 = knn_exact(b, q, k)
    np.testing.assert_array_equal(idx, ridx)          # canonical order, ties by id
    np.testing.assert_array_equal(dis, g[f"dis_k{k}"])  # exact integers, same as the reference
    assert check_knn_ties(g[f"idx_k{k}"], exact_dist64(b, q, g[f"idx_k{k}"]), idx, r64) == 0
    assert st["exact_class"] == 1


@pytest.mark.parametrize("prec", PRECS + ["fp16"])
def test_golden_float(prec):
    g = np.load(os.path.join(GOLDEN, "knn_float.npz"))
    assert_exact(g["b"], g["q"], 10, prec)
    idx, dis, _ = gpu_knn(g["b"], g["q"], 1, prec)
    np.testing.assert_array_equal(idx, g["idx_k1"])


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
def test_k1_near_twin_rows(prec):
    """Base rows in pairs ~2e-7 of their norm apart (as an empty-cluster split
    leaves them): a query near a pair is a near tie in FP32, settled by the
    sign of the two distances' difference; ids identical to the FP64 oracle."""
    rng = np.random.default_rng(41)
    b0 = rng.standard_normal((6000, 64)).astype(np.float32)
    tw = rng.choice(6000, 1500, replace=False)
    e = (rng.standard_normal((1500, 64)) *
         (np.linalg.norm(b0[tw], axis=1, keepdims=True) * 1e-7)).astype(np.float32)
    b = np.concatenate([b0, b0[tw] - e]).astype(np.float32)
    b[tw] += e
    q = (b0[rng.choice(tw, 4000)] + 0.05 * rng.standard_normal((4000, 64))).astype(np.float32)
    idx, dis, _ = gpu_knn(b, q, 1, prec)
    ridx, rdis, _ = knn_exact(b, q, 1, NT)
    np.testing.assert_array_equal(idx, ridx)
    np.testing.assert_allclose(dis, rdis, rtol=5e-6, atol=1e-7)


@pytest.mark.parametrize("prec", PRECS + ["bf16x3", "fp16"])
@pytest.mark.parametrize("nq,nb,d,k", [(1, 1, 1, 1), (7, 5, 3, 5), (33, 300, 129, 17),
                                        (130, 2000, 64, 100), (300, 9000, 96, 33),
                                        (257, 1000, 7, 1), (64, 3000, 200, 250),
                                        (100, 5000, 300, 10)])
def test_shapes_gaussian(prec, nq, nb, d, k):
    rng = np.random.default_rng(nq * 7 + nb + d)
    b = rng.standard_normal((nb, d)).astype(np.float32)
    q = rng.standard_normal((nq, d)).astype(np.float32)
    assert_exact(b, q, k, prec)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("k", [1, 10, 100])
def test_sift_like_medium(prec, k):
    b = synth.sift_like(120_000, 128, seed=1)
    q = synth.sift_like(300, 128, seed=2)
    idx, dis, st = gpu_knn(b, q, k, prec)
    ridx, rdis, _ = knn_exact(b, q, k, NT)
    np.testing.assert_array_equal(idx, ridx)
    np.testing.assert_array_equal(dis, rdis)
    assert st["exact_class"] == 1 and st["n_fallback"] == 0


@pytest.mark.parametrize("prec", PRECS + ["bf16x3", "fp16"])
def test_unit_vectors_oversampled(prec):
    b = synth.unit_gaussian(50_000, 128, seed=3)
    q = synth.unit_gaussian(200, 128, seed=4)
    st = assert_exact(b, q, 32, prec)
    assert st["n_fallback"] <= 2


@pytest.mark.parametrize("prec", PRECS)
def test_k_equals_nb_and_duplicates(prec):
    rng = np.random.default_rng(9)
    b = rng.integers(0, 3, (50, 4)).astype(np.float32)   # many exact duplicates
    q = rng.integers(0, 3, (20, 4)).astype(np.float32)
    for k in (50, 13, 1):
        idx, dis, _ = gpu_knn(b, q, k, prec)
        ridx, rdis, _ = knn_exact(b, q, k)
        np.testing.assert_array_equal(idx, ridx)
        np.testing.assert_array_equal(dis, rdis)


@pytest.mark.parametrize("k", [1, 10])
def test_fp16_rows_out_of_range_still_exact(k):
    """Rows fp16 cannot hold (here ||b||^2 up to ~6e6 > 2^15, and query values
    of 4e4 whose -2q overflows) get an infinite error bound: their queries
    fail the certificate and the later passes (3xBF16 band, FP64) settle them."""
    b = synth.sift_like(6000, 64, seed=21)
    q = synth.sift_like(50, 64, seed=22)
    q[::7, 3] = 4.0e4
    idx, dis, st = gpu_knn(b, q, k, "fp16")
    ridx, rdis, _ = knn_exact(b, q, k)
    np.testing.assert_array_equal(idx, ridx)
    np.testing.assert_array_equal(dis, rdis)
    assert st["n_band"] + st["n_second"] + st["n_fallback"] > 0


def test_nan_rows_follow_reference_padding():
    rng = np.random.default_rng(5)
    b = rng.standard_normal((400, 16)).astype(np.float32)
    q = rng.standard_normal((6, 16)).astype(np.float32)
    q[2, 3] = np.nan
    for k in (1, 4):
        idx, dis, _ = gpu_knn(b, q, k, "fp32")
        pidx, pdis = knn_port(b, q, k, nt=1)
        np.testing.assert_array_equal(idx[2], pidx[2])
        np.testing.assert_array_equal(dis[2].view(np.uint32), pdis[2].view(np.uint32))
        ok = [0, 1, 3, 4, 5]
        np.testing.assert_array_equal(idx[ok], knn_exact(b, q[ok], k)[0])


@pytest.mark.parametrize("prec", PRECS + ["fp16"])
@pytest.mark.parametrize("k", [7, 1])
def test_dot_product_metric(prec, k):
    """k = 1 takes the short re-rank's k = 1 form (reductions, FP32 certificate)."""
    rng = np.random.default_rng(6)
    b = rng.standard_normal((3000, 40)).astype(np.float32)
    q = rng.standard_normal((50, 40)).astype(np.float32)
    idx, dis, _ = gpu_knn(b, q, k, prec, dt=16)
    full = q.astype(np.float64) @ b.astype(np.float64).T
    order = np.lexsort((np.broadcast_to(np.arange(3000), full.shape), full), axis=1)[:, :k]
    np.testing.assert_array_equal(idx, order)
    np.testing.assert_allclose(dis, np.take_along_axis(full, order, 1), rtol=1e-5, atol=1e-5)


def test_weights_drop_in(gpu_lib):
    rng = np.random.default_rng(8)
    b = rng.standard_normal((800, 12)).astype(np.float32)
    q = rng.standard_normal((30, 12)).astype(np.float32)
    w = rng.uniform(0.5, 2.0, 800).astype(np.float32)
    idx = np.empty((30, 6), np.int32)
    dis = np.empty((30, 6), np.float32)
    gpu_lib.knn_full(2, 30, 800, 12, 6, ptr(b), ptr(q), ptr(w), ptr(idx), ptr(dis))
    full = ((q.astype(np.float64)[:, None] - b.astype(np.float64)[None]) ** 2).sum(-1) * w
    order = np.lexsort((np.broadcast_to(np.arange(800), full.shape), full), axis=1)[:, :6]
    np.testing.assert_array_equal(idx, order)


def test_drop_in_wrappers(gpu_lib):
    rng = np.random.default_rng(10)
    b = rng.standard_normal((500, 9)).astype(np.float32)
    v = rng.standard_normal((70, 9)).astype(np.float32)
    assign = np.empty(70, np.int32)
    s = gpu_lib.nn(70, 500, 9, ptr(b), ptr(v), ptr(assign))
    ridx, rdis, _ = knn_exact(b, v, 1)
    np.testing.assert_array_equal(assign, ridx[:, 0])
    assert abs(s - float(rdis.astype(np.float64).sum())) < 1e-4 * s
    idx = np.empty((70, 4), np.int32)
    p = gpu_lib.knn_thread(70, 500, 9, 4, ptr(b), ptr(v), ptr(idx), 8)
    dis = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_float)), shape=(70, 4)).copy()
    ctypes.CDLL(None).free(ctypes.c_void_p(p))
    np.testing.assert_array_equal(idx, knn_exact(b, v, 4)[0])
    np.testing.assert_allclose(dis, knn_exact(b, v, 4)[1], rtol=1e-5)


def test_cross_distances_vs_golden_and_fp64():
    g = np.load(os.path.join(GOLDEN, "cross.npz"))
    a, b = g["a"], g["b"]
    dis = yg.cross_distances(a, b)
    np.testing.assert_allclose(dis, g["dist2"], rtol=1e-5, atol=1e-4)
    full = ((b.astype(np.float64)[:, None] - a.astype(np.float64)[None]) ** 2).sum(-1)
    np.testing.assert_allclose(dis, full, rtol=1e-5, atol=1e-4)
    dot = yg.cross_distances(a, b, distance_type=16)
    np.testing.assert_allclose(dot, b.astype(np.float64) @ a.astype(np.float64).T, rtol=1e-5,
                               atol=1e-4)


def test_cross_distances_nonpacked_leaves_padding(gpu_lib):
    rng = np.random.default_rng(12)
    a = rng.standard_normal((20, 5)).astype(np.float32)
    b = rng.standard_normal((300, 5)).astype(np.float32)
    out = np.full((300, 25), 7.0, np.float32)  # ldd = 25 > na = 20
    gpu_lib.compute_cross_distances_nonpacked(5, 20, 300, ptr(a), 5, ptr(b), 5, ptr(out), 25)
    assert (out[:, 20:] == 7.0).all()
    full = ((b.astype(np.float64)[:, None] - a.astype(np.float64)[None]) ** 2).sum(-1)
    np.testing.assert_allclose(out[:, :20], full, rtol=1e-5, atol=1e-5)


def test_reorder_shortlist_and_recompute(gpu_lib):
    rng = np.random.default_rng(13)
    b = rng.standard_normal((1000, 24)).astype(np.float32)
    v = rng.standard_normal((40, 24)).astype(np.float32)
    idx = rng.integers(0, 1000, (40, 16)).astype(np.int32)
    idx[3, 10:] = -1  # short list stops at the first negative id
    dis = np.zeros((40, 16), np.float32)
    before = idx.copy()
    gpu_lib.knn_reorder_shortlist(40, 1000, 24, 16, ptr(b), ptr(v), ptr(idx), ptr(dis))
    for r in range(40):
        ki = 16 if r != 3 else 10
        d = ((v[r].astype(np.float64) - b[before[r, :ki]].astype(np.float64)) ** 2).sum(1)
        o = np.lexsort((np.arange(ki), d))
        np.testing.assert_array_equal(idx[r, :ki], before[r, :ki][o])
        np.testing.assert_allclose(dis[r, :ki], d[o], rtol=1e-6)
        np.testing.assert_array_equal(idx[r, ki:], before[r, ki:])
    # recompute over a base slice [label0, label0 + nb)
    srt = np.sort(rng.integers(0, 1000, (40, 8)), axis=1).astype(np.int32)
    kp = np.zeros(40, np.int32)
    d2 = np.zeros((40, 8), np.float32)
    gpu_lib.knn_recompute_exact_dists(40, 500, 24, 8, ptr(b), ptr(v), 0, ptr(kp), ptr(srt), ptr(d2))
    for r in range(40):
        n_in = int((srt[r] < 500).sum())
        assert kp[r] == n_in
        d = ((v[r].astype(np.float64) - b[srt[r, :n_in]].astype(np.float64)) ** 2).sum(1)
        np.testing.assert_array_equal(d2[r, :n_in], d.astype(np.float32))


def test_split_pass_settles_bf16_rejections():
    """Clustered float data with close neighbours: the BF16 certificate rejects
    many queries; the 3xBF16 second pass must settle them with exact ids."""
    v, _, _ = synth.gaussian_mixture(60000, 64, 30, 0.05, seed=31)
    q, _, _ = synth.gaussian_mixture(400, 64, 30, 0.05, seed=31)
    st = assert_exact(v, q, 1, "bf16")
    assert st["n_fallback"] <= 5
    st = assert_exact(v, q, 3, "bf16")
    assert st["n_fallback"] <= 5


def shell_data(nb=4000, nq=64, d=64, seed=41):
    """Base rows on thin shells around a far-away centre: the BF16 error bound
    dwarfs the spread of the distances, so every later-chance pass runs."""
    rng = np.random.default_rng(seed)
    c = rng.standard_normal(d) * 3.0
    u = rng.standard_normal((nb, d))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    r = 1.0 + 0.5 * rng.random(nb)
    b = (c + r[:, None] * u).astype(np.float32)
    q = (c + 1e-3 * rng.standard_normal((nq, d))).astype(np.float32)
    return b, q


@pytest.mark.parametrize("prec", ["fp32", "bf16", "bf16x3", "fp16"])
@pytest.mark.parametrize("k", [1, 5])
def test_later_chance_chain(prec, k):
    b, q = shell_data()
    st = assert_exact(b, q, k, prec)
    assert st["n_fallback"] <= 2
    if prec == "bf16":
        assert st["n_band"] > 0 and st["n_second"] > 0


def test_cta_pair_kernel_matches():
    """The CTA-pair form of the tensor-core pass (tcgen05 cta_group::2, chosen
    with YAEL_GPU_TC_PAIR=1) gives the same exact results; run in a child
    process since the switch is read once per process."""
    import subprocess
    import sys
    code = (
        "import numpy as np, sys; sys.path.insert(0, 'tests');"
        "from _util import knn_exact; import yael_gb300 as yg;"
        "rng = np.random.default_rng(77);"
        "b = rng.standard_normal((20000, 128)).astype(np.float32);"
        "q = rng.standard_normal((700, 128)).astype(np.float32);"
        "i1, d1 = yg.knn(q, b, nnn=10, precision='bf16');"
        "i2, d2 = yg.knn(q, b, nnn=1, precision='bf16x3');"
        "r1 = knn_exact(b, q, 10)[0]; r2 = knn_exact(b, q, 1)[0];"
        "assert (i1 == r1).all() and (i2 == r2).all(); print('pair ok')")
    env = dict(os.environ, YAEL_GPU_TC_PAIR="1")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0 and "pair ok" in r.stdout, r.stdout + r.stderr


@pytest.mark.parametrize("k", [1, 8, 100])
def test_host_upload_in_parts(k):
    """Host arrays with a large base go up in parts overlapped with the passes
    (thresholds from the first part); ids are still exact, including a base
    whose parts differ (sorted rows: part 0 is not representative)."""
    rng = np.random.default_rng(91)
    nb, nq, d = 300_000, 300, 64
    b = rng.standard_normal((nb, d)).astype(np.float32)
    b = b[np.argsort(b[:, 0])]  # ordered rows: a worst case for the first-part sample
    q = rng.standard_normal((nq, d)).astype(np.float32)
    idx, dis, st = gpu_knn(b, q, k, "bf16")
    ridx, rdis, r64 = knn_exact(b, q, k, NT)
    mism = np.nonzero((idx != ridx).any(1))[0]
    if len(mism):
        assert check_knn_ties(idx, exact_dist64(b, q, idx), ridx, r64) == 0
    np.testing.assert_allclose(dis, rdis, rtol=2e-6, atol=1e-5)
