"""k-means and hierarchical k-means on the GPU against the oracle.

The oracle's exact mode implements the same semantics (FP64 nearest centroid,
ties to the lowest index; exact fixed-point centroid sums; the reference's RNG
stream for init and empty-cluster splits), so assignments, counts and
centroids must be bit-identical; distances and the objective within FP32
rounding of the FP64 values.
"""
import ctypes
import os

import numpy as np
import pytest

import yael_gb300 as yg
from _util import GOLDEN, oracle, ptr, srand48
from yael_gb300 import synth

pytestmark = pytest.mark.gpu
QUIET = yg.KMEANS_QUIET | yg.KMEANS_INIT_RANDOM | 4


def oracle_kmeans(v, k, niter, flags, seed, redo, C0=None):
    n, d = v.shape
    C = np.zeros((k, d), np.float32) if C0 is None else C0.copy()
    dis = np.empty(n, np.float32)
    assign = np.empty(n, np.int32)
    nassign = np.empty(k, np.int32)
    iters = ctypes.c_long(0)
    q = oracle().orc_kmeans(d, n, k, niter, ptr(v), flags, seed, redo, ptr(C), ptr(dis),
                            ptr(assign), ptr(nassign), 1, ctypes.addressof(iters))
    return dict(C=C, dis=dis, assign=assign, nassign=nassign, qerr=q, iters=iters.value)


def gpu_kmeans(v, k, niter, flags, seed, redo, prec, C0=None):
    n, d = v.shape
    C = np.zeros((k, d), np.float32) if C0 is None else C0.copy()
    dis = np.empty(n, np.float32)
    assign = np.empty(n, np.int32)
    nassign = np.empty(k, np.int32)
    o = yg.KmeansOpts({"fp32": 0, "bf16": 1, "bf16x3": 2, "fp16": 3}[prec], 0, None, 0, 0, 0,
                      0, 0, 0)
    q = yg.lib().yael_gpu_kmeans_ex(d, n, k, niter, ptr(v), flags, seed, redo, ptr(C), ptr(dis),
                                    ptr(assign), ptr(nassign), ctypes.byref(o))
    assert o.status == 0, yg.last_error()
    return dict(C=C, dis=dis, assign=assign, nassign=nassign, qerr=q, iters=o.iterations,
                n_band=o.n_band, prec_used=o.prec_used)


def same(g, o, rtol=2e-6):
    np.testing.assert_array_equal(g["assign"], o["assign"])
    np.testing.assert_array_equal(g["nassign"], o["nassign"])
    np.testing.assert_array_equal(g["C"], o["C"])
    np.testing.assert_allclose(g["dis"], o["dis"], rtol=rtol, atol=1e-6)
    assert abs(g["qerr"] - o["qerr"]) <= 1e-6 * abs(o["qerr"]) + 1e-12
    assert g["iters"] == o["iters"]


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_kmeans_small_k(prec):
    v, _, _ = synth.gaussian_mixture(5000, 16, 20, 0.3, seed=4)
    same(gpu_kmeans(v, 20, 12, QUIET, 1234, 1, prec), oracle_kmeans(v, 20, 12, QUIET, 1234, 1))


@pytest.mark.parametrize("prec", ["fp32", "bf16", "bf16x3", "fp16"])
def test_kmeans_large_k_knn_path(prec):
    v, _, _ = synth.gaussian_mixture(20000, 32, 128, 0.15, seed=5)
    g = gpu_kmeans(v, 100, 10, QUIET, 777, 1, prec)
    same(g, oracle_kmeans(v, 100, 10, QUIET, 777, 1))
    # the chosen form runs fp16 operands on data whose range fp16 holds
    assert g["prec_used"] == {"fp32": 0, "bf16": 3, "bf16x3": 2, "fp16": 3}[prec]


def test_kmeans_large_k_bf16_operands():
    """Values up to 255 (norms far above fp16's range): the chosen form keeps
    bf16 operands, with the same exact assignments."""
    v = synth.sift_like(12000, 64, seed=8)
    g = gpu_kmeans(v, 80, 6, QUIET, 99, 1, "bf16")
    same(g, oracle_kmeans(v, 80, 6, QUIET, 99, 1))
    assert g["prec_used"] == 1


@pytest.mark.parametrize("prec", ["fp32", "bf16", "fp16"])
def test_kmeans_k_above_256_prior_bound_pass(prec):
    """k > 256: the k-NN assignment.  From the second iteration on the chosen
    form runs a threshold pass from each point's distance to its previous
    centroid (no sample pass); iteration counts, assignments and centroids
    equal the oracle's."""
    v, _, _ = synth.gaussian_mixture(30000, 32, 500, 0.2, seed=15)
    g = gpu_kmeans(v, 400, 8, QUIET, 21, 1, prec)
    same(g, oracle_kmeans(v, 400, 8, QUIET, 21, 1))


def duplicate_heavy(seed):
    """40% of the points are one vector: random init picks many identical
    centroids.  On the k-NN assignment (k > 256) the candidate lists of those
    points tie and the certificate rejects them (band passes settle them); on
    the small-k tensor-core assignment their error bands overflow the band
    lists (every centroid is then re-checked) and the ties go to FP64."""
    v, _, _ = synth.gaussian_mixture(20000, 32, 50, 0.2, seed=seed)
    v[::5] = v[1]
    v[1::5] = v[1]
    return v


def test_kmeans_deferred_check_rejections():
    """The k-NN assignment with its certificate check deferred to the end of
    the iteration (YAEL_GPU_KMEANS_DEFER=1, read once per process: child
    process): rejected points are re-run and the update repeated; results
    bit-identical to the oracle."""
    import subprocess
    import sys
    import tempfile
    v = duplicate_heavy(31)
    with tempfile.TemporaryDirectory() as tmp:
        np.save(os.path.join(tmp, "v.npy"), v)
        code = (
            "import sys, numpy as np; sys.path.insert(0, 'tests');"
            "import test_kmeans_gpu as T;"
            f"v = np.load('{tmp}/v.npy');"
            "r = T.gpu_kmeans(v, 300, 8, T.QUIET, 5, 1, 'bf16');"
            f"np.savez('{tmp}/r.npz', **r); print('ran')")
        env = dict(os.environ, YAEL_GPU_KMEANS_DEFER="1")
        root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
        p = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, capture_output=True,
                           text=True, timeout=300)
        assert p.returncode == 0 and "ran" in p.stdout, p.stdout + p.stderr
        g = dict(np.load(os.path.join(tmp, "r.npz")))
    assert g["n_band"] > 0  # rejected points went through the re-run
    same(g, oracle_kmeans(v, 300, 8, QUIET, 5, 1))


def test_kmeans_inline_check_rejections():
    """The same data with the check in line (first iteration: adaptive mode)."""
    v = duplicate_heavy(31)
    g = gpu_kmeans(v, 300, 8, QUIET, 5, 1, "bf16")
    assert g["n_band"] > 0
    same(g, oracle_kmeans(v, 300, 8, QUIET, 5, 1))


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
@pytest.mark.parametrize("k", [100, 256])
def test_kmeans_tensor_core_assignment_ties(prec, k):
    """The small-k tensor-core assignment on duplicate-heavy data (bands wider
    than their lists, exact FP32 ties decided in FP64): bit-identical to the
    oracle.  The centroid sums come with the pass: through shared memory for
    k = 100 (k * d * 8 bytes fit), straight into the global sums for k = 256."""
    v = duplicate_heavy(31)
    g = gpu_kmeans(v, k, 8, QUIET, 5, 1, prec)
    assert g["prec_used"] == 3  # fp16 holds this data's range
    same(g, oracle_kmeans(v, k, 8, QUIET, 5, 1))


@pytest.mark.parametrize("d,k", [(4, 7), (20, 33), (96, 32), (128, 200), (256, 16), (128, 256),
                                 (256, 256)])
def test_kmeans_tensor_core_assignment_shapes(d, k):
    """Dimensions from 4 to 256 (one to four 64-column K blocks, partial
    blocks zero padded) and k not a multiple of 32 (masked accumulator
    columns), bf16 operands (values far outside fp16's range); the shared
    memory layout gives up staging and shared-memory sums where they do not
    fit, and d = 256 with k = 256 (no room for two stages) takes the k-NN
    assignment instead."""
    rng = np.random.default_rng(d * 100 + k)
    v = (rng.standard_normal((6000, d)) * 300).astype(np.float32)
    g = gpu_kmeans(v, k, 5, QUIET, 11, 1, "bf16")
    assert g["prec_used"] == 1
    same(g, oracle_kmeans(v, k, 5, QUIET, 11, 1))


def test_kmeans_empty_cluster_splits():
    g = np.load(os.path.join(GOLDEN, "kmeans_empty.npz"))
    v = g["v"]
    r = gpu_kmeans(v, 40, 20, QUIET, 77, 1, "fp32")
    same(r, oracle_kmeans(v, 40, 20, QUIET, 77, 1))


def test_kmeans_redo_keeps_best():
    g = np.load(os.path.join(GOLDEN, "kmeans_redo.npz"))
    v = g["v"]
    same(gpu_kmeans(v, 10, 10, QUIET, 5, 3, "fp32"), oracle_kmeans(v, 10, 10, QUIET, 5, 3))


@pytest.mark.parametrize("prec", ["bf16", "fp32"])
def test_kmeans_empty_cluster_splits_both_forms(prec):
    """Empty clusters split into pairs of centroids 1e-7 apart: every point of
    the original cluster is then a near tie of the pair, settled in the
    tensor-core form by the sign of the two distances' difference (or FP64);
    bit-identical to the oracle either way."""
    g = np.load(os.path.join(GOLDEN, "kmeans_empty.npz"))
    v = g["v"]
    r = gpu_kmeans(v, 40, 20, QUIET, 77, 1, prec)
    same(r, oracle_kmeans(v, 40, 20, QUIET, 77, 1))


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
def test_kmeans_large_k_splits(prec):
    """k = 300 (the k-NN assignment and its short re-rank) on points with many
    duplicates: random init draws equal centroids, the empty clusters split
    into pairs ~1e-7 of their norm apart, and the split cluster's points are
    near ties of the pair, settled by the sign of the distance difference
    (FP64 where it does not clear its bound); bit-identical to the oracle."""
    rng = np.random.default_rng(43)
    v = rng.integers(0, 4, (6000, 6)).astype(np.float32)
    r = gpu_kmeans(v, 300, 12, QUIET, 91, 1, prec)
    same(r, oracle_kmeans(v, 300, 12, QUIET, 91, 1))


@pytest.mark.parametrize("flags", [QUIET, yg.KMEANS_QUIET | yg.KMEANS_INIT_RANDOM
                                   | yg.KMEANS_NORMALIZE_CENTS])
def test_kmeans_tensor_core_redo(flags):
    """Several runs (nredo = 3) through the tensor-core assignment: each run
    starts its incremental centroid sums from zero; the best run is kept as
    in the oracle."""
    v, _, _ = synth.gaussian_mixture(9000, 32, 24, 0.25, seed=15)
    g = gpu_kmeans(v, 24, 9, flags, 321, 3, "bf16")
    assert g["prec_used"] == 3
    same(g, oracle_kmeans(v, 24, 9, flags, 321, 3))


@pytest.mark.parametrize("offset,sigma", [(40.0, 0.3), (3.0, 1e-3)])
def test_kmeans_tensor_core_centred_packing(offset, sigma):
    """Points far from the origin (40 + N(0, 0.3)): packed relative to their
    mean they fit fp16; a very tight cloud (3 + 1e-3 N(0, 1)): the centred
    centroid norms are tiny and their fp16 norm parts fall among fp16's
    subnormals.  Both exact against the oracle."""
    rng = np.random.default_rng(int(offset * 10))
    centres = rng.standard_normal((12, 48)).astype(np.float32) * (10 * sigma)
    lab = rng.integers(0, 12, 7000)
    v = (offset + centres[lab] + sigma * rng.standard_normal((7000, 48))).astype(np.float32)
    g = gpu_kmeans(v, 12, 8, QUIET, 41, 1, "bf16")
    assert g["prec_used"] == 3
    same(g, oracle_kmeans(v, 12, 8, QUIET, 41, 1))


def test_kmeans1_full_size_vs_oracle():
    """The kmeans1 configuration at full size (n = 100k, d = 128, k = 256, 20
    iterations, random init, seed 0) through the chosen form: assignments,
    counts and centroids bit-identical to the oracle's exact mode (FP64
    nearest centroid, exact sums)."""
    v, _, _ = synth.gaussian_mixture(100_000, 128, 256, 0.15, seed=0)
    srand48(0)  # seed 0: the k-means seed comes from lrand48()
    g = gpu_kmeans(v, 256, 20, QUIET, 0, 1, "bf16")
    assert g["prec_used"] == 3
    srand48(0)
    same(g, oracle_kmeans(v, 256, 20, QUIET, 0, 1))


def test_kmeans_plus_plus_init():
    g = np.load(os.path.join(GOLDEN, "kmeans_pp.npz"))
    v = g["v"]
    fl = int(g["flags"])
    same(gpu_kmeans(v, 30, 8, fl, 99, 1, "fp32"), oracle_kmeans(v, 30, 8, fl, 99, 1))


def test_kmeans_init_user_and_normalize():
    v, _, _ = synth.gaussian_mixture(3000, 24, 10, 0.2, seed=6)
    C0 = v[:10].copy()
    fl = yg.KMEANS_QUIET | yg.KMEANS_INIT_USER | yg.KMEANS_NORMALIZE_CENTS
    same(gpu_kmeans(v, 10, 6, fl, 3, 5, "fp32", C0), oracle_kmeans(v, 10, 6, fl, 3, 5, C0))


def test_kmeans_seed_zero_uses_lrand48():
    v, _, _ = synth.gaussian_mixture(2000, 8, 12, 0.2, seed=7)
    srand48(2024)
    o = oracle_kmeans(v, 12, 5, QUIET, 0, 1)
    srand48(2024)
    same(gpu_kmeans(v, 12, 5, QUIET, 0, 1, "fp32"), o)


def test_kmeans_drop_in_symbol(gpu_lib):
    v, _, _ = synth.gaussian_mixture(4000, 16, 30, 0.2, seed=8)
    n, d = v.shape
    C = np.zeros((30, d), np.float32)
    assign = np.empty(n, np.int32)
    q = gpu_lib.kmeans(d, n, 30, 10, ptr(v), QUIET, 31, 1, ptr(C), None, ptr(assign), None)
    o = oracle_kmeans(v, 30, 10, QUIET, 31, 1)
    np.testing.assert_array_equal(assign, o["assign"])
    np.testing.assert_array_equal(C, o["C"])
    assert abs(q - o["qerr"]) <= 1e-6 * o["qerr"]


def oracle_hkm(v, nlevel, bf, niter):
    n, d = v.shape
    sizes = [bf ** (l + 1) for l in range(nlevel)]
    cent = np.zeros(sum(sizes) * d, np.float32)
    assign = np.empty(n, np.int32)
    rc = oracle().orc_hkm_learn(n, d, nlevel, bf, ptr(v), niter, ptr(cent), ptr(assign), 1)
    assert rc == 0
    return cent, assign


def test_hkm_exact_vs_oracle():
    v, _, _ = synth.gaussian_mixture(30000, 16, 200, 0.1, seed=9)
    srand48(42)
    oc, oa = oracle_hkm(v, 3, 5, 10)
    srand48(42)
    levels, ga = yg.hkm(v, 3, 5, 10)
    np.testing.assert_array_equal(ga, oa)
    np.testing.assert_array_equal(np.concatenate([l.ravel() for l in levels]), oc)


@pytest.mark.parametrize("prec", ["bf16", "fp32"])
def test_hkm_chosen_form_vs_oracle(prec, monkeypatch):
    """hkm with the tensor-core assignment and fused centroid sums (bf16
    requested; fp16 operands for this data) and the plain FP32 form: the
    same tree as the oracle's exact mode, bit for bit."""
    monkeypatch.setenv("YAEL_GPU_PRECISION", prec)
    v, _, _ = synth.gaussian_mixture(40000, 96, 300, 0.1, seed=19)
    srand48(7)
    oc, oa = oracle_hkm(v, 3, 8, 6)
    srand48(7)
    levels, ga = yg.hkm(v, 3, 8, 6)
    np.testing.assert_array_equal(ga, oa)
    np.testing.assert_array_equal(np.concatenate([l.ravel() for l in levels]), oc)
    st = yg.CallStats()
    yg.lib().yael_gpu_last_stats(ctypes.byref(st))
    assert st.prec_used == (3 if prec == "bf16" else 0)
    assert st.point_iterations >= st.instance_iterations > 0


@pytest.mark.parametrize("prec", ["bf16", "fp32"])
def test_hkm_small_nodes_vs_oracle(prec, monkeypatch):
    """Nodes with fewer points than bf (small_nodes = 1: one child per point,
    the seed draw still made): the oracle's restatement of that rule gives
    the same tree, bit for bit, in both forms (and the tensor-core assignment
    runs with many small instances)."""
    monkeypatch.setenv("YAEL_GPU_PRECISION", prec)
    v, _, _ = synth.gaussian_mixture(6000, 32, 60, 0.15, seed=23)
    n, d = v.shape
    nl, bf = 3, 16
    cent = np.zeros(sum(bf ** (l + 1) for l in range(nl)) * d, np.float32)
    oa = np.empty(n, np.int32)
    srand48(3)
    assert oracle().orc_hkm_learn(n, d, nl, bf, ptr(v), 5, ptr(cent), ptr(oa), 1 | 0x100) == 0
    srand48(3)
    levels, ga = yg.hkm(v, nl, bf, 5, small_nodes=True)
    np.testing.assert_array_equal(ga, oa)
    np.testing.assert_array_equal(np.concatenate([l.ravel() for l in levels]), cent)


def test_hkm_golden_and_quantize(gpu_lib):
    g = np.load(os.path.join(GOLDEN, "hkm.npz"))
    v = g["v"]
    n, d = v.shape
    srand48(int(g["srand"]))
    ap = ctypes.POINTER(ctypes.c_int)()
    h = gpu_lib.hkm_learn(n, d, 2, 4, ptr(v), 8, 4, 0, ctypes.byref(ap))
    hk = yg.Hkm.from_address(h)
    assign = np.ctypeslib.as_array(ap, shape=(n,)).copy()
    lv0 = np.ctypeslib.as_array(hk.centroids[0], shape=(4 * d,)).reshape(4, d)
    lv1 = np.ctypeslib.as_array(hk.centroids[1], shape=(16 * d,)).reshape(16, d)
    # well separated data: the reference's FP32 path makes the same choices
    np.testing.assert_array_equal(assign, g["assign"])
    np.testing.assert_allclose(lv0, g["level0"], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(lv1, g["level1"], rtol=1e-5, atol=1e-5)
    q = np.empty(n, np.int32)
    gpu_lib.hkm_quantize(h, n, ptr(v), ptr(q))
    cent = np.concatenate([lv0.ravel(), lv1.ravel()]).astype(np.float32)
    oq = np.empty(n, np.int32)
    oracle().orc_hkm_quantize(2, 4, d, ptr(cent), n, ptr(v), ptr(oq), 1)
    np.testing.assert_array_equal(q, oq)
    gpu_lib.hkm_delete(h)
    ctypes.CDLL(None).free(ctypes.cast(ap, ctypes.c_void_p))


@pytest.mark.parametrize("name", ["kmeans_l1", "kmeans_chi2"])
def test_kmeans_l1_chi2_golden(name):
    """KMEANS_L1 (medians) and KMEANS_CHI2 (chi2 minimisers) against the
    reference's own outputs (tests/golden/make_golden_alt.py): assignments,
    counts, centroids and distances bit-identical, objective to 1e-6."""
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    v = g["v"]
    r = gpu_kmeans(v, int(g["k"]), int(g["niter"]), int(g["flags"]), int(g["seed"]), 1, "fp32")
    np.testing.assert_array_equal(r["assign"], g["assign"])
    np.testing.assert_array_equal(r["nassign"], g["nassign"])
    np.testing.assert_array_equal(r["C"], g["C"])
    np.testing.assert_array_equal(r["dis"], g["dis"])
    assert abs(r["qerr"] - float(g["qerr"])) <= 1e-6 * abs(float(g["qerr"]))
