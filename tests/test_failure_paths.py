"""Failure paths, none of which faults, traps or hangs the GPU.

* A bounded wait that expires: the tensor-core kernels' producers are told
  (YAEL_GPU_TEST_WITHHOLD_LOADS, read at every launch) to issue no load, so
  the consumers' waits run out after the call's wait_limit_us; the call
  returns YAEL_GPU_ETIMEOUT and the next call on the same context is exact.
* An out-of-memory workspace growth, made on the host
  (YAEL_GPU_TEST_FAIL_ALLOC: the n-th growth fails as cudaMalloc would).
* The reference's own error exits: k-means abandoning after too many
  empty-cluster splits (yael/kmeans.c:302-306, returns -1), hkm stopping on an
  empty node (yael/hkm.c:77-80, exit(1); run in a child process), k > nb
  (yael/nn.c:456).
* compute_distances_1 and its variants (yael/nn.c:132-162, 830-860), which
  nothing else in the suite calls, against FP64.
"""
import ctypes
import os
import subprocess
import sys
import threading

import numpy as np
import pytest

import yael_gb300 as yg
from _util import knn_exact, oracle, ptr, srand48
from yael_gb300 import synth

ETIMEOUT, ENOMEM, EARG = 5, 4, 2
QUIET = yg.KMEANS_QUIET | yg.KMEANS_INIT_RANDOM


def knn_ex(b, q, k, prec, wait_us=0):
    nq, d = q.shape
    idx = np.full((nq, k), -7, np.int32)
    dis = np.empty((nq, k), np.float32)
    o = yg.KnnOpts(prec, 2, 0, None)
    o.wait_limit_us = wait_us
    rc = yg.lib().yael_gpu_knn_ex(nq, b.shape[0], d, k, ptr(b), ptr(q), ptr(idx), ptr(dis),
                                  ctypes.byref(o))
    return rc, idx, dis


def kmeans_ex(v, k, niter, prec, wait_us=0, seed=5):
    n, d = v.shape
    C = np.zeros((k, d), np.float32)
    assign = np.empty(n, np.int32)
    o = yg.KmeansOpts(prec, 0, None)
    o.wait_limit_us = wait_us
    q = yg.lib().yael_gpu_kmeans_ex(d, n, k, niter, ptr(v), QUIET, seed, 1, ptr(C), None,
                                    ptr(assign), None, ctypes.byref(o))
    return o.status, q, C, assign


@pytest.mark.gpu
@pytest.mark.parametrize("k", [1, 10])
def test_bounded_wait_expires_then_next_call_exact(k, monkeypatch):
    b = synth.unit_gaussian(20000, 64, seed=3)
    q = synth.unit_gaussian(300, 64, seed=4)
    monkeypatch.setenv("YAEL_GPU_TEST_WITHHOLD_LOADS", "1")
    rc, _, _ = knn_ex(b, q, k, yg.PREC_BF16, wait_us=2000)
    assert rc == ETIMEOUT, yg.last_error()
    assert "bounded wait" in yg.last_error()
    monkeypatch.delenv("YAEL_GPU_TEST_WITHHOLD_LOADS")
    rc, idx, _ = knn_ex(b, q, k, yg.PREC_BF16)
    assert rc == 0, yg.last_error()
    ridx, _, _ = knn_exact(b, q, k)
    np.testing.assert_array_equal(idx, ridx)


@pytest.mark.gpu
def test_bounded_wait_expires_in_kmeans_assignment(monkeypatch):
    """The small-k tensor-core assignment of k-means: the call reports the
    expired wait, and the next run is the oracle's."""
    v, _, _ = synth.gaussian_mixture(8000, 32, 40, 0.2, seed=6)
    monkeypatch.setenv("YAEL_GPU_TEST_WITHHOLD_LOADS", "1")
    status, q, _, _ = kmeans_ex(v, 32, 4, yg.PREC_BF16, wait_us=2000)
    assert status == ETIMEOUT and q == -2.0, yg.last_error()
    monkeypatch.delenv("YAEL_GPU_TEST_WITHHOLD_LOADS")
    status, q, C, assign = kmeans_ex(v, 32, 4, yg.PREC_BF16)
    assert status == 0, yg.last_error()
    Co = np.zeros_like(C)
    ao = np.empty_like(assign)
    oracle().orc_kmeans(32, v.shape[0], 32, 4, ptr(v), QUIET, 5, 1, ptr(Co), None, ptr(ao), None,
                        1, None)
    np.testing.assert_array_equal(assign, ao)
    np.testing.assert_array_equal(C, Co)


@pytest.mark.gpu
def test_workspace_out_of_memory_reported_then_recovered():
    """A fresh host thread (a fresh context and workspace) whose first
    workspace growth fails: the call returns YAEL_GPU_ENOMEM; the thread's
    next call allocates and is exact."""
    b = synth.unit_gaussian(5000, 32, seed=7)
    q = synth.unit_gaussian(50, 32, seed=8)
    out = {}

    def worker():
        os.environ["YAEL_GPU_TEST_FAIL_ALLOC"] = "1"
        try:
            out["rc1"] = knn_ex(b, q, 5, yg.PREC_FP32)[0]
            out["msg"] = yg.last_error()
        finally:
            del os.environ["YAEL_GPU_TEST_FAIL_ALLOC"]
        out["rc2"], out["idx"], _ = knn_ex(b, q, 5, yg.PREC_FP32)

    t = threading.Thread(target=worker)
    t.start()
    t.join()
    assert out["rc1"] == ENOMEM and "cudaMalloc" in out["msg"]
    assert out["rc2"] == 0
    np.testing.assert_array_equal(out["idx"], knn_exact(b, q, 5)[0])


def abandon_data():
    """3000 copies of one point: random init gives 1500 equal centroids, every
    point goes to the first (ties to the lowest index), 1499 clusters are
    empty and get split, which passes the abandon limit at once."""
    return np.full((3000, 8), 0.5, np.float32)


def test_oracle_kmeans_abandons():
    v = abandon_data()
    C = np.zeros((1500, 8), np.float32)
    q = oracle().orc_kmeans(8, 3000, 1500, 5, ptr(v), QUIET, 3, 1, ptr(C), None, None, None, 0,
                            None)
    assert q == -1.0


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_kmeans_abandons_like_the_reference(prec, gpu_lib, monkeypatch):
    v = abandon_data()
    C = np.zeros((1500, 8), np.float32)
    monkeypatch.setenv("YAEL_GPU_PRECISION", prec)
    q = gpu_lib.kmeans(8, 3000, 1500, 5, ptr(v), QUIET, 3, 1, ptr(C), None, None, None)
    assert q == -1.0
    qo = oracle().orc_kmeans(8, 3000, 1500, 5, ptr(v), QUIET, 3, 1, ptr(C), None, None, None, 1,
                             None)
    assert qo == -1.0


def empty_node_data():
    """64 copies of one point: level 0 of a bf = 2 tree starts from two equal
    centroids, every point goes to the first, and after its single iteration
    the second child is still empty (the split moved its centroid but nothing
    was reassigned yet): level 1 meets an empty node, the first node it
    visits with fewer than bf points."""
    return np.full((64, 4), 0.25, np.float32)


def test_oracle_hkm_reports_empty_node():
    v = empty_node_data()
    cent = np.zeros((2 + 4) * 4, np.float32)
    srand48(1)
    assert oracle().orc_hkm_learn(64, 4, 2, 2, ptr(v), 1, ptr(cent), None, 1) == -1


@pytest.mark.gpu
def test_hkm_exits_on_empty_node():
    """hkm_learn leaves the process with exit(1) and the reference's message,
    as yael/hkm.c:77-80 does (a child process)."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys, numpy as np; sys.path.insert(0, 'tests');"
            "import test_failure_paths as T, yael_gb300 as yg; from _util import ptr, srand48;"
            "L = yg.lib(); v = T.empty_node_data(); srand48(1);"
            "L.hkm_learn(64, 4, 2, 2, ptr(v), 1, 1, 0, None); print('returned')")
    p = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True,
                       timeout=300)
    assert p.returncode == 1, p.stdout + p.stderr
    assert "Problem2" in p.stderr and "returned" not in p.stdout


@pytest.mark.gpu
def test_k_greater_than_nb_refused():
    b = synth.unit_gaussian(10, 16, seed=1)
    q = synth.unit_gaussian(3, 16, seed=2)
    rc, _, _ = knn_ex(b, q, 11, yg.PREC_FP32)
    assert rc == EARG and "k=11 > nb=10" in yg.last_error()


@pytest.mark.gpu
def test_compute_distances_1_variants_vs_fp64(gpu_lib):
    rng = np.random.default_rng(12)
    d, nb, ldb = 37, 2000, 41
    a = rng.standard_normal(d).astype(np.float32)
    bp = rng.standard_normal((nb, ldb)).astype(np.float32)  # rows of ldb floats, d used
    b = np.ascontiguousarray(bp[:, :d])
    ref = ((b.astype(np.float64) - a.astype(np.float64)) ** 2).sum(1)
    tol = dict(rtol=1e-5, atol=1e-5 * float(ref.max()))
    out = np.empty(nb, np.float32)
    gpu_lib.compute_distances_1(d, nb, ptr(a), ptr(b), ptr(out))
    np.testing.assert_allclose(out, ref, **tol)
    gpu_lib.compute_distances_1_thread(d, nb, ptr(a), ptr(b), ptr(out), 4)
    np.testing.assert_allclose(out, ref, **tol)
    out[:] = -1
    gpu_lib.compute_distances_1_nonpacked(d, nb, ptr(a), ptr(bp), ldb, ptr(out))
    np.testing.assert_allclose(out, ref, **tol)
    out[:] = -1
    gpu_lib.compute_distances_1_nonpacked_thread(d, nb, ptr(a), ptr(bp), ldb, ptr(out), 3)
    np.testing.assert_allclose(out, ref, **tol)
