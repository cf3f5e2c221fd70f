"""Batched uneven k-NN (yael_gpu_knn_batch) against the FP64 oracle, pair by
pair: the batch must return what a loop of knn_full calls returns."""
import ctypes
import os

import numpy as np
import pytest

import yael_gb300 as yg
from _util import knn_exact

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 8


def unit_pairs(seed, sizes, d):
    rng = np.random.default_rng(seed)
    out = []
    for nq, nb in sizes:
        q = rng.standard_normal((nq, d)).astype(np.float32)
        b = rng.standard_normal((nb, d)).astype(np.float32)
        q /= np.maximum(np.linalg.norm(q, axis=1, keepdims=True), 1e-30)
        b /= np.linalg.norm(b, axis=1, keepdims=True)
        out.append((q, b))
    return out


SIZES = [(0, 40), (1, 40), (5, 3000), (130, 700), (300, 9000), (257, 64), (64, 20000), (1, 1),
         (700, 2500)]


def dot_order(q, b, k):
    full = q.astype(np.float64) @ b.astype(np.float64).T
    ids = np.broadcast_to(np.arange(b.shape[0]), full.shape)
    order = np.lexsort((ids, full), axis=1)[:, :k]
    return order, np.take_along_axis(full, order, 1)


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
@pytest.mark.parametrize("metric", [2, 16])
def test_batch_matches_per_pair(prec, metric):
    k = 1
    pairs = unit_pairs(3, SIZES, 64)
    for kk in (1, 8):
        k = kk
        sizes_ok = [(q, b) for q, b in pairs if b.shape[0] >= k]
        out, st = yg.knn_batch(sizes_ok, nnn=k, distance_type=metric, precision=prec,
                               stats=True)
        assert len(out) == len(sizes_ok)
        for (q, b), (idx, dis) in zip(sizes_ok, out):
            if q.shape[0] == 0:
                assert idx.shape == (0, k)
                continue
            if metric == 2:
                ridx, rdis, _ = knn_exact(b, q, k, NT)
            else:
                ridx, rdis = dot_order(q, b, k)
            np.testing.assert_array_equal(idx, ridx)
            np.testing.assert_allclose(dis, rdis, rtol=2e-6, atol=2e-6)


def test_batch_rejects_small_base():
    pairs = unit_pairs(4, [(3, 5)], 16)
    with pytest.raises(RuntimeError):
        yg.knn_batch(pairs, nnn=8)


def test_batch_device_pointers():
    torch = pytest.importorskip("torch")
    pairs = unit_pairs(5, [(50, 4000), (1, 300), (200, 1000)], 32)
    dq = [torch.from_numpy(q).cuda() for q, _ in pairs]
    db = [torch.from_numpy(b).cuda() for _, b in pairs]
    k = 4
    di = [torch.empty((q.shape[0], k), dtype=torch.int32, device="cuda") for q, _ in pairs]
    dd = [torch.empty((q.shape[0], k), device="cuda") for q, _ in pairs]
    descs = (yg.KnnPair * len(pairs))()
    for i in range(len(pairs)):
        descs[i] = yg.KnnPair(pairs[i][0].shape[0], pairs[i][1].shape[0], dq[i].data_ptr(),
                              db[i].data_ptr(), di[i].data_ptr(), dd[i].data_ptr())
    stream = torch.cuda.current_stream()
    o = yg.KnnOpts(1, 2, 1, ctypes.c_void_p(stream.cuda_stream))
    rc = yg.lib().yael_gpu_knn_batch(len(pairs), ctypes.cast(descs, ctypes.c_void_p), 32, k,
                                     ctypes.byref(o))
    assert rc == 0, yg.last_error()
    for (q, b), i in zip(pairs, di):
        np.testing.assert_array_equal(i.cpu().numpy(), knn_exact(b, q, k)[0])


def _device_batch(pairs, k, metric, torch):
    dq = [torch.from_numpy(q).cuda() for q, _ in pairs]
    db = [torch.from_numpy(b).cuda() for _, b in pairs]
    di = [torch.full((q.shape[0], k), -7, dtype=torch.int32, device="cuda") for q, _ in pairs]
    dd = [torch.empty((q.shape[0], k), device="cuda") for q, _ in pairs]
    descs = (yg.KnnPair * len(pairs))()
    for i in range(len(pairs)):
        descs[i] = yg.KnnPair(pairs[i][0].shape[0], pairs[i][1].shape[0], dq[i].data_ptr(),
                              db[i].data_ptr(), di[i].data_ptr(), dd[i].data_ptr())
    stream = torch.cuda.current_stream()
    o = yg.KnnOpts(1, metric, 1, ctypes.c_void_p(stream.cuda_stream))
    d = pairs[0][0].shape[1]
    rc = yg.lib().yael_gpu_knn_batch(len(pairs), ctypes.cast(descs, ctypes.c_void_p), d, k,
                                     ctypes.byref(o))
    assert rc == 0, yg.last_error()
    torch.cuda.synchronize()
    return [(i.cpu().numpy(), x.cpu().numpy()) for i, x in zip(di, dd)], o


@pytest.mark.parametrize("metric", [2, 16])
@pytest.mark.parametrize("d", [64, 128])
def test_grouped_batch_uneven(metric, d):
    """Device arrays, BF16, k = 32: the grouped pipeline (one launch per pass).
    Pairs cover empty and single queries, bases of exactly k rows, bases where
    every row is a candidate and bases with a threshold sample, and query
    counts that are not multiples of the 128-row tile."""
    torch = pytest.importorskip("torch")
    k = 32
    sizes = [(0, 40), (1, 32), (5, 3000), (130, 700), (300, 9000), (257, 64), (64, 20000),
             (1, 33), (700, 2500), (33, 50000), (129, 12000)]
    pairs = unit_pairs(11 + d + metric, sizes, d)
    out, o = _device_batch(pairs, k, metric, torch)
    for (q, b), (idx, dis) in zip(pairs, out):
        if q.shape[0] == 0:
            continue
        if metric == 2:
            ridx, rdis, _ = knn_exact(b, q, k, NT)
        else:
            ridx, rdis = dot_order(q, b, k)
        np.testing.assert_array_equal(idx, ridx)
        np.testing.assert_allclose(dis, rdis, rtol=2e-6, atol=2e-6)


def test_grouped_batch_rejections_rerun():
    """A base with hundreds of copies of one row next to the queries overflows
    the candidate regions: those queries fail the certificate in the grouped
    pass and are settled by the single-pair pipeline; the others stay."""
    torch = pytest.importorskip("torch")
    k = 32
    rng = np.random.default_rng(21)
    d = 64
    pairs = unit_pairs(22, [(200, 30000), (50, 15000)], d)
    q, b = pairs[0]
    b = b.copy()
    b[1000:1600] = q[7]  # 600 exact copies of query 7
    b[5000:5400] = q[9] + 1e-4 * rng.standard_normal(d).astype(np.float32)
    pairs[0] = (q, b)
    out, o = _device_batch(pairs, k, 2, torch)
    assert o.n_band > 0  # the rejected queries were re-run
    for (q, b), (idx, dis) in zip(pairs, out):
        ridx, rdis, _ = knn_exact(b, q, k, NT)
        np.testing.assert_array_equal(idx, ridx)
        np.testing.assert_allclose(dis, rdis, rtol=2e-6, atol=2e-6)


@pytest.mark.parametrize("pipeline", ["1", "0"])
def test_grouped_batch_many_waves(pipeline):
    """A 3 MB wave budget splits the batch into many waves: the two buffer sets
    alternate, and with the pipeline on each wave is packed on a side stream
    while the previous wave's passes run (child process: the switches are
    read once per process)."""
    import subprocess
    import sys
    code = (
        "import sys, ctypes, numpy as np, torch; sys.path.insert(0, 'tests');"
        "import test_knn_batch_gpu as T; from _util import knn_exact;"
        "sizes = [(40, 9000), (3, 12000), (129, 20000), (1, 33), (77, 15000), (0, 50), (200, 10000)];"
        "pairs = T.unit_pairs(41, sizes, 64);"
        "out, o = T._device_batch(pairs, 16, 2, torch);"
        "ok = all((idx == knn_exact(b, q, 16)[0]).all() for (q, b), (idx, _) in zip(pairs, out) if q.shape[0]);"
        "print('waves ok' if ok else 'MISMATCH')")
    env = dict(os.environ, YAEL_GPU_GROUP_BYTES="3e6", YAEL_GPU_GROUP_PIPELINE=pipeline)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0 and "waves ok" in r.stdout, r.stdout + r.stderr
