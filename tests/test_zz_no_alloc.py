"""yael_gpu_knn_noalloc: the k-NN entry point for callers that cannot let the
library allocate GPU memory (their device memory belongs to their own pool,
or a cudaMalloc would stall a latency-critical path).  It must give the same
results as the regular entry point, call after call, while its scratch lives
in one static device array that every call reuses."""
import ctypes

import numpy as np
import pytest

import yael_gb300 as yg
from yael_gb300 import synth

pytestmark = pytest.mark.gpu


def reference_call(b, q, k):
    # the regular entry point, plain FP32 pass
    return yg.knn(q, b, nnn=k, precision="fp32")


def noalloc_call(L, torch, b, q, k):
    db, dq = torch.from_numpy(b).cuda(), torch.from_numpy(q).cuda()
    idx = torch.full((q.shape[0], k), -7, dtype=torch.int32, device="cuda")
    dis = torch.full((q.shape[0], k), -7.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = L.yael_gpu_knn_noalloc(q.shape[0], b.shape[0], b.shape[1], k, db.data_ptr(),
                                dq.data_ptr(), idx.data_ptr(), dis.data_ptr(), None)
    assert rc == 0, yg.last_error()
    return idx.cpu().numpy(), dis.cpu().numpy()


def tie_heavy(seed):
    """40 exact copies of one float row in the base and queries equal to it:
    the k-th and the list's last entries tie, the FP32 certificate rejects
    those queries and the exhaustive FP64 path (batched in the static
    scratch) settles them."""
    rng = np.random.default_rng(seed)
    b = rng.standard_normal((5000, 24)).astype(np.float32)
    b[1000:1040] = b[7]
    q = rng.standard_normal((64, 24)).astype(np.float32)
    q[::2] = b[7]
    return b, q, 4


def test_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    from _util import knn_exact
    L = yg.lib()
    cases = [
        (synth.gaussian_mixture(20000, 48, 64, 0.3, seed=21)[0],
         synth.gaussian_mixture(300, 48, 64, 0.3, seed=22)[0], 10),
        (synth.sift_like(30000, 128, seed=23), synth.sift_like(200, 128, seed=24), 16),
        tie_heavy(25),
    ]
    for b, q, k in cases:
        ridx, rdis = reference_call(b, q, k)
        oidx, odis, _ = knn_exact(b, q, k)  # the oracle's FP64 (distance, id) order
        np.testing.assert_array_equal(ridx, oidx)
        for _ in range(2):  # two calls in a row share (and must reset) the scratch
            idx, dis = noalloc_call(L, torch, b, q, k)
            np.testing.assert_array_equal(idx, ridx)
            np.testing.assert_array_equal(idx, oidx)
            np.testing.assert_allclose(dis, rdis, rtol=2e-6, atol=1e-6)
            np.testing.assert_allclose(dis, odis, rtol=2e-6, atol=1e-6)


def test_noalloc_allocates_no_device_memory():
    """After a first call (which may load the library's kernels), further
    calls leave the device's free memory exactly as it was."""
    torch = pytest.importorskip("torch")
    L = yg.lib()
    b, q, k = tie_heavy(26)
    db, dq = torch.from_numpy(b).cuda(), torch.from_numpy(q).cuda()
    idx = torch.empty((q.shape[0], k), dtype=torch.int32, device="cuda")
    dis = torch.empty((q.shape[0], k), dtype=torch.float32, device="cuda")
    args = (q.shape[0], b.shape[0], b.shape[1], k, db.data_ptr(), dq.data_ptr(), idx.data_ptr(),
            dis.data_ptr(), None)
    assert L.yael_gpu_knn_noalloc(*args) == 0, yg.last_error()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert L.yael_gpu_knn_noalloc(*args) == 0, yg.last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    L = yg.lib()
    dummy = torch.zeros(16, device="cuda")
    p = dummy.data_ptr()
    # k above its maximum
    assert L.yael_gpu_knn_noalloc(10, 100, 4, 17, p, p, p, p, None) != 0
    assert "16" in yg.last_error()
    # a base too large for the static scratch (checked before any GPU work)
    assert L.yael_gpu_knn_noalloc(10, 4_000_000, 4, 1, p, p, p, p, None) != 0
    assert "scratch" in yg.last_error()
