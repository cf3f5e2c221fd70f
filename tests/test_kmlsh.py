"""k-means LSH (yael/kmlsh.c).  The oracle's restatement (orc_kmlsh_ann) in
the reference's arithmetic is bit-identical to the reference library compiled
here, list slots included (CPU); the list merge, the index accessors and the
files are compared with the reference directly (CPU); the GPU library equals
the restatement in the exact arithmetic on integer-valued vectors, where every
distance between vectors is exact (GPU)."""
import ctypes

import numpy as np
import pytest

import yael_gb300 as yg
from _util import oracle, read_bytes, reference, srand48

P = ctypes.c_void_p
I = ctypes.c_int
ORC_PORT, ORC_EXACT = 0, 1


class NNList(ctypes.Structure):
    _fields_ = [("n", ctypes.c_long), ("k", ctypes.c_long), ("idx", ctypes.POINTER(ctypes.c_int)),
                ("dis", ctypes.POINTER(ctypes.c_float))]


class KmLsh(ctypes.Structure):
    _fields_ = [("nhash", I), ("d", I), ("nclust", I),
                ("centroids", ctypes.POINTER(ctypes.POINTER(ctypes.c_float)))]


class KmLshIdx(ctypes.Structure):
    _fields_ = [("nhash", I), ("n", I), ("nclust", I), ("perm", ctypes.POINTER(I)),
                ("boundaries", ctypes.POINTER(I))]


def ptr(a):
    return a.ctypes.data_as(P)


def bind(lib):
    for name, (res, args) in yg.SIGNATURES.items():
        if name.startswith(("nnlist_", "kmlsh_", "kmeans_cohash")) and hasattr(lib, name):
            getattr(lib, name).restype = res
            getattr(lib, name).argtypes = args
    return lib


def lists(lp):
    nl = ctypes.cast(lp, ctypes.POINTER(NNList)).contents
    n, k = nl.n, nl.k
    idx = np.ctypeslib.as_array(nl.idx, shape=(n * k,)).reshape(n, k).copy()
    dis = np.ctypeslib.as_array(nl.dis, shape=(n * k,)).reshape(n, k).copy()
    return idx, dis


def orc_ann(vb, vq, k, nhash, vec_type, mode, nt=1):
    o = oracle()
    o.orc_kmlsh_ann.argtypes = [P, I, P, I, I, I, I, I, I, I, P, P]
    nq, d = vq.shape
    idx = np.empty((nq, k), np.int32)
    dis = np.empty((nq, k), np.float32)
    o.orc_kmlsh_ann(ptr(vb), vb.shape[0], ptr(vq), nq, d, k, nhash, vec_type, mode, nt,
                    ptr(idx), ptr(dis))
    return idx, dis


def lib_ann(lib, vb, vq, k, nhash, nt=1):
    nq, d = vq.shape
    fn = lib.kmlsh_ann_bvec if vb.dtype == np.uint8 else lib.kmlsh_ann_fvec
    lp = fn(ptr(vb), vb.shape[0], ptr(vq), nq, d, k, nhash, nt)
    out = lists(lp)
    lib.nnlist_delete(lp)
    return out


def clustered(seed, nb, nq, d, ncl=40):
    rng = np.random.default_rng(seed)
    C = rng.standard_normal((ncl, d)) * 3
    vb = (C[rng.integers(0, ncl, nb)] + rng.standard_normal((nb, d))).astype(np.float32)
    vq = (C[rng.integers(0, ncl, nq)] + rng.standard_normal((nq, d))).astype(np.float32)
    return vb, vq


def byte_rows(seed, nb, nq, d, ncl=30):
    """Integer rows in 0..255 around ncl centres: squared distances between
    rows are exact in float32 (d * 255^2 < 2^24)."""
    rng = np.random.default_rng(seed)
    C = rng.integers(40, 216, (ncl, d))
    vb = np.clip(C[rng.integers(0, ncl, nb)] + rng.integers(-30, 31, (nb, d)), 0, 255)
    vq = np.clip(C[rng.integers(0, ncl, nq)] + rng.integers(-30, 31, (nq, d)), 0, 255)
    return vb.astype(np.uint8), vq.astype(np.uint8)


def test_restatement_pinned_to_reference():
    """Learn (sampling, k-means), cell assignment, per-cell search and merge in
    the reference's arithmetic: identical lists, slot for slot."""
    R = reference()
    if R is None:
        pytest.skip("reference library not built here (oracle/_ref)")
    bind(R)
    for seed, (vb, vq) in ((1, clustered(1, 3000, 200, 24)), (2, byte_rows(2, 2500, 150, 16))):
        for k, nhash in ((10, 3), (1, 2)):
            srand48(100 + seed)
            got = lib_ann(R, vb, vq, k, nhash)
            srand48(100 + seed)
            exp = orc_ann(vb, vq, k, nhash, 1 if vb.dtype == np.uint8 else 0, ORC_PORT)
            np.testing.assert_array_equal(got[0], exp[0], err_msg=f"seed {seed} k {k}")
            np.testing.assert_array_equal(got[1], exp[1], err_msg=f"seed {seed} k {k}")
            assert (got[0] >= 0).all()


def test_threaded_restatement_pinned_to_reference():
    """Three threads in the reference (its k-means and knn_full_thread calls
    split the work) and in the restatement: the same lists."""
    R = reference()
    if R is None:
        pytest.skip("reference library not built here (oracle/_ref)")
    bind(R)
    vb, vq = clustered(4, 3000, 200, 24)
    srand48(104)
    got = lib_ann(R, vb, vq, 10, 2, nt=3)
    srand48(104)
    exp = orc_ann(vb, vq, 10, 2, 0, ORC_PORT, nt=3)
    np.testing.assert_array_equal(got[0], exp[0])
    np.testing.assert_array_equal(got[1], exp[1])


def test_restatement_small_cells_pinned_to_reference():
    """400 base vectors in 20 cells per partition and k = 30: most cells hold
    fewer than k vectors (k2 = cell size), and the lists keep empty slots
    (-1, 1e30) where the partitions found fewer than k distinct neighbours."""
    R = reference()
    if R is None:
        pytest.skip("reference library not built here (oracle/_ref)")
    bind(R)
    vb, vq = clustered(3, 400, 60, 8, ncl=10)
    for nhash in (1, 3):
        srand48(300 + nhash)
        got = lib_ann(R, vb, vq, 30, nhash)
        srand48(300 + nhash)
        exp = orc_ann(vb, vq, 30, nhash, 0, ORC_PORT)
        np.testing.assert_array_equal(got[0], exp[0])
        np.testing.assert_array_equal(got[1], exp[1])
        assert (got[0] == -1).any() and (got[0] >= 0).any()


def test_nnlist_merge_against_the_reference():
    """Repeated ids, equal distances and values above the current largest, in
    the same sequence: the same lists, slot for slot."""
    R = bind(reference()) if reference() is not None else None
    if R is None:
        pytest.skip("reference library not built here (oracle/_ref)")
    L_ = bind(yg.lib())
    rng = np.random.default_rng(9)
    n, k = 20, 7
    a, b = L_.nnlist_new(n, k), R.nnlist_new(n, k)
    assert (lists(a)[0] == -1).all() and (lists(a)[1] == np.float32(1e30)).all()
    for _ in range(300):
        lno = int(rng.integers(0, n))
        m = int(rng.integers(1, 12))
        ids = rng.integers(0, 40, m).astype(np.int32)
        dis = rng.integers(0, 25, m).astype(np.float32)  # many equal distances
        L_.nnlist_addn(a, lno, m, ptr(ids), ptr(dis))
        R.nnlist_addn(b, lno, m, ptr(ids), ptr(dis))
    for x, y in zip(lists(a), lists(b)):
        np.testing.assert_array_equal(x, y)
    L_.nnlist_delete(a)
    R.nnlist_delete(b)


def test_index_accessors_and_files(tmp_path):
    """kmlsh_write / kmlsh_read and kmlsh_idx_write / kmlsh_idx_read round trips,
    the partition file byte-identical to the reference's, and the cell
    accessors on a hand-made index (no search)."""
    L_ = bind(yg.lib())
    nhash, nclust, d, n = 3, 5, 4, 11
    lp = L_.kmlsh_new(nhash, nclust, d)
    lsh = ctypes.cast(lp, ctypes.POINTER(KmLsh)).contents
    cent = np.arange(nhash * nclust * d, dtype=np.float32).reshape(nhash, -1) * 0.5
    for h in range(nhash):
        ctypes.memmove(lsh.centroids[h], ptr(cent[h]), cent[h].nbytes)
    f1 = str(tmp_path / "a.kmlsh").encode()
    L_.kmlsh_write(f1, lp)
    R = reference()
    if R is not None:
        bind(R)
        f2 = str(tmp_path / "b.kmlsh").encode()
        R.kmlsh_write(f2, lp)
        assert read_bytes(f1) == read_bytes(f2)
    lp2 = L_.kmlsh_new(nhash, nclust, d)
    L_.kmlsh_read(f1, lp2)
    lsh2 = ctypes.cast(lp2, ctypes.POINTER(KmLsh)).contents
    for h in range(nhash):
        got = np.ctypeslib.as_array(lsh2.centroids[h], shape=(nclust * d,))
        np.testing.assert_array_equal(got, cent[h])
    ip = L_.kmlsh_idx_new(lp, n)
    ix = ctypes.cast(ip, ctypes.POINTER(KmLshIdx)).contents
    rng = np.random.default_rng(4)
    perms, bnds = [], []
    for h in range(nhash):
        cells = rng.integers(0, nclust, n)
        perm = np.argsort(cells, kind="stable").astype(np.int32)
        bnd = np.concatenate([[0], np.cumsum(np.bincount(cells, minlength=nclust))]).astype(np.int32)
        ctypes.memmove(ctypes.addressof(ix.perm.contents) + 4 * h * n, ptr(perm), perm.nbytes)
        ctypes.memmove(ctypes.addressof(ix.boundaries.contents) + 4 * h * (nclust + 1), ptr(bnd),
                       bnd.nbytes)
        perms.append(perm)
        bnds.append(bnd)
        for c in range(nclust):
            assert L_.kmlsh_idx_get_nvec(ip, h, c) == bnd[c + 1] - bnd[c]
            got = ctypes.cast(L_.kmlsh_idx_get_vecids(ip, h, c), ctypes.POINTER(I))
            np.testing.assert_array_equal([got[i] for i in range(bnd[c + 1] - bnd[c])],
                                          perm[bnd[c]:bnd[c + 1]])
        assert L_.kmlsh_idx_get_maxincell(ip, h) == np.diff(bnd).max()
    fi = str(tmp_path / "a.kmlshidx").encode()
    L_.kmlsh_idx_write(fi, ip)
    ip2 = L_.kmlsh_idx_new(lp, n)
    L_.kmlsh_idx_read(fi, ip2)
    ix2 = ctypes.cast(ip2, ctypes.POINTER(KmLshIdx)).contents
    np.testing.assert_array_equal(np.ctypeslib.as_array(ix2.perm, shape=(nhash * n,)),
                                  np.concatenate(perms))
    np.testing.assert_array_equal(np.ctypeslib.as_array(ix2.boundaries, shape=(nhash * (nclust + 1),)),
                                  np.concatenate(bnds))
    for x in (ip, ip2):
        L_.kmlsh_idx_delete(x)
    for x in (lp, lp2):
        L_.kmlsh_delete(x)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp32", "bf16"])
@pytest.mark.parametrize("rows", ["bvec", "fvec"])
def test_gpu_kmlsh_ann_matches_oracle(monkeypatch, prec, rows):
    """kmlsh_ann on the GPU (k-means partitions, one k = 1 search per
    partition, one batched search over the occupied cells: the per-cell pool
    with fp32, the grouped pass with bf16 and k = 10) equals the exact
    restatement slot for slot."""
    monkeypatch.setenv("YAEL_GPU_PRECISION", prec)
    vb, vq = byte_rows(5, 4000, 300, 16)
    if rows == "fvec":
        vb, vq = vb.astype(np.float32), vq.astype(np.float32)
    L_ = bind(yg.lib())
    for k, nhash in ((10, 3), (3, 2)):
        srand48(77)
        got = lib_ann(L_, vb, vq, k, nhash)
        srand48(77)
        exp = orc_ann(vb, vq, k, nhash, 1 if rows == "bvec" else 0, ORC_EXACT)
        np.testing.assert_array_equal(got[0], exp[0])
        np.testing.assert_array_equal(got[1], exp[1])
