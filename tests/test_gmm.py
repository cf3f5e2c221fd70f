"""Gaussian mixtures and Fisher vectors (yael/gmm.c).  An FP64 restatement
(oracle/gmm_oracle.py) is pinned to the reference library compiled here (CPU);
the GPU library must agree with it (GPU).  The reference evaluates float32
expanded sgemm forms and the GPU direct forms with FP64 moments, so both are
compared with the FP64 restatement under the tolerances written below."""
import ctypes
import sys

import numpy as np
import pytest

import yael_gb300 as yg
from _util import ORACLE_DIR, oracle, read_bytes, reference
from yael_gb300 import synth

sys.path.insert(0, ORACLE_DIR)
import gmm_oracle as go  # noqa: E402

P = ctypes.c_void_p
libc = ctypes.CDLL(None)
libc.fopen.restype = P
libc.fopen.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
libc.fclose.argtypes = [P]
ORC_PORT, ORC_EXACT = 0, 1

# tolerances against the FP64 restatement
P_ATOL = 1e-5        # posteriors (in [0, 1]); about 1e-6 observed
FV_RTOL, FV_ATOL = 2e-4, 2e-4   # Fisher vectors, relative to their largest entry (1e-4 observed)
LEARN_RTOL = 2e-4    # parameters after EM, relative to each array's largest entry (4e-5 observed)


class Gmm(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int), ("k", ctypes.c_int), ("w", ctypes.POINTER(ctypes.c_float)),
                ("mu", ctypes.POINTER(ctypes.c_float)), ("sigma", ctypes.POINTER(ctypes.c_float))]


def ptr(a):
    return a.ctypes.data_as(P)


def bind(lib):
    for name, (res, args) in yg.SIGNATURES.items():
        if name.startswith("gmm_") and hasattr(lib, name):
            getattr(lib, name).restype = res
            getattr(lib, name).argtypes = args
    return lib


def ref_lib():
    r = reference()
    if r is None or not hasattr(r, "gmm_learn"):
        pytest.skip("reference library with gmm.c not built here (oracle/_ref)")
    return bind(r)


def make_gmm(w, mu, sigma):
    k, d = mu.shape
    keep = [np.ascontiguousarray(a, np.float32) for a in (w, mu, sigma)]
    g = Gmm(d, k, *(a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) for a in keep))
    return g, keep


def read_gmm(gp):
    g = ctypes.cast(gp, ctypes.POINTER(Gmm)).contents
    k, d = g.k, g.d
    w = np.ctypeslib.as_array(g.w, shape=(k,)).copy()
    mu = np.ctypeslib.as_array(g.mu, shape=(k * d,)).reshape(k, d).copy()
    sg = np.ctypeslib.as_array(g.sigma, shape=(k * d,)).reshape(k, d).copy()
    return w, mu, sg


def mixture(seed, n=3000, d=12, k=6):
    """Overlapping components at d = 12 (about half the vectors have
    fractional posteriors); mostly one-hot posteriors in higher dimensions."""
    v, lab, C = synth.gaussian_mixture(n, d, k, 0.8, seed=seed)
    rng = np.random.default_rng(seed + 1)
    w = rng.uniform(0.5, 1.5, k).astype(np.float32)
    w /= w.sum()
    mu = (C + 0.05 * rng.standard_normal(C.shape)).astype(np.float32)
    sigma = rng.uniform(0.5, 1.0, (k, d)).astype(np.float32)
    return v, w, mu, sigma


FLAG_SETS = [go.FLAGS_MU, go.FLAGS_W | go.FLAGS_MU | go.FLAGS_SIGMA,
             go.FLAGS_MU | go.FLAGS_NO_NORM, go.FLAGS_SIGMA, go.FLAGS_SIGMA | go.FLAGS_NO_NORM,
             go.FLAGS_1SIGMA, go.FLAGS_1SIGMA | go.FLAGS_SIGMA | go.FLAGS_W,
             go.FLAGS_1SIGMA | go.FLAGS_SIGMA | go.FLAGS_NO_NORM]


def close(got, exp, rtol, atol):
    scale = max(1.0, float(np.abs(exp).max()))
    np.testing.assert_allclose(got, exp, rtol=rtol, atol=atol * scale)


def run_p(lib, v, g, flags):
    p = np.empty((v.shape[0], g.k), np.float32)
    lib.gmm_compute_p(v.shape[0], ptr(v), ctypes.byref(g), ptr(p), flags)
    return p


def run_fisher(lib, v, g, flags, p=None):
    out = np.full(go.fisher_sizeof(g.d, g.k, flags), np.nan, np.float32)
    assert lib.gmm_fisher_sizeof(ctypes.byref(g), flags) == out.size
    if p is None:
        lib.gmm_fisher(v.shape[0], ptr(v), ctypes.byref(g), flags, ptr(out))
    else:
        lib.gmm_fisher_from_posteriors(v.shape[0], ptr(v), ctypes.byref(g), flags, ptr(p),
                                       ptr(out))
    return out


def spatial_case(seed, N=2000, K=7, D=3):
    rng = np.random.default_rng(seed)
    Q = rng.dirichlet(np.ones(K), N).astype(np.float32)       # N x K
    ll = rng.uniform(0, 1, (D, N)).astype(np.float32)          # D x N
    sgmm = np.concatenate([rng.uniform(0.3, 0.7, D), rng.uniform(0.05, 0.1, D)]).astype(np.float32)
    return Q, sgmm, ll


def run_spatial(lib, Q, sgmm, ll):
    N, K = Q.shape
    D = ll.shape[0]
    out = np.full(2 * K * D, np.nan, np.float32)
    lib.gmm_fisher_spatial(N, K, D, ptr(Q), ptr(sgmm), ptr(ll), ptr(out))
    return out


def seeded_kmeans(v, k, niter, seed, mode):
    """the oracle's kmeans in the given mode: the reference's own arithmetic
    (ORC_PORT) or the GPU library's (ORC_EXACT)"""
    n, d = v.shape
    C = np.zeros((k, d), np.float32)
    dis = np.empty(n, np.float32)
    assign = np.empty(n, np.int32)
    nassign = np.empty(k, np.int32)
    oracle().orc_kmeans(d, n, k, niter, ptr(v), 1, seed, 1, ptr(C), ptr(dis), ptr(assign),
                        ptr(nassign), mode, None)
    return C, dis


def run_learn(lib, v, k, niter, seed, flags):
    n, d = v.shape
    gp = lib.gmm_learn(d, n, k, niter, ptr(v), 1, seed, 1, flags)
    out = read_gmm(gp)
    lib.gmm_delete(gp)
    return out


def check_learn(got, exp):
    for a, b in zip(got, exp[:3]):
        close(a, b, LEARN_RTOL, LEARN_RTOL)


# ---------------------------------------------------------------- CPU pins

def test_posteriors_and_fisher_restatement_pinned_to_reference():
    R = ref_lib()
    v, w, mu, sigma = mixture(3)
    g, keep = make_gmm(w, mu, sigma)
    for flags in (0, go.FLAGS_W):
        np.testing.assert_allclose(run_p(R, v, g, flags), go.compute_p(v, w, mu, sigma, flags),
                                   rtol=0, atol=P_ATOL)
    p = go.compute_p(v, w, mu, sigma, go.FLAGS_W)
    for flags in FLAG_SETS:
        close(run_fisher(R, v, g, flags), go.fisher_from_posteriors(v, w, mu, sigma, p, flags),
              FV_RTOL, FV_ATOL)
        pf = p.astype(np.float32)
        close(run_fisher(R, v, g, flags, pf),
              go.fisher_from_posteriors(v, w, mu, sigma, pf.astype(np.float64), flags),
              FV_RTOL, FV_ATOL)


def test_spatial_restatement_pinned_to_reference():
    R = ref_lib()
    Q, sgmm, ll = spatial_case(4)
    close(run_spatial(R, Q, sgmm, ll), go.fisher_spatial(Q, sgmm, ll), FV_RTOL, FV_ATOL)


@pytest.mark.parametrize("flags", [go.FLAGS_W, go.FLAGS_W | go.FLAGS_1SIGMA, 0,
                                   go.FLAGS_W | go.FLAGS_PURE_KMEANS])
def test_learn_restatement_pinned_to_reference(flags):
    """k-means seeding in the reference's arithmetic (identical centroids and
    distances), then EM: the reference's float32 parameters against the FP64
    restatement's."""
    R = ref_lib()
    v, _, _ = synth.gaussian_mixture(3000, 10, 6, 0.9, seed=11)
    k, niter, seed = 6, 8, 5
    got = run_learn(R, v, k, niter, seed, flags)
    mu0, dis0 = seeded_kmeans(v, k, niter, seed, ORC_PORT)
    check_learn(got, go.learn(v, k, niter, mu0, dis0, flags))


def test_files(tmp_path):
    """gmm_write / gmm_read round-trip and write the reference's bytes."""
    L_ = bind(yg.lib())
    v, w, mu, sigma = mixture(6, n=500, d=5, k=4)
    g, keep = make_gmm(w, mu, sigma)
    f1 = str(tmp_path / "a.gmm").encode()
    fh = libc.fopen(f1, b"w")
    L_.gmm_write(ctypes.byref(g), fh)
    libc.fclose(fh)
    raw = read_bytes(f1)
    assert raw == (np.array([5, 4], np.int32).tobytes() + w.tobytes() + mu.tobytes() +
                   sigma.tobytes())
    fh = libc.fopen(f1, b"r")
    gp = L_.gmm_read(fh)
    libc.fclose(fh)
    for a, b in zip(read_gmm(gp), (w, mu, sigma)):
        np.testing.assert_array_equal(a, b)
    L_.gmm_delete(gp)
    R = reference()
    if R is not None and hasattr(R, "gmm_write"):
        bind(R)
        f2 = str(tmp_path / "b.gmm").encode()
        fh = libc.fopen(f2, b"w")
        R.gmm_write(ctypes.byref(g), fh)
        libc.fclose(fh)
        assert read_bytes(f2) == raw


# ---------------------------------------------------------------- GPU

@pytest.mark.gpu
def test_gpu_posteriors():
    L_ = bind(yg.lib())
    for seed, (n, d, k) in ((3, (3000, 12, 6)), (8, (1037, 70, 45))):
        v, w, mu, sigma = mixture(seed, n, d, k)
        g, keep = make_gmm(w, mu, sigma)
        for flags in (0, go.FLAGS_W):
            np.testing.assert_allclose(run_p(L_, v, g, flags),
                                       go.compute_p(v, w, mu, sigma, flags), rtol=0, atol=P_ATOL)
        pt = np.empty((n, k), np.float32)
        L_.gmm_compute_p_thread(n, ptr(v), ctypes.byref(g), ptr(pt), go.FLAGS_W, 4)
        np.testing.assert_array_equal(pt, run_p(L_, v, g, go.FLAGS_W))


@pytest.mark.gpu
def test_gpu_fisher_vectors():
    L_ = bind(yg.lib())
    v, w, mu, sigma = mixture(3, 3000, 12, 6)
    g, keep = make_gmm(w, mu, sigma)
    p = go.compute_p(v, w, mu, sigma, go.FLAGS_W)
    pf = p.astype(np.float32)
    for flags in FLAG_SETS:
        close(run_fisher(L_, v, g, flags), go.fisher_from_posteriors(v, w, mu, sigma, p, flags),
              FV_RTOL, FV_ATOL)
        close(run_fisher(L_, v, g, flags, pf),
              go.fisher_from_posteriors(v, w, mu, sigma, pf.astype(np.float64), flags),
              FV_RTOL, FV_ATOL)
    Q, sgmm, ll = spatial_case(4)
    close(run_spatial(L_, Q, sgmm, ll), go.fisher_spatial(Q, sgmm, ll), FV_RTOL, FV_ATOL)
    Q, sgmm, ll = spatial_case(5, N=777, K=40, D=2)
    close(run_spatial(L_, Q, sgmm, ll), go.fisher_spatial(Q, sgmm, ll), FV_RTOL, FV_ATOL)


@pytest.mark.gpu
@pytest.mark.parametrize("flags", [go.FLAGS_W, go.FLAGS_W | go.FLAGS_1SIGMA, 0,
                                   go.FLAGS_W | go.FLAGS_PURE_KMEANS])
def test_gpu_learn(flags):
    """The drop-in kmeans seeds exactly as the oracle's exact mode, then EM on
    the GPU against the FP64 restatement."""
    L_ = bind(yg.lib())
    v, _, _ = synth.gaussian_mixture(3000, 10, 6, 0.9, seed=11)
    k, niter, seed = 6, 8, 5
    got = run_learn(L_, v, k, niter, seed, flags)
    mu0, dis0 = seeded_kmeans(v, k, niter, seed, ORC_EXACT)
    check_learn(got, go.learn(v, k, niter, mu0, dis0, flags))


def test_numpy_front_end_plumbing(monkeypatch, tmp_path):
    """ynumpy's gmm_learn / gmm_read / fisher (yael/ynumpy.py:268-353): the
    module's wrappers, run over the reference library (same C ABI), return
    what direct calls into it return -- the argument and result handling
    checked without a GPU.  The GPU library behind them is checked above."""
    R = ref_lib()
    v, _, _ = synth.gaussian_mixture(1500, 6, 4, 0.9, seed=12)
    n, d = v.shape
    srand48_ = ctypes.CDLL(None).srand48
    srand48_(5)
    exp = run_learn(R, v, 4, 5, 3, go.FLAGS_W)
    monkeypatch.setattr(yg, "_lib", R)
    srand48_(5)
    got = yg.gmm_learn(v, 4, nt=1, niter=5, seed=3, use_weights=True)
    for a, b in zip(got, exp):
        np.testing.assert_array_equal(a, b)
    g, keep = make_gmm(*exp)
    for include, flags in (("mu", go.FLAGS_MU), ("mu sigma w", go.FLAGS_MU | go.FLAGS_SIGMA |
                                                   go.FLAGS_W), ("sigma", go.FLAGS_SIGMA)):
        np.testing.assert_array_equal(yg.fisher(exp, v, include=include),
                                      run_fisher(R, v, g, flags))
    fn = str(tmp_path / "g.gmm").encode()
    fh = libc.fopen(fn, b"w")
    R.gmm_write(ctypes.byref(g), fh)
    libc.fclose(fh)
    for a, b in zip(yg.gmm_read(fn.decode()), exp):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("nt", [1, 3])
def test_port_restatement_bit_identical_to_reference(nt):
    """The oracle's restatement in the reference's own arithmetic (expanded
    sgemm forms, float roundings, slice order for nt > 1) equals the reference
    library bit for bit: posteriors and learned mixtures.  It is the timed CPU
    baseline of the mixture workload."""
    R = ref_lib()
    o = oracle()
    o.orc_gmm_compute_p.argtypes = [ctypes.c_int, P, ctypes.c_int, ctypes.c_int, P, P, P, P,
                                    ctypes.c_int, ctypes.c_int]
    o.orc_gmm_learn.argtypes = [ctypes.c_int] * 4 + [P] + [ctypes.c_int] * 4 + [P, P, P, P]
    v, w, mu, sigma = mixture(3)
    n, d = v.shape
    k = mu.shape[0]
    g, keep = make_gmm(w, mu, sigma)
    for flags in (0, go.FLAGS_W):
        exp = np.empty((n, k), np.float32)
        R.gmm_compute_p_thread(n, ptr(v), ctypes.byref(g), ptr(exp), flags, nt)
        got = np.empty((n, k), np.float32)
        o.orc_gmm_compute_p(n, ptr(v), d, k, ptr(w), ptr(mu), ptr(sigma), ptr(got), flags, nt)
        np.testing.assert_array_equal(got, exp)
    v, _, _ = synth.gaussian_mixture(3000, 10, 6, 0.9, seed=11)
    n, d = v.shape
    for flags in (go.FLAGS_W, go.FLAGS_W | go.FLAGS_1SIGMA):
        gp = R.gmm_learn(d, n, 6, 8, ptr(v), nt, 5, 1, flags)
        exp = read_gmm(gp)
        R.gmm_delete(gp)
        gw, gm, gs = np.empty(6, np.float32), np.empty((6, d), np.float32), np.empty((6, d), np.float32)
        it = ctypes.c_int(0)
        assert o.orc_gmm_learn(d, n, 6, 8, ptr(v), nt, 5, 1, flags, ptr(gw), ptr(gm), ptr(gs),
                               ctypes.byref(it)) == 0
        for a, b in zip((gw, gm, gs), exp):
            np.testing.assert_array_equal(a, b)
