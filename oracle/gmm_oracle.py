"""gmm_oracle.py -- TEST INFRASTRUCTURE ONLY.

An FP64 numpy restatement of yael's Gaussian mixture code (yael/gmm.c), the
checker for the GPU library's gmm_* functions.  Nothing in the product library
imports, loads or calls it.  The formulas are the reference's definitions (its
"simple and slow" forms where it gives one); the reference computes the same
quantities in float32 through expanded sgemm forms, so the comparisons carry a
tolerance (stated in the tests).  The parameters are rounded to float32 after
every EM iteration, as the reference stores them.
"""
import numpy as np

FLAGS_W, FLAGS_NO_NORM, FLAGS_1SIGMA, FLAGS_SIGMA, FLAGS_MU, FLAGS_PURE_KMEANS = 1, 2, 4, 8, 16, 32
NORM_TO_0 = 16.636   # yael/gmm.c:264
MIN_SIGMA = 1e-10    # yael/gmm.c:111
BIGPRIME = 1000003   # yael/gmm.c:376


def mahalanobis(v, mu, sigma):
    """M[i, j] = sum_l (v_il - mu_jl)^2 / sigma_jl (yael/gmm.c:334-341)"""
    v = v.astype(np.float64)
    M = np.empty((v.shape[0], mu.shape[0]))
    for j in range(mu.shape[0]):
        M[:, j] = (((v - mu[j].astype(np.float64)) ** 2) / sigma[j].astype(np.float64)).sum(1)
    return M


def compute_p(v, w, mu, sigma, flags):
    """gmm_compute_p (yael/gmm.c:305-362) with softmax_ref (262-300)"""
    d = v.shape[1]
    logdet = -d / 2.0 * np.log(2 * np.pi) - 0.5 * np.log(sigma.astype(np.float64)).sum(1)
    lg = np.log(w.astype(np.float64)) if flags & FLAGS_W else np.zeros(len(w))
    x = logdet[None, :] - 0.5 * mahalanobis(v, mu, sigma) + lg[None, :]
    mx = x.max(1, keepdims=True)
    e = np.where(x >= mx - NORM_TO_0, np.exp(x - mx), 0.0)
    s = e.sum(1, keepdims=True)
    return np.where(s != 0, e / np.where(s != 0, s, 1), e)


def handle_empty(v, mu, sigma, p):
    """gmm_handle_empty (yael/gmm.c:366-433), in place on p; returns the
    (empty, donor, dimension, moved) splits made"""
    n, k = p.shape
    w = (p > 0).sum(0).astype(np.float64)  # positive exactly when the float sum is
    splits = []
    for j in range(k):
        if w[j] != 0:
            continue
        j2 = j
        while True:
            for _ in range(k):
                j2 = (j2 + BIGPRIME) % k
                if w[j2] > 0:
                    break
            else:
                raise RuntimeError("could not find centroid to split")
            nnz = int((p[:, j2] > 0).sum())
            if nnz >= n // k:
                break
        sd = int(np.argmax(sigma[j2]))  # first maximum
        move = (p[:, j2] > 0) & (v[:, sd] < mu[j2, sd])
        p[move, j] = p[move, j2]
        p[move, j2] = 0
        splits.append((j, j2, sd, int(move.sum())))
        w[j2] = -1
    return splits


def compute_params(v, p, mu_old, flags):
    """gmm_compute_params (yael/gmm.c:114-199): (w, mu, sigma) as float32"""
    v = v.astype(np.float64)
    w = p.sum(0)
    mu = p.T @ v
    sigma = np.empty_like(mu)
    for j in range(p.shape[1]):
        sigma[j] = (p[:, j:j + 1] * (v - mu_old[j].astype(np.float64)) ** 2).sum(0)
    if flags & FLAGS_1SIGMA:
        sigma[:] = sigma.mean(1, keepdims=True)
    sigma = np.where(sigma < MIN_SIGMA, MIN_SIGMA, sigma)
    mu = mu / w[:, None]
    sigma = sigma / w[:, None]
    w = w / np.abs(w).sum()
    return w.astype(np.float32), mu.astype(np.float32), sigma.astype(np.float32)


def learn(v, k, niter, mu0, dis0, flags):
    """gmm_learn (yael/gmm.c:436-502) from the k-means result (mu0, dis0);
    returns (w, mu, sigma, iterations)"""
    n, d = v.shape
    niter = 10000 if niter == 0 else niter
    w = np.full(k, 1.0 / k, np.float32)
    sig = float(np.sum(dis0.astype(np.float64))) / n
    mu = mu0.astype(np.float32).copy()
    sigma = np.full((k, d), sig, np.float32)
    if flags & FLAGS_PURE_KMEANS:
        niter = 0
    key, it = 666.0, 0
    for it in range(1, niter + 1):
        p = compute_p(v, w, mu, sigma, flags)
        handle_empty(v, mu, sigma, p)
        w, mu, sigma = compute_params(v, p, mu, flags)
        old_key, key = key, float(np.sum(mu.astype(np.float64)))
        if key == old_key:
            break
    return w, mu, sigma, it


def fisher_from_posteriors(v, w, mu, sigma, p, flags):
    """gmm_fisher_from_posteriors (yael/gmm.c:527-725)"""
    v = v.astype(np.float64)
    n, d = v.shape
    k = mu.shape[0]
    w64, mu64, sg64 = w.astype(np.float64), mu.astype(np.float64), sigma.astype(np.float64)
    out = []
    if flags & FLAGS_W:
        for j in range(1, k):
            accu = (p[:, j] / w64[j] - p[:, 0] / w64[0]).sum()
            out.append(accu / np.sqrt(n * (1 / w64[j] + 1 / w64[0])))
    if flags & FLAGS_MU:
        dmu = np.empty((k, d))
        for j in range(k):
            dmu[j] = (p[:, j:j + 1] * (v - mu64[j]) / sg64[j]).sum(0)
            if not flags & FLAGS_NO_NORM:
                dmu[j] /= np.sqrt(n * w64[j] / sg64[j])
        out.extend(dmu.ravel())
    if flags & (FLAGS_SIGMA | FLAGS_1SIGMA):
        for j in range(k):
            acc = (p[:, j:j + 1] * (((v - mu64[j]) ** 2) / sg64[j] - 1) / np.sqrt(sg64[j])).sum(0)
            if flags & FLAGS_1SIGMA:
                if flags & FLAGS_SIGMA:
                    f = np.ones(d) if flags & FLAGS_NO_NORM else 2 * n * w64[j] / sg64[j]
                    out.extend(acc / np.sqrt(f))
                f = 1.0 if flags & FLAGS_NO_NORM else 2 * d * n * w64[j] / sg64[j, 0]
                out.append(acc.sum() / np.sqrt(f))
            else:
                f = np.ones(d) if flags & FLAGS_NO_NORM else 2 * n * w64[j] / sg64[j]
                out.extend(acc / np.sqrt(f))
    return np.array(out)


def fisher_sizeof(d, k, flags):
    """gmm_fisher_sizeof (yael/gmm.c:505-512)"""
    return ((k - 1 if flags & FLAGS_W else 0) + (d * k if flags & FLAGS_MU else 0) +
            (k if flags & FLAGS_1SIGMA else 0) + (d * k if flags & FLAGS_SIGMA else 0))


def fisher_spatial(Q, sgmm, ll):
    """gmm_fisher_spatial (yael/gmm.c:728-791): Q (N x K), sgmm (2 x D),
    ll (D x N) -> (D x K mean terms, D x K variance terms), flattened"""
    Q = Q.astype(np.float64)
    N = Q.shape[0]
    D = ll.shape[0]
    llv = ll.astype(np.float64).T           # N x D
    qs = Q.sum(0) / N                        # K
    qll = Q.T @ llv / N                      # K x D
    qll2 = Q.T @ (llv ** 2) / N
    mm = sgmm[:D].astype(np.float64)
    S = sgmm[D:].astype(np.float64)
    d_mm = qll - qs[:, None] * mm[None, :]
    d_S = -qll2 + 2 * qll * mm[None, :] + qs[:, None] * (S - mm ** 2)[None, :]
    return np.concatenate([d_mm.ravel(), d_S.ravel()])
