"""The GPU library's host-side k-means draws (yael_gb300/csrc/km_host.h)
against the oracle's restatements, on the host (no GPU):
* the random initialisation's first k of a partial Fisher-Yates shuffle
  (an open-addressing table instead of an n-entry permutation) against
  orc_random_init;
* the empty-cluster split (planned from the counts and the seed, then applied
  to the touched rows only) against the oracle's kmeans_reassign_empty
  (yael/kmeans.c:166-209) on the whole centroid array: the same rows, bit for
  bit, and the same number of splits."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from _util import oracle, ptr

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("kmhost") / "libkmhostshim.so")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-o", out,
                    os.path.join(HERE, "km_host_shim.cpp")], check=True)
    lib = ctypes.CDLL(out)
    lib.shim_split.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 4
    lib.shim_split.restype = ctypes.c_int
    lib.shim_random_init.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.c_void_p]
    lib.shim_random_init.restype = None
    return lib


@pytest.mark.parametrize("n,k,seed", [(1, 1, 5), (10, 10, 7), (1000, 3, 11), (5000, 4999, 3),
                                      (2_000_000, 32, 12345), (10_000_000, 65536, 99),
                                      (65537, 65536, 2**31 - 1)])
def test_random_init_matches_oracle(shim, n, k, seed):
    got = np.empty(k, np.int64)
    shim.shim_random_init(n, k, seed, ptr(got))
    want = np.empty(k, np.int32)
    oracle().orc_random_init(n, k, seed, ptr(want))
    np.testing.assert_array_equal(got, want)
    assert len(np.unique(got)) == k


def counts(rng, k, kind):
    if kind == "mixed":  # a few empty clusters among clusters of all sizes
        c = rng.integers(2, 3000, k)
        c[rng.random(k) < 0.08] = 0
        c[rng.random(k) < 0.05] = 1
    elif kind == "many_empty":
        c = rng.integers(0, 4, k) * rng.integers(1, 50, k)
    elif kind == "wrap":  # squares past 2^31: negative probabilities, as in the reference
        c = rng.integers(0, 100, k)
        h = min(3, k - 1)
        c[rng.choice(k, h, replace=False)] = rng.integers(46341, 200000, h)
        c[rng.choice(k, 1)] = 0
    elif kind == "no_splittable":  # every count 0 or 1: zero total, NaN probabilities
        c = rng.integers(0, 2, k)
        c[0] = 0
    else:  # "none": no empty cluster
        c = rng.integers(1, 100, k)
    return c.astype(np.int32)


@pytest.mark.parametrize("kind", ["mixed", "many_empty", "wrap", "no_splittable", "none"])
@pytest.mark.parametrize("d,k,ni", [(16, 300, 1), (96, 32, 7), (5, 2, 3), (128, 4096, 1)])
def test_split_host_matches_oracle(shim, kind, d, k, ni):
    rng = np.random.default_rng(d * 1000 + k + ni)
    C = rng.standard_normal((ni, k, d)).astype(np.float32)
    cnt = np.stack([counts(rng, k, kind) for _ in range(ni)])
    seeds = rng.integers(0, 2**31, ni).astype(np.uint32)
    Co = C.copy()
    nre_o = [oracle().orc_reassign_empty(d, k, ptr(Co[i]), ptr(cnt[i]), int(seeds[i]))
             for i in range(ni)]
    Cg = C.copy()
    nre_g = np.zeros(ni, np.int32)
    tot = shim.shim_split(d, k, ni, ptr(Cg), ptr(cnt), ptr(seeds), ptr(nre_g))
    assert list(nre_g) == nre_o and tot == sum(nre_o)
    np.testing.assert_array_equal(Cg.view(np.uint32), Co.view(np.uint32))
    if kind != "none":
        assert (Cg != C).any()
