"""yael_knn, the command-line program of yael's progs/knn.c: options and
formats (CPU), and its results against the FP64 oracle (GPU)."""
import os
import subprocess

import numpy as np
import pytest

from _util import knn_exact, read_bytes, read_text

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "yael_gb300", "bin", "yael_knn")


@pytest.fixture(scope="module")
def cli():
    from yael_gb300 import build
    build.build()
    assert os.path.exists(CLI)
    return CLI


def write_vecs(path, a, dtype):
    with open(path, "wb") as f:
        for row in a:
            f.write(np.int32(row.shape[0]).tobytes() + row.astype(dtype).tobytes())


def read_vecs(path, dtype):
    raw = read_bytes(path)
    out, pos = [], 0
    while pos < len(raw):
        d = int(np.frombuffer(raw, np.int32, 1, pos)[0])
        out.append(np.frombuffer(raw, dtype, d, pos + 4))
        pos += 4 + d * np.dtype(dtype).itemsize
    return np.stack(out)


def test_usage_and_argument_errors(cli):
    r = subprocess.run([cli, "-h"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "-onn idxfile" in r.stdout
    r = subprocess.run([cli, "-k", "5"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "are needed" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", ["fvec", "bvec", "text"])
def test_knn_program_matches_oracle(cli, tmp_path, fmt):
    rng = np.random.default_rng(17)
    nb, nq, d, k = 3000, 40, 32, 10
    if fmt == "bvec":
        b = rng.integers(0, 256, (nb, d)).astype(np.float32)
        q = rng.integers(0, 256, (nq, d)).astype(np.float32)
    else:
        b = rng.standard_normal((nb, d)).astype(np.float32)
        q = rng.standard_normal((nq, d)).astype(np.float32)
    args = [cli, "-k", str(k), "-silence"]
    if fmt == "fvec":
        write_vecs(tmp_path / "b.fvecs", b, np.float32)
        write_vecs(tmp_path / "q.fvecs", q, np.float32)
        args += ["-b", str(tmp_path / "b.fvecs"), "-q", str(tmp_path / "q.fvecs")]
    elif fmt == "bvec":
        write_vecs(tmp_path / "b.bvecs", b, np.uint8)
        write_vecs(tmp_path / "q.bvecs", q, np.uint8)
        args += ["-bb", str(tmp_path / "b.bvecs"), "-qb", str(tmp_path / "q.bvecs")]
    else:
        np.savetxt(tmp_path / "b.txt", b, fmt="%.9g")
        np.savetxt(tmp_path / "q.txt", q, fmt="%.9g")
        args += ["-bt", str(tmp_path / "b.txt"), "-qt", str(tmp_path / "q.txt"), "-nb", str(nb),
                 "-nq", str(nq), "-d", str(d)]
    if fmt == "text":
        args += ["-onnt", str(tmp_path / "nn.txt"), "-odist", str(tmp_path / "dis.txt")]
    else:
        args += ["-onn", str(tmp_path / "nn.ivecs"), "-odis", str(tmp_path / "dis.fvecs")]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    if fmt == "text":
        idx = np.loadtxt(tmp_path / "nn.txt", dtype=np.int64).reshape(nq, k)
        dis = np.loadtxt(tmp_path / "dis.txt").reshape(nq, k)
    else:
        idx = read_vecs(tmp_path / "nn.ivecs", np.int32)
        dis = read_vecs(tmp_path / "dis.fvecs", np.float32)
    ridx, rdis, _ = knn_exact(b, q, k)
    np.testing.assert_array_equal(idx, ridx)
    np.testing.assert_allclose(dis, rdis, rtol=1e-5, atol=1e-4)


KMEANS_CLI = os.path.join(ROOT, "yael_gb300", "bin", "yael_kmeans")


def test_kmeans_usage_and_argument_errors(cli, tmp_path):
    """yael_kmeans (progs/kmeans.c): usage, missing files, text input without
    its sizes, k above the number of vectors -- all before any GPU work."""
    r = subprocess.run([KMEANS_CLI, "-h"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "-otxt clustfile" in r.stdout and "Default: 40" in r.stdout
    r = subprocess.run([KMEANS_CLI, "-k", "5"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "are needed" in r.stderr
    r = subprocess.run([KMEANS_CLI, "-i", str(tmp_path / "none.fvecs"), "-o", "x"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "cannot read" in r.stderr
    r = subprocess.run([KMEANS_CLI, "-itxt", str(tmp_path / "none.txt"), "-o", "x"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "needs -n and -d" in r.stderr
    write_vecs(tmp_path / "few.fvecs", np.ones((5, 4), np.float32), np.float32)
    r = subprocess.run([KMEANS_CLI, "-i", str(tmp_path / "few.fvecs"), "-o", "x", "-k", "10"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "k is larger" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", ["fvec", "text"])
def test_kmeans_program_matches_oracle(cli, tmp_path, fmt):
    """The centroid file equals the exact-mode oracle's k-means of the same
    points, seed and iterations (fvec: bit for bit; text: the same "%f " lines)."""
    import ctypes
    from _util import oracle, ptr
    from yael_gb300 import synth
    v, _, _ = synth.gaussian_mixture(4000, 24, 20, 0.3, seed=13)
    n, d = v.shape
    k, niter, seed = 20, 12, 7
    args = [KMEANS_CLI, "-k", str(k), "-niter", str(niter), "-seed", str(seed), "-nt", "4"]
    if fmt == "fvec":
        write_vecs(tmp_path / "v.fvecs", v, np.float32)
        args += ["-i", str(tmp_path / "v.fvecs"), "-o", str(tmp_path / "c.fvecs")]
    else:
        np.savetxt(tmp_path / "v.txt", v, fmt="%.9g")
        args += ["-itxt", str(tmp_path / "v.txt"), "-n", str(n), "-d", str(d),
                 "-otxt", str(tmp_path / "c.txt")]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    C = np.zeros((k, d), np.float32)
    oracle().orc_kmeans(d, n, k, niter, ptr(v), 4, seed, 1, ptr(C), None, None, None, 1,
                        ctypes.c_void_p())
    if fmt == "fvec":
        np.testing.assert_array_equal(read_vecs(tmp_path / "c.fvecs", np.float32), C)
    else:
        want = "".join("".join(f"{x:f} " for x in row) + "\n" for row in C)
        assert read_text(tmp_path / "c.txt") == want
