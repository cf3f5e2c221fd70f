"""Vector file I/O (.fvecs / .ivecs / .bvecs): the record format, round trips,
edge cases, and -- where the reference library compiled from its own sources
is present -- byte-identical files and identical reads against it.  Host code
only: no GPU."""
import ctypes
import os

import numpy as np
import pytest

import yael_gb300 as yg
from _util import read_bytes, read_text, reference, write_text

P = ctypes.c_void_p
I = ctypes.c_int
L = ctypes.c_long
libc = ctypes.CDLL(None)
libc.fopen.restype = P
libc.fopen.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
libc.fclose.argtypes = [P]
libc.free.argtypes = [P]
libc.fflush.argtypes = [P]


def ptr(a):
    return a.ctypes.data_as(P)


def records(path, dtype):
    """numpy restatement of the record format: int32 d, then d elements."""
    raw = read_bytes(path)
    out, pos, item = [], 0, np.dtype(dtype).itemsize
    while pos < len(raw):
        d = int(np.frombuffer(raw, np.int32, 1, pos)[0])
        out.append(np.frombuffer(raw, dtype, d, pos + 4))
        pos += 4 + d * item
    return out


def ref_lib():
    r = reference()
    if r is None:
        return None
    for name, (res, args) in yg.SIGNATURES.items():
        if name.endswith(("vec_fwrite", "vecs_fwrite", "vecs_write", "vecs_fsize", "vecs_new_read",
                          "vecs_new_fread_max", "vecs_read", "vec_fread", "vecs_fread", "_raw",
                          "_txt")) \
                and hasattr(r, name):
            getattr(r, name).restype = res
            getattr(r, name).argtypes = args
    return r


@pytest.fixture(scope="module")
def data():
    rng = np.random.default_rng(3)
    f = rng.standard_normal((37, 24)).astype(np.float32)
    i = rng.integers(-1000, 1000, (37, 24)).astype(np.int32)
    b = rng.integers(0, 256, (37, 24)).astype(np.uint8)
    return f, i, b


def test_writers_follow_the_record_format(tmp_path, data):
    f, i, b = data
    L_ = yg.lib()
    for name, arr, dt, w in (("a.fvecs", f, np.float32, L_.fvecs_write),
                             ("a.ivecs", i, np.int32, L_.ivecs_write),
                             ("a.bvecs", b, np.uint8, L_.bvecs_write)):
        path = str(tmp_path / name)
        assert w(path.encode(), arr.shape[1], arr.shape[0], ptr(arr)) == arr.shape[0]
        recs = records(path, dt)
        assert len(recs) == arr.shape[0]
        np.testing.assert_array_equal(np.stack(recs), arr)


def test_readers_round_trip(tmp_path, data):
    f, i, b = data
    L_ = yg.lib()
    fp, ip, bp = (str(tmp_path / n).encode() for n in ("r.fvecs", "r.ivecs", "r.bvecs"))
    L_.fvecs_write(fp, 24, 37, ptr(f))
    L_.ivecs_write(ip, 24, 37, ptr(i))
    L_.bvecs_write(bp, 24, 37, ptr(b))
    d, n = I(), I()
    assert L_.fvecs_fsize(fp, ctypes.byref(d), ctypes.byref(n)) == 37 * (4 + 24 * 4)
    assert (d.value, n.value) == (24, 37)
    assert L_.bvecs_fsize(bp, ctypes.byref(d), ctypes.byref(n)) == 37 * (4 + 24)
    for fn, dt, arr, path in ((L_.fvecs_new_read, np.float32, f, fp),
                              (L_.ivecs_new_read, np.int32, i, ip),
                              (L_.bvecs_new_read, np.uint8, b, bp),
                              (L_.b2fvecs_new_read, np.float32, b.astype(np.float32), bp)):
        out = P()
        cnt = fn(path, ctypes.byref(d), ctypes.byref(out))
        assert (cnt, d.value) == (37, 24)
        got = np.ctypeslib.as_array(ctypes.cast(out, ctypes.POINTER(np.ctypeslib.as_ctypes_type(dt))),
                                    shape=(37 * 24,)).reshape(37, 24).copy()
        libc.free(out)
        np.testing.assert_array_equal(got, arr)
    # the first n records; asking for more than the file holds reads what is there
    buf = np.zeros((40, 24), np.float32)
    assert L_.fvecs_read(fp, 24, 10, ptr(buf)) == 10
    np.testing.assert_array_equal(buf[:10], f[:10])
    assert L_.fvecs_read(fp, 24, 40, ptr(buf)) == 37
    assert L_.fvecs_read(fp, 23, 5, ptr(buf)) == -1  # wrong dimension
    assert L_.b2fvecs_read(bp, 24, 5, ptr(buf)) == 5
    np.testing.assert_array_equal(buf[:5], b[:5].astype(np.float32))
    # streams: at most nmax records, then one record at a time
    fh = libc.fopen(fp, b"r")
    out = P()
    assert L_.fvecs_new_fread_max(fh, ctypes.byref(d), ctypes.byref(out), 5) == 5
    got = np.ctypeslib.as_array(ctypes.cast(out, ctypes.POINTER(ctypes.c_float)), shape=(5 * 24,))
    np.testing.assert_array_equal(got.reshape(5, 24), f[:5])
    libc.free(out)
    row = np.zeros(24, np.float32)
    assert L_.fvec_fread(fh, ptr(row), 24) == 24
    np.testing.assert_array_equal(row, f[5])
    rest = np.zeros((40, 24), np.float32)
    assert L_.fvecs_fread(fh, ptr(rest), 40, 24) == 31
    np.testing.assert_array_equal(rest[:31], f[6:])
    assert L_.fvec_fread(fh, ptr(row), 24) == 0  # end of file
    libc.fclose(fh)


def test_edge_cases(tmp_path):
    L_ = yg.lib()
    d, n, out = I(), I(), P()
    empty = str(tmp_path / "e.fvecs").encode()
    open(empty, "wb").close()
    assert L_.fvecs_fsize(empty, ctypes.byref(d), ctypes.byref(n)) == 0 and n.value == 0
    assert L_.fvecs_new_read(empty, ctypes.byref(d), ctypes.byref(out)) == 0
    assert d.value == -1
    missing = str(tmp_path / "none.fvecs").encode()
    assert L_.fvecs_new_read(missing, ctypes.byref(d), ctypes.byref(out)) == -1
    assert L_.fvecs_fsize(missing, ctypes.byref(d), ctypes.byref(n)) == -1
    # records of different dimensions
    mixed = str(tmp_path / "m.fvecs").encode()
    with open(mixed, "wb") as fh:
        fh.write(np.int32(3).tobytes() + np.ones(3, np.float32).tobytes())
        fh.write(np.int32(2).tobytes() + np.ones(2, np.float32).tobytes())
    assert L_.fvecs_new_read(mixed, ctypes.byref(d), ctypes.byref(out)) == -1
    assert L_.fvecs_fsize(mixed, ctypes.byref(d), ctypes.byref(n)) == -1  # 20 bytes, records of 16
    # truncated last record
    trunc = str(tmp_path / "t.fvecs").encode()
    with open(trunc, "wb") as fh:
        fh.write(np.int32(4).tobytes() + np.ones(4, np.float32).tobytes())
        fh.write(np.int32(4).tobytes() + np.ones(2, np.float32).tobytes())
    assert L_.fvecs_new_read(trunc, ctypes.byref(d), ctypes.byref(out)) == -1
    # zero vectors written
    z = str(tmp_path / "z.ivecs").encode()
    assert L_.ivecs_write(z, 5, 0, None) == 0 and os.path.getsize(z) == 0


def test_against_the_reference(tmp_path, data):
    """Same bytes written and same values read as the reference library."""
    R = ref_lib()
    if R is None:
        pytest.skip("reference library not built here (oracle/_ref)")
    f, i, b = data
    L_ = yg.lib()
    for ext, arr, ours, theirs in (("fvecs", f, L_.fvecs_write, R.fvecs_write),
                                   ("ivecs", i, L_.ivecs_write, R.ivecs_write),
                                   ("bvecs", b, L_.bvecs_write, R.bvecs_write)):
        p1, p2 = (str(tmp_path / f"{w}.{ext}").encode() for w in ("ours", "ref"))
        assert ours(p1, 24, 37, ptr(arr)) == theirs(p2, 24, 37, ptr(arr)) == 37
        assert read_bytes(p1) == read_bytes(p2)
    d1, d2, o1, o2 = I(), I(), P(), P()
    for name in ("fvecs_new_read", "ivecs_new_read", "bvecs_new_read", "b2fvecs_new_read"):
        ext = "bvecs" if name.startswith(("bvecs", "b2f")) else name[:5]
        path = str(tmp_path / f"ref.{ext}").encode()
        n1 = getattr(L_, name)(path, ctypes.byref(d1), ctypes.byref(o1))
        n2 = getattr(R, name)(path, ctypes.byref(d2), ctypes.byref(o2))
        assert (n1, d1.value) == (n2, d2.value) == (37, 24)
        nbytes = 37 * 24 * (1 if name == "bvecs_new_read" else 4)
        assert ctypes.string_at(o1, nbytes) == ctypes.string_at(o2, nbytes)
        libc.free(o1)
        libc.free(o2)
    path = str(tmp_path / "ref.fvecs").encode()
    for nread in (5, 37, 50):
        a1, a2 = np.zeros((50, 24), np.float32), np.zeros((50, 24), np.float32)
        assert L_.fvecs_read(path, 24, nread, ptr(a1)) == R.fvecs_read(path, 24, nread, ptr(a2))
        np.testing.assert_array_equal(a1, a2)
    s1, s2 = (I(), I()), (I(), I())
    assert L_.fvecs_fsize(path, *map(ctypes.byref, s1)) == R.fvecs_fsize(path, *map(ctypes.byref, s2))
    assert [x.value for x in s1] == [x.value for x in s2]


def as_array(p, n, dtype):
    return np.ctypeslib.as_array(
        ctypes.cast(p, ctypes.POINTER(np.ctypeslib.as_ctypes_type(dtype))), shape=(n,)).copy()


def test_raw_and_text(tmp_path, data):
    """Headerless files hold exactly the elements; text files one line per
    vector with a space after each element; both read back."""
    f, i, b = data
    L_ = yg.lib()
    for name, arr, w, rd, nf in (("r.f", f, L_.fvec_write_raw, L_.fvec_new_read_raw, L_.fvec_fread_raw),
                                 ("r.i", i, L_.ivec_write_raw, L_.ivec_new_read_raw, L_.ivec_fread_raw),
                                 ("r.b", b, L_.bvec_write_raw, L_.bvec_new_read_raw, L_.bvec_fread_raw)):
        path = str(tmp_path / name).encode()
        assert w(path, ptr(arr), arr.size) == 0
        assert read_bytes(path) == arr.tobytes()
        out = rd(path, arr.size)
        np.testing.assert_array_equal(as_array(out, arr.size, arr.dtype), arr.ravel())
        libc.free(out)
        assert rd(path, arr.size + 1) is None          # short file
        fh = libc.fopen(path, b"r")
        half = np.zeros(arr.size // 2, arr.dtype)
        assert nf(fh, ptr(half), half.size) == half.size
        np.testing.assert_array_equal(half, arr.ravel()[:half.size])
        rest = np.zeros(arr.size, arr.dtype)
        assert nf(fh, ptr(rest), rest.size) == -1      # past the end
        libc.fclose(fh)
    assert L_.fvec_new_read_raw(str(tmp_path / "none").encode(), 4) is None
    ft, it = str(tmp_path / "f.txt").encode(), str(tmp_path / "i.txt").encode()
    assert L_.fvecs_write_txt(ft, 24, 37, ptr(f)) == 37
    assert L_.ivecs_write_txt(it, 24, 37, ptr(i)) == 37
    lines = read_text(it).split("\n")
    assert lines[-1] == "" and len(lines) == 38
    assert lines[0] == "".join(f"{x} " for x in i[0])
    assert read_text(ft).split("\n")[1] == "".join(f"{x:f} " for x in f[1])
    got = np.zeros((40, 24), np.float32)
    assert L_.fvecs_read_txt(ft, 24, 40, ptr(got)) == 37  # fewer vectors than asked
    np.testing.assert_array_equal(got[:37], np.array([[float(f"{x:f}") for x in r] for r in f],
                                                     np.float32))
    assert L_.fvecs_read_txt(ft, 24, 3, ptr(got)) == 3
    bad = str(tmp_path / "bad.txt").encode()
    write_text(bad, "1 2 x 4\n")
    assert L_.fvecs_read_txt(bad, 2, 2, ptr(got)) == -1


def test_raw_and_text_against_the_reference(tmp_path, data):
    """Same bytes written and same values read as the reference library (its
    success paths only: on a short raw read it frees the caller's buffer)."""
    R = ref_lib()
    if R is None:
        pytest.skip("reference library not built here (oracle/_ref)")
    f, i, b = data
    L_ = yg.lib()
    for ext, arr, fn in (("f", f, "fvec"), ("i", i, "ivec"), ("b", b, "bvec")):
        p1, p2 = (str(tmp_path / f"{w}.raw{ext}").encode() for w in ("ours", "ref"))
        assert getattr(L_, fn + "_write_raw")(p1, ptr(arr), arr.size) == 0
        assert getattr(R, fn + "_write_raw")(p2, ptr(arr), arr.size) == 0
        assert read_bytes(p1) == read_bytes(p2)
        o1 = getattr(L_, fn + "_new_read_raw")(p2, arr.size - 5)
        o2 = getattr(R, fn + "_new_read_raw")(p2, arr.size - 5)
        nbytes = (arr.size - 5) * arr.itemsize
        assert ctypes.string_at(o1, nbytes) == ctypes.string_at(o2, nbytes)
        libc.free(o1)
        libc.free(o2)
    for fn, arr in (("fvecs_write_txt", f), ("ivecs_write_txt", i)):
        p1, p2 = (str(tmp_path / f"{w}.{fn}").encode() for w in ("ours", "ref"))
        assert getattr(L_, fn)(p1, 24, 37, ptr(arr)) == getattr(R, fn)(p2, 24, 37, ptr(arr)) == 37
        libc.fflush(None)  # the reference leaves its text file open
        assert read_bytes(p1) == read_bytes(p2)
    path = str(tmp_path / "ours.fvecs_write_txt").encode()
    for nread in (5, 37, 50):
        a1, a2 = np.zeros((50, 24), np.float32), np.zeros((50, 24), np.float32)
        assert L_.fvecs_read_txt(path, 24, nread, ptr(a1)) == R.fvecs_read_txt(path, 24, nread,
                                                                              ptr(a2))
        np.testing.assert_array_equal(a1, a2)


def test_numpy_front_end(tmp_path, data):
    """The ynumpy file helpers (yael/ynumpy.py:158-226) over the library's
    readers and writers: round trips, nmax, appends to an open file, errors."""
    f, i, b = data
    fp, ip, bp = (str(tmp_path / n) for n in ("a.fvecs", "a.ivecs", "a.bvecs"))
    yg.fvecs_write(fp, f)
    yg.ivecs_write(ip, i)
    yg.bvecs_write(bp, b)
    assert yg.fvecs_fsize(fp) == (37, 24)
    np.testing.assert_array_equal(yg.fvecs_read(fp), f)
    np.testing.assert_array_equal(yg.fvecs_read(fp, nmax=5), f[:5])
    np.testing.assert_array_equal(yg.fvecs_read(fp, nmax=100), f)
    np.testing.assert_array_equal(yg.ivecs_read(ip), i)
    np.testing.assert_array_equal(np.stack(records(bp, np.uint8)), b)
    with open(str(tmp_path / "app.fvecs"), "wb") as fh:
        fh.write(np.int32(24).tobytes() + f[0].tobytes())
        yg.fvecs_fwrite(fh, f[1:4])
        yg.fvecs_fwrite(fh, f[4:6])
    np.testing.assert_array_equal(yg.fvecs_read(str(tmp_path / "app.fvecs")), f[:6])
    empty = str(tmp_path / "e.fvecs")
    open(empty, "wb").close()
    assert yg.fvecs_read(empty).shape == (0, 0)
    assert yg.fvecs_read(empty, nmax=3).shape == (0, 0)
    with pytest.raises(IOError):
        yg.fvecs_read(str(tmp_path / "none.fvecs"), nmax=3)
    with pytest.raises(IOError):
        yg.ivecs_read(str(tmp_path / "none.ivecs"))
    with pytest.raises(IOError):
        yg.fvecs_fsize(str(tmp_path / "none.fvecs"))
