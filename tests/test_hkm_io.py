"""hkm_write / hkm_read of the C ABI (host code only, no GPU): the binary
format of yael/hkm.c:181-232 -- int nlevel, bf, d, then one fvec record
(int count, count floats) per level."""
import ctypes
import struct

import numpy as np

import yael_gb300 as yg
from _util import read_bytes, reference


def test_hkm_file_roundtrip(tmp_path):
    from yael_gb300 import build
    build.build()
    L = yg.lib()
    nlevel, bf, d = 2, 3, 4
    path = str(tmp_path / "t.hkm")
    rng = np.random.default_rng(0)
    lv = [rng.standard_normal(bf ** (l + 1) * d).astype(np.float32) for l in range(nlevel)]
    with open(path, "wb") as f:
        f.write(struct.pack("iii", nlevel, bf, d))
        for a in lv:
            f.write(struct.pack("i", a.size))
            f.write(a.tobytes())
    h = L.hkm_read(path.encode())
    assert h
    hk = yg.Hkm.from_address(h)
    assert (hk.nlevel, hk.bf, hk.d, hk.k) == (nlevel, bf, d, bf ** nlevel)
    for l in range(nlevel):
        got = np.ctypeslib.as_array(hk.centroids[l], shape=(lv[l].size,))
        np.testing.assert_array_equal(got, lv[l])
    c = L.hkm_get_centroids(h, 1, 2)
    np.testing.assert_array_equal(
        np.ctypeslib.as_array(ctypes.cast(c, ctypes.POINTER(ctypes.c_float)), shape=(bf * d,)),
        lv[1][2 * bf * d:3 * bf * d])
    out = str(tmp_path / "u.hkm")
    L.hkm_write(out.encode(), h)
    assert read_bytes(out) == read_bytes(path)
    L.hkm_delete(h)
    assert not L.hkm_read(str(tmp_path / "missing.hkm").encode())


def test_hkm_files_against_the_reference(tmp_path):
    """The reference library reads what this one writes and writes the same
    bytes back; get_centroids agrees."""
    R = reference()
    if R is None:
        import pytest
        pytest.skip("reference library not built here (oracle/_ref)")
    for name in ("hkm_read", "hkm_write", "hkm_delete", "hkm_get_centroids"):
        res, args = yg.SIGNATURES[name]
        getattr(R, name).restype = res
        getattr(R, name).argtypes = args
    L = yg.lib()
    nlevel, bf, d = 3, 2, 5
    rng = np.random.default_rng(1)
    path = str(tmp_path / "a.hkm")
    with open(path, "wb") as f:
        f.write(struct.pack("iii", nlevel, bf, d))
        for l in range(nlevel):
            a = rng.standard_normal(bf ** (l + 1) * d).astype(np.float32)
            f.write(struct.pack("i", a.size) + a.tobytes())
    ours, theirs = L.hkm_read(path.encode()), R.hkm_read(path.encode())
    o1, o2 = str(tmp_path / "o.hkm"), str(tmp_path / "r.hkm")
    L.hkm_write(o1.encode(), theirs)
    R.hkm_write(o2.encode(), ours)
    assert read_bytes(o1) == read_bytes(o2) == read_bytes(path)
    for l in range(nlevel):
        for node in range(bf ** l):
            a = ctypes.string_at(L.hkm_get_centroids(ours, l, node), 4 * bf * d)
            b = ctypes.string_at(R.hkm_get_centroids(theirs, l, node), 4 * bf * d)
            assert a == b
    L.hkm_delete(ours)
    R.hkm_delete(theirs)
