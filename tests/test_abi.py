"""The C-ABI library builds for sm_103a, loads, and exports every symbol that
include/yael_gpu.h declares.  No GPU needed (nothing is computed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "yael_gpu.h")


def declared_functions():
    with open(HEADER) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    src = re.sub(r"typedef\s+struct\s*\{.*?\}\s*\w+\s*;", "", src, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def built():
    from yael_gb300 import build
    return build.build()


def test_header_parses():
    names = declared_functions()
    assert "knn_full" in names and "yael_gpu_knn_ex" in names and "kmeans" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built, mode=ctypes.RTLD_LOCAL)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_version_and_error_string(built):
    lib = ctypes.CDLL(built, mode=ctypes.RTLD_LOCAL)
    lib.yael_gpu_version.restype = ctypes.c_int
    lib.yael_gpu_last_error.restype = ctypes.c_char_p
    assert lib.yael_gpu_version() == 1
    assert lib.yael_gpu_last_error() == b""


def test_python_signatures_cover_header(built):
    import yael_gb300
    assert set(declared_functions()) <= set(yael_gb300.SIGNATURES), \
        sorted(set(declared_functions()) - set(yael_gb300.SIGNATURES))
