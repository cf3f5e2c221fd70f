"""Compile the CUDA sources into the in-tree C-ABI library libyael_gb300.so.

sm_103a only (``-gencode arch=compute_103a,code=sm_103a``), translation units
compiled in parallel, relinked only when a source or header changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OBJDIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libyael_gb300.so")
# the command-line programs of yael's progs/knn.c and progs/kmeans.c, linked
# against the library
CLIS = [(os.path.join(HERE, "cli", name + ".cpp"), os.path.join(HERE, "bin", name))
        for name in ("yael_knn", "yael_kmeans")]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-ffp-contract=off",
              "-Xcompiler", "-fvisibility=default", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libyael_gb300")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Build (if needed) and return the path of libyael_gb300.so."""
    nvcc = _nvcc()
    os.makedirs(OBJDIR, exist_ok=True)
    hdrs = _headers()
    srcs = sources()
    objs = [os.path.join(OBJDIR, os.path.basename(s)[:-3] + ".o") for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if _stale(o, [s] + hdrs)]

    def compile_one(so):
        s, o = so
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", s, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(s)}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(f"[yael_gb300] compiled {os.path.basename(s)}", file=sys.stderr)

    if todo:
        n = jobs or min(len(todo), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            list(ex.map(compile_one, todo))
    if todo or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs,
               "-Xlinker", "-Bsymbolic", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
        if verbose:
            print(f"[yael_gb300] linked {LIB}", file=sys.stderr)
    for cli_src, cli in CLIS:
        if not _stale(cli, [cli_src, LIB] + hdrs):
            continue
        os.makedirs(os.path.dirname(cli), exist_ok=True)
        cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
        cmd = [cxx, "-O2", "-std=c++17", "-o", cli + ".tmp", cli_src, "-L" + HERE, "-lyael_gb300",
               "-Wl,-rpath,$ORIGIN/.."]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"building {os.path.basename(cli)} failed:\n{r.stdout}\n{r.stderr}")
        os.replace(cli + ".tmp", cli)
        if verbose:
            print(f"[yael_gb300] built {cli}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
