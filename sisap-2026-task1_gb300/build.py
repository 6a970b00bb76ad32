"""Build libknng.so (CUDA, sm_103a) and the knng_main CLI in place.

    python sisap-2026-task1_gb300/build.py [--force] [--checked]

Each csrc/*.cu compiles to _build/<name>.o in parallel (one -gencode, sm_103a
only), then nvcc links libknng.so next to this file; host/*.cpp link into
knng_main against it (rpath $ORIGIN), with zlib (deflate-compressed HDF5
input) when the host has its header and library.  Targets are rebuilt only
when a source or header is newer.

--checked builds the bounds-checked library libknng_checked.so instead
(-DKNNG_CHECKS, objects in _build_checked/): every index a kernel derives from
its inputs is checked before it addresses memory and a failed check returns
KNNG_E_BOUNDS.  Load it by setting KNNG_LIBRARY to its path.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys
import tempfile

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libknng.so")
LIB_CHECKED = os.path.join(PKG, "libknng_checked.so")
OUT_CHECKED = os.path.join(PKG, "_build_checked")
CLI = os.path.join(PKG, "knng_main")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-diag-suppress", "550"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _zlib_flags():
    """["-DKNNG_HAVE_ZLIB", "-lz"] when a zlib program compiles and links here."""
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "z.cpp")
        with open(src, "w") as f:
            f.write("#include <zlib.h>\nint main() { return zlibVersion()[0] == 0; }\n")
        r = subprocess.run(["g++", src, "-o", os.path.join(d, "z"), "-lz"], capture_output=True)
    return ["-DKNNG_HAVE_ZLIB", "-lz"] if r.returncode == 0 else []


def _library(out_dir, lib, extra, force, verbose):
    os.makedirs(out_dir, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    jobs = []
    for src in sources:
        obj = os.path.join(out_dir, os.path.basename(src)[:-3] + ".o")
        if force or _newer(obj, [src] + headers):
            jobs.append([nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                print(r.stderr, file=sys.stderr)
    objs = [os.path.join(out_dir, os.path.basename(s)[:-3] + ".o") for s in sources]
    if force or jobs or _newer(lib, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcublas", "-lcusolver"])  # knng_pca


def build_checked(force=False, verbose=False):
    """libknng_checked.so: the same library with the device bounds checks compiled in."""
    _library(OUT_CHECKED, LIB_CHECKED, ["-DKNNG_CHECKS"], force, verbose)
    return LIB_CHECKED


def build(force=False, verbose=False):
    _library(OUT, LIB, [], force, verbose)
    host_srcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    host_hdrs = glob.glob(os.path.join(HOST, "*.h"))
    if host_srcs and (force or _newer(CLI, host_srcs + host_hdrs + [LIB])):
        z = _zlib_flags()
        _run(["g++", "-std=c++20", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include")] + z[:1] +
             host_srcs + ["-o", CLI, "-L", PKG, "-lknng", "-Wl,-rpath,$ORIGIN"] + z[1:])
    return LIB


if __name__ == "__main__":
    if "--checked" in sys.argv:
        print(build_checked(force="--force" in sys.argv, verbose=True))
    else:
        build(force="--force" in sys.argv, verbose=True)
        print(LIB)
