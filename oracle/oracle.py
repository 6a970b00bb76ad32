"""ctypes front end of the oracle (test infrastructure only).

Loads oracle/_build/liboracle.so (the CPU restatement of the reference,
knng_oracle.cpp) and, where it was built, runs oracle/_ref/main (the unmodified
reference src/main.cpp compiled against h5shim/H5Cpp.h).  Only tests/, the
smoke check and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "sisap-2026-task1_gb300"))
import h5container  # noqa: E402

TIE_REF, TIE_STABLE = 0, 1
QUANT_TRUNC, QUANT_ROUND = 0, 1


class Params(C.Structure):
    _fields_ = [
        ("k_build", C.c_int), ("k_eval", C.c_int), ("num_trees", C.c_int),
        ("rerank_mult", C.c_int), ("leaf_size", C.c_int), ("max_iterations", C.c_int),
        ("early_stop_rate", C.c_float), ("rate_diff_tol", C.c_float),
        ("quant_mode", C.c_int), ("tie_mode", C.c_int), ("jacobi", C.c_int),
        ("threads", C.c_int), ("seed", C.c_uint32), ("sketch_mode", C.c_int),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("quantize_s", C.c_double), ("forest_s", C.c_double), ("init_s", C.c_double),
        ("join_s", C.c_double), ("build_s", C.c_double), ("iterations", C.c_int),
        ("updates", C.c_int64 * 64),
    ]


_lib = None


def build():
    """Compile liboracle.so (and oracle/_ref when the reference sources exist).

    Where the reference sources are is the Makefile's REF variable (settable
    from the environment); `make have-ref` succeeds only when they are there."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    have = subprocess.run(["make", "-s", "-C", HERE, "have-ref"], capture_output=True)
    if have.returncode == 0:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        L.oracle_default_params.argtypes = [P(Params)]
        L.oracle_quantize.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        L.oracle_forest.argtypes = [C.c_void_p, C.c_int64, C.c_int, P(Params), C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_int64, P(C.c_int64)]
        L.oracle_init.argtypes = [C.c_void_p, C.c_int64, C.c_int, P(Params), C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p]
        L.oracle_init_random.argtypes = [C.c_void_p, C.c_int64, C.c_int, P(Params), C.c_void_p, C.c_void_p]
        L.oracle_init_block.argtypes = [C.c_void_p, C.c_int64, C.c_int, P(Params), C.c_int, C.c_int, C.c_void_p,
                                        C.c_void_p]
        L.oracle_join_iter.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int64, C.c_int, P(Params),
                                       C.c_void_p, C.c_void_p]
        L.oracle_join_iter.restype = C.c_int64
        L.oracle_hyperplane_sketch.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_uint32, C.c_void_p]
        L.oracle_plane_value.argtypes = [C.c_uint32, C.c_int, C.c_int]
        L.oracle_plane_value.restype = C.c_int8
        L.oracle_export.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        L.oracle_build.argtypes = [C.c_void_p, C.c_int64, C.c_int, P(Params), C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, P(Stats)]
        _lib = L
    return _lib


def params(**kw) -> Params:
    p = Params()
    lib().oracle_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def quantize(x, quant_mode=QUANT_TRUNC):
    x = np.ascontiguousarray(x, dtype=np.float32)
    n, d = x.shape
    words = (d + 63) // 64
    codes = np.empty((n, d), np.int8)
    sk = np.empty((n, words), np.uint64)
    lib().oracle_quantize(_ptr(x), n, d, quant_mode, _ptr(codes), _ptr(sk), words)
    return codes, sk


def hyperplane_sketch(codes, seed=1337):
    """128-bit sketches from 128 seeded integer hyperplanes: (n, 2) uint64."""
    codes = np.ascontiguousarray(codes)
    n, d = codes.shape
    sk = np.empty((n, 2), np.uint64)
    lib().oracle_hyperplane_sketch(_ptr(codes), n, d, seed, _ptr(sk))
    return sk


def plane_value(seed, k, j):
    return int(lib().oracle_plane_value(seed, k, j))


def forest(codes, prm=None, log_pivots=False):
    """Return (perm[T, n], leaf_flag[T, n], pivots[(m, 6)] or None)."""
    prm = prm or params()
    codes = np.ascontiguousarray(codes)
    n, d = codes.shape
    perm = np.empty((prm.num_trees, n), np.int32)
    lf = np.empty((prm.num_trees, n), np.uint8)
    nn = C.c_int64(0)
    cap = 0
    piv = None
    if log_pivots:
        cap = prm.num_trees * max(1, (2 * n) // max(1, prm.leaf_size // 2)) + 64
        piv = np.zeros((cap, 6), np.int32)
    rc = lib().oracle_forest(_ptr(codes), n, d, C.byref(prm), _ptr(perm), _ptr(lf),
                             _ptr(piv) if piv is not None else None, cap, C.byref(nn))
    if rc:
        raise ValueError("oracle_forest failed")
    if piv is not None:
        if nn.value > cap:
            raise RuntimeError("pivot log overflow")
        piv = piv[: nn.value]
    return perm, lf, piv


def init_graph(codes, perm, leaf_flag, prm=None):
    prm = prm or params()
    n, d = codes.shape
    ids = np.empty((n, prm.k_build), np.int32)
    sc = np.empty((n, prm.k_build), np.int32)
    rc = lib().oracle_init(_ptr(np.ascontiguousarray(codes)), n, d, C.byref(prm),
                           _ptr(np.ascontiguousarray(perm)), _ptr(np.ascontiguousarray(leaf_flag)),
                           _ptr(ids), _ptr(sc))
    if rc:
        raise ValueError("oracle_init failed")
    return ids, sc


def init_random(codes, prm=None):
    """Random initial graph (archive/nndescent_optimized.cpp:97-118, xorshift32 per row)."""
    prm = prm or params()
    n, d = codes.shape
    ids = np.empty((n, prm.k_build), np.int32)
    sc = np.empty((n, prm.k_build), np.int32)
    if lib().oracle_init_random(_ptr(np.ascontiguousarray(codes)), n, d, C.byref(prm), _ptr(ids), _ptr(sc)):
        raise ValueError("oracle_init_random failed")
    return ids, sc


def init_block(codes, prm=None, block_size=10000, bridges=2):
    """Block-partitioned hybrid init (archive/nndescent_hybrid.cpp:98-144, reproducible draws)."""
    prm = prm or params()
    n, d = codes.shape
    ids = np.empty((n, prm.k_build), np.int32)
    sc = np.empty((n, prm.k_build), np.int32)
    if lib().oracle_init_block(_ptr(np.ascontiguousarray(codes)), n, d, C.byref(prm), block_size, bridges,
                               _ptr(ids), _ptr(sc)):
        raise ValueError("oracle_init_block failed (every block needs k_build + 1 rows)")
    return ids, sc


def join_iter(codes, sketch, ids, scores, prm=None):
    """One NN-Descent iteration; updates ids/scores in place, returns the count."""
    prm = prm or params()
    n, d = codes.shape
    return lib().oracle_join_iter(_ptr(codes), _ptr(sketch), sketch.shape[1], n, d, C.byref(prm),
                                  _ptr(ids), _ptr(scores))


def export(ids, scores, k_eval=15):
    n, K = ids.shape
    knns = np.empty((n, k_eval), np.int32)
    dists = np.empty((n, k_eval), np.float32)
    lib().oracle_export(_ptr(ids), _ptr(scores), n, K, k_eval, _ptr(knns), _ptr(dists))
    return knns, dists


def build_graph(x, prm=None, want_graph=False):
    """Full pipeline; returns (knns, dists, stats[, ids, scores])."""
    prm = prm or params()
    x = np.ascontiguousarray(x, dtype=np.float32)
    n, d = x.shape
    knns = np.empty((n, prm.k_eval), np.int32)
    dists = np.empty((n, prm.k_eval), np.float32)
    ids = np.empty((n, prm.k_build), np.int32) if want_graph else None
    sc = np.empty((n, prm.k_build), np.int32) if want_graph else None
    st = Stats()
    rc = lib().oracle_build(_ptr(x), n, d, C.byref(prm), _ptr(knns), _ptr(dists),
                            _ptr(ids) if want_graph else None, _ptr(sc) if want_graph else None,
                            C.byref(st))
    if rc:
        raise ValueError("oracle_build failed")
    return (knns, dists, st, ids, sc) if want_graph else (knns, dists, st)


def ref_binary(d=1024):
    path = os.path.join(REF_DIR, "main" if d == 1024 else f"main_d{d}")
    return path if os.path.exists(path) else None


def run_reference(x, threads=1, task="task1", d=None, workdir=None):
    """Run the reference binary on x; returns (knns, dists, attrs, stdout)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    binpath = ref_binary(d or x.shape[1])
    if binpath is None:
        raise FileNotFoundError("oracle/_ref was not built (reference sources absent)")
    with tempfile.TemporaryDirectory(dir=workdir) as tmp:
        inp = os.path.join(tmp, "data.h5")
        h5container.write(inp, {"train": x})
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        r = subprocess.run([binpath, "--task", task, "--dataset", inp], cwd=tmp, env=env,
                           capture_output=True, text=True, check=True)
        ds, attrs = h5container.read(os.path.join(tmp, "results", task, "apex_simd.h5"), mmap=False)
        return np.array(ds["knns"]), np.array(ds["dists"]), attrs, r.stdout
