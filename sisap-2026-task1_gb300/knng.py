"""Python front end of libknng.so (ctypes), the GB300 kNN-graph builder.

Mirrors the reference engine's one operation -- build the all-points k-NN
graph of /train and export knns/dists (Aftab5550/SISAP-2026-task1
src/main.cpp:143-457) -- plus the per-stage entry points the parity tests
drive.  Every call goes through the C ABI declared in include/knng.h; there
is no CPU fallback: if libknng.so is missing or no GPU is visible the calls
raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
# KNNG_LIBRARY selects another build of the library, e.g. the bounds-checked
# libknng_checked.so (build.py --checked)
LIB_PATH = os.environ.get("KNNG_LIBRARY") or os.path.join(PKG, "libknng.so")

QUANT_TRUNC, QUANT_ROUND = 0, 1
JOIN_JACOBI, JOIN_INPLACE = 0, 1
ORDER_NATURAL, ORDER_LEAF = 0, 1
GRAM_DP4A, GRAM_TCGEN05 = 0, 1
INIT_FOREST, INIT_RANDOM, INIT_BLOCK = 0, 1, 2
SKETCH_SIGN, SKETCH_HYPERPLANE = 0, 1

STATUS = {0: "ok", -1: "E_ARGS", -2: "E_DIM", -3: "E_OOM", -4: "E_ADMIT", -5: "E_TIMEOUT", -6: "E_CUDA",
          -7: "E_REPLAY", -8: "E_BUSY", -9: "E_NOTFOUND", -10: "E_SCRATCH", -11: "E_BOUNDS"}


class KnngError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {msg}")


class Params(C.Structure):
    _fields_ = [
        ("k_build", C.c_int), ("k_eval", C.c_int), ("num_trees", C.c_int), ("rerank_mult", C.c_int),
        ("leaf_size", C.c_int), ("max_iterations", C.c_int), ("early_stop_rate", C.c_float),
        ("rate_diff_tol", C.c_float), ("quant_mode", C.c_int), ("join_mode", C.c_int),
        ("row_order", C.c_int), ("seed", C.c_uint32), ("device", C.c_int), ("autotune", C.c_int),
        ("use_graph", C.c_int), ("gram_mode", C.c_int), ("init_mode", C.c_int), ("join_cache", C.c_int),
        ("block_size", C.c_int), ("bridges", C.c_int), ("wait_limit", C.c_int), ("join_ctas_per_sm", C.c_int),
        ("join_cblock", C.c_int), ("sketch_mode", C.c_int), ("forest_fuse", C.c_int),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("quantize_s", C.c_double), ("forest_s", C.c_double), ("init_s", C.c_double), ("join_s", C.c_double),
        ("export_s", C.c_double), ("build_s", C.c_double), ("total_s", C.c_double), ("iterations", C.c_int),
        ("updates", C.c_int64 * 64), ("forest_levels", C.c_int64), ("leaves", C.c_int64),
        ("device_s", C.c_double), ("join_ms", C.c_double * 64), ("join_candidates", C.c_int64 * 64),
        ("join_dots", C.c_int64 * 64), ("kernel_launches", C.c_int64), ("join_ctas_per_sm", C.c_int),
        ("join_cblock", C.c_int), ("graph_used", C.c_int), ("join_distinct", C.c_int64 * 64),
        ("join_skipped", C.c_int64 * 64),
    ]

    def as_dict(self):
        arrays = ("updates", "join_ms", "join_candidates", "join_dots", "join_distinct", "join_skipped")
        d = {f: getattr(self, f) for f, _ in self._fields_ if f not in arrays}
        for f in arrays:
            d[f] = list(getattr(self, f)[: self.iterations])
        return d


EXPORTS = ["knng_default_params", "knng_create", "knng_destroy", "knng_build", "knng_build_batch", "knng_status_string",
           "knng_last_error", "knng_quantize", "knng_forest", "knng_init_graph", "knng_join_iter", "knng_export",
           "knng_init_graph_noalloc", "knng_footprint_bytes", "knng_trim", "knng_server_default_params",
           "knng_server_create", "knng_submit", "knng_poll", "knng_wait", "knng_release", "knng_server_destroy",
           "knng_pca", "knng_sketch_hyperplane"]

_lib = None


def lib():
    """Load libknng.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{os.path.basename(LIB_PATH)} not found at {LIB_PATH}: run __graft_entry__.build() "
                               "first")
        L = C.CDLL(LIB_PATH)
        P, V, I64 = C.POINTER, C.c_void_p, C.c_int64
        L.knng_default_params.argtypes = [P(Params)]
        L.knng_default_params.restype = None
        L.knng_create.argtypes = [P(V), P(Params)]
        L.knng_destroy.argtypes = [V]
        L.knng_destroy.restype = None
        L.knng_build.argtypes = [V, V, I64, C.c_int, C.c_int, V, V, C.c_int, P(Stats)]
        L.knng_build_batch.argtypes = [V, P(Job), C.c_int, P(Stats)]
        L.knng_status_string.argtypes = [C.c_int]
        L.knng_status_string.restype = C.c_char_p
        L.knng_last_error.argtypes = [V]
        L.knng_last_error.restype = C.c_char_p
        L.knng_quantize.argtypes = [V, I64, C.c_int, C.c_int, V, V, V]
        L.knng_sketch_hyperplane.argtypes = [V, I64, C.c_int, C.c_uint32, V, V]
        L.knng_forest.argtypes = [V, V, I64, C.c_int, V, I64, V, V]
        L.knng_init_graph.argtypes = [V, V, I64, C.c_int, V, V, V, V]
        L.knng_join_iter.argtypes = [V, V, V, I64, C.c_int, V, V, V, V, P(I64)]
        L.knng_export.argtypes = [V, V, I64, C.c_int, C.c_int, V, V, V, V]
        L.knng_pca.argtypes = [V, I64, C.c_int, C.c_int, C.c_int, V, C.POINTER(C.c_double)]
        L.knng_init_graph_noalloc.argtypes = [V, I64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint32, V, V, V, V, V]
        L.knng_footprint_bytes.argtypes = [P(Params), I64, C.c_int, C.c_int]
        L.knng_footprint_bytes.restype = I64
        L.knng_trim.argtypes = [V]
        L.knng_server_default_params.argtypes = [P(ServerParams)]
        L.knng_server_default_params.restype = None
        L.knng_server_create.argtypes = [P(V), P(ServerParams)]
        L.knng_submit.argtypes = [V, P(Job), P(C.c_uint64)]
        L.knng_poll.argtypes = [V, C.c_uint64, P(Result)]
        L.knng_wait.argtypes = [V, C.c_uint64, C.c_double, P(Result)]
        L.knng_release.argtypes = [V, C.c_uint64]
        L.knng_server_destroy.argtypes = [V]
        L.knng_server_destroy.restype = None
        _lib = L
    return _lib


def params(**kw) -> Params:
    p = Params()
    lib().knng_default_params(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


def _ptr(t):
    """Device or host pointer of a torch tensor / numpy array (None passes through)."""
    if t is None:
        return None
    if isinstance(t, np.ndarray):
        return t.ctypes.data_as(C.c_void_p)
    return C.c_void_p(t.data_ptr())


def _ready(*tensors):
    """The library works on its own non-blocking stream, which does not wait for
    torch's streams: finish pending torch work on the tensors' device first."""
    for t in tensors:
        if t is not None and not isinstance(t, np.ndarray) and t.is_cuda:
            import torch

            torch.cuda.synchronize(t.device)
            return


def _stream_ptr(stream):
    if stream is None:
        return None
    return C.c_void_p(stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))


class Job(C.Structure):
    _fields_ = [
        ("rows", C.c_void_p), ("n", C.c_int64), ("d", C.c_int), ("rows_on_device", C.c_int),
        ("knns", C.c_void_p), ("dists", C.c_void_p), ("out_on_device", C.c_int), ("status", C.c_int),
        ("iterations", C.c_int),
    ]


class ServerParams(C.Structure):
    _fields_ = [("build", Params), ("slots", C.c_int), ("mem_budget_gb", C.c_double), ("max_batch_jobs", C.c_int)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("batch_jobs", C.c_int), ("queued_s", C.c_double),
                ("run_s", C.c_double), ("latency_s", C.c_double)]


class Server:
    """The serving loop: submit builds as they arrive, wait on tickets."""

    def __init__(self, slots=3, mem_budget_gb=180.0, max_batch_jobs=64, **build_kw):
        sp = ServerParams()
        lib().knng_server_default_params(C.byref(sp))
        sp.build = params(**build_kw)
        sp.slots, sp.mem_budget_gb, sp.max_batch_jobs = slots, mem_budget_gb, max_batch_jobs
        self.k_eval = sp.build.k_eval
        self.h = C.c_void_p()
        st = lib().knng_server_create(C.byref(self.h), C.byref(sp))
        if st != 0:
            raise KnngError(st, "knng_server_create")
        self.live = {}

    def submit(self, rows):
        """Queue a build of rows (numpy or torch CUDA float32); returns a ticket."""
        n, d = rows.shape
        if isinstance(rows, np.ndarray):
            rows = np.ascontiguousarray(rows, dtype=np.float32)
            knns, dists, dev = np.empty((n, self.k_eval), np.int32), np.empty((n, self.k_eval), np.float32), 0
        else:
            import torch

            _ready(rows)
            dev = int(rows.is_cuda)
            knns = torch.empty((n, self.k_eval), dtype=torch.int32, device=rows.device)
            dists = torch.empty((n, self.k_eval), dtype=torch.float32, device=rows.device)
        job = Job(_ptr(rows), n, d, dev, _ptr(knns), _ptr(dists), dev, 0, 0)
        t = C.c_uint64(0)
        st = lib().knng_submit(self.h, C.byref(job), C.byref(t))
        if st != 0:
            raise KnngError(st, "knng_submit")
        self.live[t.value] = (rows, knns, dists)
        return t.value

    def poll(self, ticket):
        r = Result()
        st = lib().knng_poll(self.h, ticket, C.byref(r))
        return None if st == -8 else self._finish(ticket, st, r)

    def wait(self, ticket, timeout_s=600.0):
        r = Result()
        st = lib().knng_wait(self.h, ticket, timeout_s, C.byref(r))
        return self._finish(ticket, st, r)

    def _finish(self, ticket, st, r):
        if st != 0:
            raise KnngError(st, "knng_wait/poll")
        _, knns, dists = self.live.pop(ticket)
        lib().knng_release(self.h, ticket)
        return knns, dists, r

    def close(self):
        if self.h:
            lib().knng_server_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Context:
    """A knng_ctx: device arena + CUDA stream on one GPU."""

    def __init__(self, prm: Params | None = None, **kw):
        self.prm = prm if prm is not None else params(**kw)
        self.h = C.c_void_p()
        self._check(lib().knng_create(C.byref(self.h), C.byref(self.prm)))

    def _check(self, st):
        if st != 0:
            msg = lib().knng_last_error(self.h).decode() if self.h else ""
            raise KnngError(st, msg)

    def close(self):
        if self.h:
            lib().knng_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- whole build (src/main.cpp:179-457) --
    def build(self, rows, knns=None, dists=None, stats: Stats | None = None):
        """Build the graph of ``rows`` (numpy host array or torch tensor, (n, d) float32).

        Outputs follow ``rows``: numpy in, numpy out; torch CUDA in, torch CUDA out.
        Returns (knns, dists, stats).
        """
        st = stats or Stats()
        n, d = rows.shape
        k_eval = self.prm.k_eval
        on_dev = not isinstance(rows, np.ndarray) and rows.is_cuda
        if isinstance(rows, np.ndarray):
            rows = np.ascontiguousarray(rows, dtype=np.float32)
            knns = np.empty((n, k_eval), np.int32) if knns is None else knns
            dists = np.empty((n, k_eval), np.float32) if dists is None else dists
            out_dev = 0
        else:
            import torch

            assert rows.dtype == torch.float32 and rows.is_contiguous()
            out_dev = int(on_dev)
            if knns is None:
                knns = torch.empty((n, k_eval), dtype=torch.int32, device=rows.device if on_dev else "cpu")
                dists = torch.empty((n, k_eval), dtype=torch.float32, device=knns.device)
            out_dev = int(knns.is_cuda)
        _ready(rows, knns)
        self._check(lib().knng_build(self.h, _ptr(rows), n, d, int(on_dev), _ptr(knns), _ptr(dists), out_dev,
                                     C.byref(st)))
        return knns, dists, st

    def build_batch(self, rows_list, stats: Stats | None = None):
        """Batched build of independent datasets (numpy or torch CUDA, any n and d).

        Returns [(knns, dists, iterations), ...] in input order; outputs follow
        each input's kind (numpy in -> numpy out, CUDA tensor in -> CUDA tensors)."""
        st = stats or Stats()
        jobs = (Job * len(rows_list))()
        outs = []
        keep = []
        k_eval = self.prm.k_eval
        for b, rows in enumerate(rows_list):
            n, d = rows.shape
            if isinstance(rows, np.ndarray):
                rows = np.ascontiguousarray(rows, dtype=np.float32)
                knns = np.empty((n, k_eval), np.int32)
                dists = np.empty((n, k_eval), np.float32)
                on_dev = 0
            else:
                import torch

                on_dev = int(rows.is_cuda)
                knns = torch.empty((n, k_eval), dtype=torch.int32, device=rows.device)
                dists = torch.empty((n, k_eval), dtype=torch.float32, device=rows.device)
            keep.append(rows)
            jobs[b] = Job(_ptr(rows), n, d, on_dev, _ptr(knns), _ptr(dists), on_dev, 0, 0)
            outs.append((knns, dists))
        _ready(*[r for r in keep if not isinstance(r, np.ndarray)])
        self._check(lib().knng_build_batch(self.h, jobs, len(rows_list), C.byref(st)))
        return [(k, dd, jobs[b].iterations) for b, (k, dd) in enumerate(outs)], st

    # -- stages (torch CUDA tensors) --
    def forest(self, codes, replay=None, perm=None, leaf_flag=None):
        import torch

        n, d = codes.shape
        T = self.prm.num_trees
        perm = torch.empty((T, n), dtype=torch.int32, device=codes.device) if perm is None else perm
        leaf_flag = torch.empty((T, n), dtype=torch.uint8, device=codes.device) if leaf_flag is None else leaf_flag
        rep = None if replay is None else np.ascontiguousarray(replay, dtype=np.int32)
        _ready(codes)
        self._check(lib().knng_forest(self.h, _ptr(codes), n, d, _ptr(rep), 0 if rep is None else len(rep),
                                      _ptr(perm), _ptr(leaf_flag)))
        return perm, leaf_flag

    def init_graph(self, codes, perm, leaf_flag):
        import torch

        n, d = codes.shape
        K = self.prm.k_build
        ids = torch.empty((n, K), dtype=torch.int32, device=codes.device)
        sc = torch.empty((n, K), dtype=torch.int32, device=codes.device)
        _ready(codes)
        self._check(lib().knng_init_graph(self.h, _ptr(codes), n, d, _ptr(perm), _ptr(leaf_flag), _ptr(ids),
                                          _ptr(sc)))
        return ids, sc

    def join_iter(self, codes, sketch, ids_in, sc_in, ids_out=None, sc_out=None):
        """One NN-Descent iteration; returns (ids_out, sc_out, updates).  Pass the
        input tensors as outputs to update in place."""
        import torch

        n, d = codes.shape
        ids_out = torch.empty_like(ids_in) if ids_out is None else ids_out
        sc_out = torch.empty_like(sc_in) if sc_out is None else sc_out
        up = C.c_int64(0)
        _ready(codes)
        self._check(lib().knng_join_iter(self.h, _ptr(codes), _ptr(sketch), n, d, _ptr(ids_in), _ptr(sc_in),
                                         _ptr(ids_out), _ptr(sc_out), C.byref(up)))
        return ids_out, sc_out, up.value


def quantize(x, quant_mode=QUANT_TRUNC, stream=None):
    """K1 on a CUDA float32 tensor: returns (codes int8 (n, d), sketch int64 (n, d/64))."""
    import torch

    n, d = x.shape
    codes = torch.empty((n, d), dtype=torch.int8, device=x.device)
    sk = torch.empty((n, d // 64), dtype=torch.int64, device=x.device)
    if stream is not None:
        _ready(x)
    st = lib().knng_quantize(_ptr(x), n, d, quant_mode, _ptr(codes), _ptr(sk), _stream_ptr(stream))
    if st != 0:
        raise KnngError(st, "knng_quantize")
    torch.cuda.synchronize(x.device)
    return codes, sk


def sketch_hyperplane(codes, seed=1337, stream=None):
    """Optional 128-bit hyperplane sketches of int8 codes (CUDA tensor (n, d)):
    returns int64 (n, 2) holding the two 64-bit words of each row."""
    import torch

    n, d = codes.shape
    sk = torch.empty((n, 2), dtype=torch.int64, device=codes.device)
    _ready(codes)
    st = lib().knng_sketch_hyperplane(_ptr(codes), n, d, seed, _ptr(sk), _stream_ptr(stream))
    if st != 0:
        raise KnngError(st, "knng_sketch_hyperplane")
    torch.cuda.synchronize(codes.device)
    return sk


def pca(x, dims, device=0):
    """PCA preprocessing (scripts/data_prep/apply_pca.py:25-33) on the GPU:
    returns (float16 (n, dims) L2-normalised projections as numpy, variance kept)."""
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float32)) if not hasattr(x, "data_ptr") else x
    n, d = x.shape
    out = np.empty((n, dims), np.float16)
    kept = C.c_double(0.0)
    if hasattr(x, "data_ptr"):
        _ready(x)
    st = lib().knng_pca(_ptr(x), n, d, dims, device, out.ctypes.data_as(C.c_void_p), C.byref(kept))
    if st != 0:
        raise KnngError(st, "knng_pca")
    return out, kept.value


def export(ids, scores, k_eval=15, id_map=None, stream=None):
    import torch

    n, K = ids.shape
    knns = torch.empty((n, k_eval), dtype=torch.int32, device=ids.device)
    dists = torch.empty((n, k_eval), dtype=torch.float32, device=ids.device)
    st = lib().knng_export(_ptr(ids), _ptr(scores), n, K, k_eval, _ptr(id_map), _ptr(knns), _ptr(dists),
                           _stream_ptr(stream))
    if st != 0:
        raise KnngError(st, "knng_export")
    torch.cuda.synchronize(ids.device)
    return knns, dists


def init_graph_noalloc(codes, perm, leaf_flag, num_trees=16, leaf_size=64, k_build=50, seed=1337, ids=None,
                       scores=None, stream=None):
    """knng_init_graph_noalloc: the initial-graph stage with the library's fixed
    64 MiB device scratch instead of any allocation by the library.  For callers
    whose device memory is owned by another allocator; outputs may be passed in
    (preallocated from that allocator).  Returns (ids, scores)."""
    import torch

    n, d = codes.shape
    ids = torch.empty((n, k_build), dtype=torch.int32, device=codes.device) if ids is None else ids
    scores = torch.empty((n, k_build), dtype=torch.int32, device=codes.device) if scores is None else scores
    # buffers from a foreign pool are written by the kernels as they are: check
    # every shape, type, layout and device before the call
    want = [(codes, (n, d), torch.int8, "codes"), (perm, (num_trees, n), torch.int32, "perm"),
            (leaf_flag, (num_trees, n), torch.uint8, "leaf_flag"), (ids, (n, k_build), torch.int32, "ids"),
            (scores, (n, k_build), torch.int32, "scores")]
    for t, shape, dtype, name in want:
        if (tuple(t.shape) != shape or t.dtype != dtype or not t.is_contiguous() or not t.is_cuda
                or t.device != codes.device):
            raise KnngError(-1, f"init_graph_noalloc: {name} must be a contiguous {dtype} CUDA tensor of shape "
                                f"{shape} on {codes.device}, got {tuple(t.shape)} {t.dtype} on {t.device}")
    _ready(codes, perm, leaf_flag)
    st = lib().knng_init_graph_noalloc(_ptr(codes), n, d, num_trees, leaf_size, k_build, seed, _ptr(perm),
                                       _ptr(leaf_flag), _ptr(ids), _ptr(scores), _stream_ptr(stream))
    if st != 0:
        raise KnngError(st, "knng_init_graph_noalloc")
    return ids, scores
