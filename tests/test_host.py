"""Host-side checks that need no GPU: the C ABI library loads and exports every
entry point include/knng.h declares, the CLI keeps the reference's argv and
failure behaviour, the container I/O round-trips, and the synthetic
generator is deterministic."""
import os
import re
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sisap-2026-task1_gb300")


@pytest.fixture(scope="module")
def built():
    import importlib.util

    spec = importlib.util.spec_from_file_location("knng_build_script", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    return mod


def declared_functions():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(knng_[a-z_0-9]+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("knng_create", "knng_build", "knng_destroy", "knng_quantize", "knng_forest",
                 "knng_init_graph", "knng_join_iter", "knng_export"):
        assert must in names


def test_library_exports_every_declared_symbol(built):
    import ctypes

    lib = ctypes.CDLL(os.path.join(PKG, "libknng.so"))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_lists_exports(built):
    import knng

    assert set(knng.EXPORTS) <= set(declared_functions())
    p = knng.params()
    assert (p.k_build, p.k_eval, p.num_trees, p.rerank_mult, p.leaf_size, p.max_iterations) == (50, 15, 16, 8, 64, 30)
    assert abs(p.early_stop_rate - 0.04) < 1e-7 and abs(p.rate_diff_tol - 0.01) < 1e-7 and p.seed == 1337


def test_cli_without_dataset_fails_like_reference(built, tmp_path):
    r = subprocess.run([os.path.join(PKG, "knng_main"), "--task", "t"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 255
    assert "[FATAL] No filename provided." in r.stderr
    assert "[INFO] Target Task: t" in r.stdout


def test_cli_missing_file_fails(built, tmp_path):
    r = subprocess.run([os.path.join(PKG, "knng_main"), "nope.h5"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 255
    assert "[INFO] Target Dataset: nope.h5" in r.stdout
    assert "[FATAL]" in r.stderr


def test_container_roundtrip(tmp_path):
    import h5container

    x = np.random.default_rng(0).standard_normal((17, 128)).astype(np.float32)
    h = x.astype(np.float16)
    path = tmp_path / "a.h5"
    h5container.write(path, {"train": x, "half": h, "ids": np.arange(6, dtype=np.int32).reshape(2, 3)},
                      {"algo": "x"}, {"buildtime": 1.5})
    ds, at = h5container.read(path)
    np.testing.assert_array_equal(ds["train"], x)
    np.testing.assert_array_equal(ds["half"], h)
    assert at == {"algo": "x", "buildtime": 1.5}


def test_synth_is_deterministic():
    import synth

    a = synth.mixture(500, 128, 7, seed=3)
    b = synth.mixture(500, 128, 7, seed=3)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_allclose(np.linalg.norm(a, axis=1), 1.0, atol=1e-5)


def test_torch_mixture_is_reproducible_and_seeded():
    """The bench's generator: the same arguments give the same rows (labels from
    numpy's PCG64, centres and noise from a seeded torch generator), another
    seed gives other rows, and every row is a unit vector."""
    import torch

    import synth

    a = synth.mixture_torch(3000, 128, 40, seed=11, device="cpu", chunk=1000)
    b = synth.mixture_torch(3000, 128, 40, seed=11, device="cpu", chunk=1000)
    c = synth.mixture_torch(3000, 128, 40, seed=12, device="cpu", chunk=1000)
    assert torch.equal(a, b) and not torch.equal(a, c)
    torch.testing.assert_close(a.norm(dim=1), torch.ones(3000), atol=1e-5, rtol=0)


def test_bench_arms_print_the_same_config():
    """bench.py's GPU arm and reference arm name one configuration, so their
    lines compare like for like (the reference arm times a bounded sample of it)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)

    class P:  # the library's default parameters, as knng.params() returns them
        k_eval, k_build, num_trees, leaf_size, rerank_mult = 15, 50, 16, 64, 8

    for name in bench.CONFIGS:
        for ws in (1, 8):
            assert bench.workload_config(name, ws, P()) == bench.workload_config(name, ws)


def test_recall_matches_evaluator_definition():
    import synth

    gt = np.array([[1, 2, 3], [0, 2, 3]])
    pred = np.array([[2, 3, 4], [1, 3, 4]])  # 1-based
    # row 0: {1,2,3} vs gt {1,2,3} -> 3; row 1: {0,2,3} vs {0,2,3} -> 3
    assert synth.recall_at_k(pred, gt) == 1.0
