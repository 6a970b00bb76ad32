"""GPU ground truth and the evaluator against exact float64 brute force, and the
knng_main CLI end to end (container or HDF5 in -> results/<task>/apex_simd.h5,
an HDF5 file, out)."""
import os
import subprocess
import sys

import numpy as np
import pytest

import synth

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sisap-2026-task1_gb300")


def test_all_knn_matches_float64_brute_force():
    import torch

    import evaluate

    x = synth.mixture(6000, 768, 60, seed=3)
    ids, sc = evaluate.all_knn(torch.from_numpy(x).cuda(), k=20)
    ids = ids.cpu().numpy()
    assert np.all(ids[:, 0] == np.arange(6000))  # self first (score 1)
    gt = synth.exact_knn(x, 19)  # self excluded
    np.testing.assert_array_equal(ids[:, 1:], gt)


def test_cli_and_evaluator_end_to_end(tmp_path):
    import h5container

    x = synth.mixture(8000, 1024, 80, seed=12)
    h5container.write(tmp_path / "data.h5", {"train": x})
    r = subprocess.run([os.path.join(PKG, "knng_main"), "--task", "task1", "--dataset", "data.h5"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "-> Iteration 1 Updates:" in r.stdout
    res = tmp_path / "results" / "task1" / "apex_simd.h5"
    assert open(res, "rb").read(8) == b"\x89HDF\r\n\x1a\n"
    ds, at = h5container.read(res, mmap=False)
    assert ds["knns"].shape == (8000, 15) and ds["dists"].dtype == np.float32
    assert set(at) == {"algo", "task", "buildtime", "querytime", "params"} and at["querytime"] == 0.0
    assert at["params"] == "K_BUILD=50, RERANK=8, TREES=16, LEAF=64, STOP=0.04, DIFF=0.01"
    ev = [sys.executable, os.path.join(PKG, "evaluate.py")]
    subprocess.run(ev + ["--ground-truth", "data.h5", "gt.h5"], cwd=tmp_path, check=True, capture_output=True)
    out = subprocess.run(ev + ["gt.h5", "results/task1/apex_simd.h5"], cwd=tmp_path, check=True,
                         capture_output=True, text=True).stdout
    rec = float(out.split("True Recall:")[1].split("%")[0]) / 100
    assert abs(rec - synth.recall_at_k(ds["knns"], synth.exact_knn(x, 15))) < 1e-6  # printed to 4 decimals in %


def test_cli_hdf5_input_matches_container_input(tmp_path):
    """The same /train as a chunked, shuffled+deflated HDF5 file and as a
    container gives the identical graph (the build is deterministic)."""
    import h5container

    sys.path.insert(0, os.path.join(ROOT, "tests", "golden", "hdf5"))
    import make_hdf5

    x = synth.mixture(5000, 384, 50, seed=21)
    (tmp_path / "a").mkdir()
    (tmp_path / "b").mkdir()
    h5container.write(tmp_path / "a" / "data.h5", {"train": x})
    make_hdf5.write_datasets(tmp_path / "b" / "data.h5", {"train": x}, chunks=(1000, 128), deflate=True)
    outs = []
    for sub in ("a", "b"):
        r = subprocess.run([os.path.join(PKG, "knng_main"), "data.h5"], cwd=tmp_path / sub, capture_output=True,
                           text=True)
        assert r.returncode == 0, r.stderr
        assert "[OK] Detected 5000 vectors in /train." in r.stdout
        outs.append(h5container.read(tmp_path / sub / "results" / "task1" / "apex_simd.h5", mmap=False)[0])
    assert np.array_equal(outs[0]["knns"], outs[1]["knns"])
    assert np.array_equal(outs[0]["dists"].view(np.uint32), outs[1]["dists"].view(np.uint32))
