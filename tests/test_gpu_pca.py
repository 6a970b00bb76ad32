"""PCA preprocessing on the GPU (knng_pca, `knng_main --pca`) against an exact
float64 restatement of scripts/data_prep/apply_pca.py:25-33 (sklearn's PCA is
a centred SVD; its components are the covariance eigenvectors, signed so that
each one's largest-magnitude entry is positive, then sklearn's normalize)."""
import os
import subprocess
import sys

import numpy as np
import pytest

import synth

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sisap-2026-task1_gb300")


def pca_f64(x, dims):
    x = x.astype(np.float64)
    xc = x - x.mean(axis=0)
    w, v = np.linalg.eigh(xc.T @ xc / (x.shape[0] - 1))
    order = np.argsort(w)[::-1]
    w, v = w[order], v[:, order]
    comp = v[:, :dims]
    big = np.argmax(np.abs(comp), axis=0)
    comp = comp * np.sign(comp[big, np.arange(dims)])
    y = xc @ comp
    y /= np.maximum(np.linalg.norm(y, axis=1, keepdims=True), 1e-300)
    return y, w[:dims].sum() / w.sum()


@pytest.fixture(scope="module")
def knng_mod():
    import torch

    assert torch.cuda.is_available(), "the gpu tests need a CUDA device"
    import knng

    knng.lib()
    return knng


def test_pca_matches_float64_components(knng_mod):
    """Well separated components (fewer than the mixture's centres): every
    projected coordinate equals the float64 PCA up to f16 rounding."""
    x = synth.mixture(20000, 1024, 64, seed=71)
    y, kept = knng_mod.pca(x, 32)
    yr, kr = pca_f64(x, 32)
    assert y.dtype == np.float16 and y.shape == (20000, 32)
    assert abs(kept - kr) < 1e-4
    flip = np.sign(np.sum(y.astype(np.float64) * yr, axis=0))
    assert (flip > 0).sum() >= 30  # the sign rule agrees but for near-tied largest entries
    np.testing.assert_allclose(y.astype(np.float64) * flip, yr, rtol=0, atol=2e-3)
    np.testing.assert_allclose(np.linalg.norm(y.astype(np.float64), axis=1), 1.0, atol=2e-3)


def test_pca_subspace_for_wide_projections(knng_mod):
    """Past the mixture's centres the trailing eigenvalues are nearly equal, so
    single components are not determined; the projected rows' mutual cosines
    (invariant under rotations within the kept subspace) are."""
    x = synth.mixture(12000, 768, 40, seed=72)
    y, kept = knng_mod.pca(x, 256)
    yr, kr = pca_f64(x, 256)
    assert abs(kept - kr) < 1e-4
    s = np.arange(0, 12000, 60)
    g = y[s].astype(np.float64) @ y[s].astype(np.float64).T
    gr = yr[s] @ yr[s].T
    np.testing.assert_allclose(g, gr, rtol=0, atol=1e-2)


def test_cli_pca_writes_f16_train_and_copies_ground_truth(knng_mod, tmp_path):
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden", "hdf5"))
    import hdf5read
    import make_hdf5

    x = synth.mixture(6000, 1024, 60, seed=73)
    gt = synth.exact_knn(x[:500], 10).astype(np.int32) + 1
    make_hdf5.write_datasets(tmp_path / "in.h5", {"train": x, "allknn/knns": gt,
                                                 "allknn/dists": gt.astype(np.float32)})
    r = subprocess.run([os.path.join(PKG, "knng_main"), "--pca", str(tmp_path / "in.h5"), str(tmp_path / "out.h5"),
                        "128"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "Variance Retained" in r.stdout
    ds, _ = hdf5read.read(tmp_path / "out.h5")
    assert ds["train"].dtype == np.float16 and ds["train"].shape == (6000, 128)
    np.testing.assert_array_equal(ds["allknn/knns"], gt)
    yr, _ = pca_f64(x, 128)
    s = np.arange(0, 6000, 50)
    g = ds["train"][s].astype(np.float64) @ ds["train"][s].astype(np.float64).T
    np.testing.assert_allclose(g, yr[s] @ yr[s].T, rtol=0, atol=1e-2)
    # the reduced file is a valid build input (f16 /train read as float32)
    r = subprocess.run([os.path.join(PKG, "knng_main"), str(tmp_path / "out.h5")], capture_output=True, text=True,
                       cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "[OK] Detected 6000 vectors in /train." in r.stdout
