"""Whole-build recall parity on identical rows, at the sizes the benchmark uses.

Each input is generated once and the same float32 bytes go to the GPU build
and to the reference algorithm -- the oracle's restatement of src/main.cpp
(pinned bit for bit to the reference binary by tests/test_oracle_golden.py),
run with the reference's own tie rules and in-place race on every host
thread.  recall@15 of both graphs is measured on the same seeded rows against
exact float64 brute force (scripts/evaluation/evaluate_submission.py:17-26),
and the GPU build may be at most 0.5 points below the reference's, as the
spec tolerance states.

* 1M x 1024, the single-build configuration (Gaussian mixture, 10k centres);
* 100k x 1024 on a 64-dimensional subspace: a high-recall regime (the
  reference reaches ~84 % in 7 iterations, near its published 85.3 % on the
  SISAP data), where half a point is a real difference.
"""
import os

import numpy as np
import pytest

import oracle
import synth

pytestmark = pytest.mark.gpu
RECALL_TOL = 0.005
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def env():
    import torch

    assert torch.cuda.is_available(), "the gpu tests need a CUDA device"
    import evaluate
    import knng

    knng.lib()
    return torch, knng, evaluate


def _parity(env, x_dev, sample_rows, seed=7):
    torch, knng, evaluate = env
    n = x_dev.shape[0]
    x_host = x_dev.cpu().numpy()
    with knng.Context() as ctx:
        kg, _, st = ctx.build(x_dev)
    kg = kg.cpu().numpy()
    kr, _, sr = oracle.build_graph(x_host, oracle.params(threads=THREADS))
    rows = torch.randperm(n, generator=torch.Generator().manual_seed(seed))[:sample_rows].numpy()
    gt = evaluate.sample_knn(x_dev, rows, 15)
    r_gpu = synth.recall_at_k(kg, gt, rows=rows)
    r_ref = synth.recall_at_k(kr, gt, rows=rows)
    print(f"n={n}: reference algorithm {100 * r_ref:.3f}% ({sr.iterations} iterations), "
          f"GPU {100 * r_gpu:.3f}% ({st.iterations} iterations)")
    return r_gpu, r_ref, st, sr


def test_recall_parity_high_recall_regime_100k(env):
    torch = env[0]
    x = torch.from_numpy(synth.subspace(100_000, 1024, 64, seed=5)).cuda()
    r_gpu, r_ref, st, sr = _parity(env, x, 20_000)
    assert r_ref > 0.78  # the regime is what it is meant to be
    assert r_gpu >= r_ref - RECALL_TOL, (r_gpu, r_ref)


def test_recall_parity_one_million_identical_rows(env):
    torch = env[0]
    x = synth.mixture_torch(1_000_000, 1024, 10_000, seed=1001)
    torch.cuda.synchronize()
    r_gpu, r_ref, st, sr = _parity(env, x, 10_000)
    assert r_gpu >= r_ref - RECALL_TOL, (r_gpu, r_ref)
