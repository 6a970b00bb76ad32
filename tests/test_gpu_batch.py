"""Batched builds (knng_build_batch): each job's result is the same alone and in
any mix.

Jobs of different n and d are built together (equal-d jobs as one problem laid
out back to back).  Pivots, random fills and early stop are per job and the
NN-Descent update is double-buffered, so every job's knns/dists and iteration
count must equal knng_build of that job alone, bit for bit -- whatever the
batch composition, order, launch mode (CUDA graph or direct) or autotuned
join configuration.
"""
import numpy as np
import pytest

import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def knng_mod():
    import torch

    assert torch.cuda.is_available(), "the gpu tests need a CUDA device"
    import knng

    knng.lib()
    return knng


SPECS = [(3000, 1024, 30, 1), (40, 1024, 4, 2), (9000, 384, 90, 3), (1500, 768, 15, 4), (12000, 1024, 1200, 5),
         (70, 384, 2, 6), (5000, 768, 50, 7)]


@pytest.fixture(scope="module")
def datasets():
    return [synth.mixture(n, d, c, seed=100 + s) for n, d, c, s in SPECS]


@pytest.fixture(scope="module")
def solo(knng_mod, datasets):
    out = []
    with knng_mod.Context() as ctx:
        for x in datasets:
            k, dd, st = ctx.build(x)
            out.append((k, dd, st.iterations))
    return out


def _check(res, solo, order):
    for (k, dd, it), j in zip(res, order):
        np.testing.assert_array_equal(k, solo[j][0])
        np.testing.assert_array_equal(dd, solo[j][1])
        assert it == solo[j][2]


@pytest.mark.parametrize("graph", [1, 0])
def test_batch_equals_alone(knng_mod, datasets, solo, graph):
    with knng_mod.Context(use_graph=graph) as ctx:
        res, st = ctx.build_batch(datasets)
        assert st.graph_used == graph
    _check(res, solo, range(len(datasets)))


def test_batch_order_and_composition_do_not_matter(knng_mod, datasets, solo):
    order = [4, 0, 6, 2, 1]
    with knng_mod.Context() as ctx:
        res, _ = ctx.build_batch([datasets[j] for j in order])
        _check(res, solo, order)
        res2, _ = ctx.build_batch([datasets[j] for j in order])  # graph replay
        _check(res2, solo, order)


def test_batch_device_inputs_and_no_autotune(knng_mod, datasets, solo):
    import torch

    xs = [torch.from_numpy(x).cuda() for x in datasets[:4]]
    with knng_mod.Context(autotune=0) as ctx:
        res, _ = ctx.build_batch(xs)
    res = [(k.cpu().numpy(), dd.cpu().numpy(), it) for k, dd, it in res]
    _check(res, solo, range(4))


def test_batch_mixed_dims_dp4a_gram(knng_mod, datasets, solo):
    """Concurrent dimension groups launch the same kernels with different dynamic
    shared-memory sizes (the dp4a Gram's grows with d); each must keep working."""
    with knng_mod.Context(gram_mode=knng_mod.GRAM_DP4A, k_build=20, rerank_mult=3) as small:
        small.build_batch(datasets[:3])  # smaller join tables first
    with knng_mod.Context(gram_mode=knng_mod.GRAM_DP4A) as ctx:
        res, _ = ctx.build_batch(datasets)
    _check(res, solo, range(len(datasets)))
