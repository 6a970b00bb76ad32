"""knng_init_graph_noalloc through the C ABI against knng_init_graph.

The no-allocation entry point serves callers whose device memory belongs to
another allocator (a framework's caching pool, a database's GPU memory
manager, a plugin host) and who therefore may not let the library call
cudaMalloc/cudaFree.  It runs the same initial-graph stage on a fixed 64 MiB
device array inside libknng.so.  Its output must equal the context-owned
entry point's bit for bit (the tolerance of every integer test here), on
consecutive calls that reuse the shared array, and inputs beyond the array's
limit must be refused before any device work.

This file is collected last on purpose (test_zz_*): a failure here leaves
every other test already run.
"""
import numpy as np
import pytest

import oracle
import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch

    assert torch.cuda.is_available(), "the gpu tests need a CUDA device"
    import knng

    knng.lib()
    return torch, knng


def _forest(torch, knng, n, d, c, seed, trees=16, leaf=64):
    x = synth.mixture(n, d, c, seed=seed)
    codes_ref, _ = oracle.quantize(x)
    codes = torch.from_numpy(codes_ref).cuda()
    with knng.Context(num_trees=trees, leaf_size=leaf) as ctx:
        perm, lf = ctx.forest(codes)
        ids, sc = ctx.init_graph(codes, perm, lf)
    return codes, perm, lf, ids, sc


def test_noalloc_matches_context_entry_on_consecutive_calls(env):
    torch, knng = env
    a = _forest(torch, knng, 12000, 1024, 120, seed=31)
    b = _forest(torch, knng, 3000, 384, 30, seed=32)
    for codes, perm, lf, ids, sc in (a, a, b, a):  # the array keeps the previous call's contents
        ids2, sc2 = knng.init_graph_noalloc(codes, perm, lf)
        torch.cuda.synchronize()
        assert torch.equal(ids2, ids)
        assert torch.equal(sc2, sc)


def test_noalloc_small_trees_and_tiny_input(env):
    torch, knng = env
    codes, perm, lf, ids, sc = _forest(torch, knng, 5000, 768, 500, seed=33, trees=4, leaf=16)
    ids2, sc2 = knng.init_graph_noalloc(codes, perm, lf, num_trees=4, leaf_size=16)
    assert torch.equal(ids2, ids) and torch.equal(sc2, sc)
    codes, perm, lf, ids, sc = _forest(torch, knng, 40, 1024, 4, seed=34)  # random-fill path
    ids2, sc2 = knng.init_graph_noalloc(codes, perm, lf)
    assert torch.equal(ids2, ids) and torch.equal(sc2, sc)


def test_noalloc_refuses_inputs_beyond_its_scratch(env):
    torch, knng = env
    codes = torch.zeros((16, 1024), dtype=torch.int8, device="cuda")
    perm = torch.zeros((16, 16), dtype=torch.int32, device="cuda")
    lf = torch.zeros((16, 16), dtype=torch.uint8, device="cuda")
    ids = torch.zeros((16, 50), dtype=torch.int32, device="cuda")
    # n = 20,000 rows x 16 trees needs ~87 MiB of scratch: refused before touching the buffers
    st = knng.lib().knng_init_graph_noalloc(knng._ptr(codes), 20000, 1024, 16, 64, 50, 1337, knng._ptr(perm),
                                            knng._ptr(lf), knng._ptr(ids), knng._ptr(ids), None)
    assert st == -10
    assert knng.lib().knng_status_string(-10).decode().startswith("input exceeds")
