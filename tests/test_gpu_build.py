"""Whole builds through knng_build (C ABI), evaluated as the reference's output is.

The graph is nondeterministic in the reference (threads race, nth_element and
partial_sort ties), so builds are compared by recall@15 against exact float64
brute force: the GPU build must land no more than 0.5 points below the
reference binary's recall on the same input (fixtures in tests/golden).  At
larger sizes size-independent properties are checked instead: each exported
row is a sorted list of distinct ids != self whose dists are the exact int8
inner products.
"""
import os

import numpy as np
import pytest

import oracle
import synth

pytestmark = pytest.mark.gpu
RECALL_TOL = 0.005
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def knng_mod():
    import torch

    assert torch.cuda.is_available(), "the gpu tests need a CUDA device"
    import knng

    knng.lib()
    return knng


def _golden(name):
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    x = mg.make_input(*mg.CASES[name])
    return x, np.load(os.path.join(HERE, "golden", name + ".npz"))


def _check_export(x, knns, dists, unique_rows=None):
    """Valid ids (no self), lists sorted, exact int8 scores on a sample of rows,
    and distinct ids in every sampled row (in the rows of unique_rows only, when
    given)."""
    n = x.shape[0]
    codes, _ = oracle.quantize(x)
    ids = knns.astype(np.int64) - 1
    assert ids.min() >= 0 and ids.max() < n
    assert not np.any(ids == np.arange(n)[:, None])
    assert np.all(np.diff(dists, axis=1) >= 0)  # worst -> best
    sample = np.arange(0, n, max(1, n // 500))
    exact = np.einsum("id,ikd->ik", codes[sample].astype(np.int32), codes[ids[sample]].astype(np.int32))
    np.testing.assert_array_equal(dists[sample], exact.astype(np.float32))
    for i in sample:
        if unique_rows is None or unique_rows[i]:
            assert len(np.unique(ids[i])) == ids.shape[1], i


@pytest.mark.parametrize("name", ["mix_n2000_d1024", "mix_n6000_d1024_c600", "mix_n3000_d384", "mix_n2500_d768",
                                  "sub_n8000_d1024_m32", "sub_n6000_d768_m48"])
@pytest.mark.parametrize("join", ["jacobi", "inplace"])
def test_build_recall_vs_reference(knng_mod, name, join):
    knng = knng_mod
    x, g = _golden(name)
    gt = synth.exact_knn(x, 15)
    ref_recall = synth.recall_at_k(g["knns"], gt)
    mode = knng.JOIN_JACOBI if join == "jacobi" else knng.JOIN_INPLACE
    with knng.Context(join_mode=mode) as ctx:
        knns, dists, st = ctx.build(x)
    rec = synth.recall_at_k(knns, gt)
    assert rec >= ref_recall - RECALL_TOL, (rec, ref_recall)
    _check_export(x, knns, dists)


@pytest.mark.parametrize("name", ["tiny_n2_d1024", "tiny_n40_d1024", "edge_n300_d1024"])
def test_build_small_inputs_match_oracle_exactly(knng_mod, name):
    # With n <= leaf_size no node splits, so the forest is the reference's; the
    # whole build then equals the oracle's double-buffered, stable-tie build
    # (random fills, adjacent-duplicate removal and pads included).  For n above
    # leaf_size the pivots differ and only recall is compared.
    knng = knng_mod
    x, g = _golden(name)
    with knng.Context() as ctx:
        knns, dists, st = ctx.build(x)
    if x.shape[0] <= 64:
        kr, dr, sr = oracle.build_graph(x, oracle.params(threads=1, tie_mode=oracle.TIE_STABLE, jacobi=1))
        assert st.iterations == sr.iterations
        np.testing.assert_array_equal(knns, kr)
        np.testing.assert_array_equal(dists, dr)
    else:
        gt = synth.exact_knn(x, 15)
        assert synth.recall_at_k(knns, gt) >= synth.recall_at_k(g["knns"], gt) - RECALL_TOL


def test_build_is_deterministic_and_io_independent(knng_mod):
    import torch

    knng = knng_mod
    x = synth.mixture(20000, 1024, 200, seed=21)
    with knng.Context() as ctx:
        k1, d1, _ = ctx.build(x)
        k2, d2, _ = ctx.build(x)
        xd = torch.from_numpy(x).cuda()
        k3, d3, _ = ctx.build(xd)
    np.testing.assert_array_equal(k1, k2)
    np.testing.assert_array_equal(d1, d2)
    np.testing.assert_array_equal(k1, k3.cpu().numpy())
    np.testing.assert_array_equal(d1, d3.cpu().numpy())


CHILD_BUILD = """
import hashlib, sys
sys.path[:0] = [{pkg!r}]
import knng, synth, torch
x = synth.mixture_torch(400_000, 1024, 4_000, seed=3003)
with knng.Context() as ctx:
    k, d, st = ctx.build(x)
h = hashlib.sha1()
for t in (x, k, d):
    h.update(t.contiguous().view(torch.uint8).cpu().numpy().tobytes())
print("digest", h.hexdigest(), [int(st.updates[i]) for i in range(st.iterations)])
"""


def test_build_is_deterministic_across_processes(knng_mod):
    """The same seeded rows give the same graph in separate processes (each
    autotunes its join on its own clock, so the variant choice may differ):
    400k rows generated on the GPU, built twice, in two child processes."""
    import subprocess
    import sys

    pkg = os.path.join(os.path.dirname(HERE), "sisap-2026-task1_gb300")
    outs = []
    for _ in range(2):
        r = subprocess.run([sys.executable, "-c", CHILD_BUILD.format(pkg=pkg)], capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stderr[-3000:]
        outs.append([ln for ln in r.stdout.splitlines() if ln.startswith("digest")][-1])
    assert outs[0] == outs[1], outs


def test_build_natural_and_leaf_order_agree(knng_mod):
    knng = knng_mod
    x = synth.mixture(8000, 768, 80, seed=22)
    with knng.Context(row_order=knng.ORDER_NATURAL) as a, knng.Context(row_order=knng.ORDER_LEAF) as b:
        ka, da, _ = a.build(x)
        kb, db, _ = b.build(x)
    np.testing.assert_array_equal(ka, kb)  # the Jacobi join does not depend on the row order
    np.testing.assert_array_equal(da, db)


@pytest.mark.parametrize("n,d,centres", [(30000, 1024, 300), (12000, 384, 60)])
def test_candidate_cache_changes_nothing(knng_mod, n, d, centres):
    """Builds with and without the per-row candidate cache give identical
    graphs and per-iteration update counts; with it, later iterations score
    far fewer sketches and rerank far fewer rows."""
    knng = knng_mod
    x = synth.mixture(n, d, centres, seed=31)
    with knng.Context(join_cache=1) as a, knng.Context(join_cache=0) as b:
        sa, sb = knng.Stats(), knng.Stats()
        ka, da, _ = a.build(x, None, None, sa)
        kb, db, _ = b.build(x, None, None, sb)
    np.testing.assert_array_equal(ka, kb)
    np.testing.assert_array_equal(da.view(np.uint32), db.view(np.uint32))
    assert sa.iterations == sb.iterations >= 3
    it = sa.iterations
    assert list(sa.updates[:it]) == list(sb.updates[:it])
    assert sa.join_candidates[0] == sb.join_candidates[0]  # empty cache in the first iteration
    assert sum(sa.join_candidates[2:it]) < 0.5 * sum(sb.join_candidates[2:it])
    assert sum(sa.join_dots[2:it]) < 0.5 * sum(sb.join_dots[2:it])


def test_candidate_cache_with_the_inplace_join(knng_mod):
    """The in-place join races like the reference's, so its graphs differ from
    run to run; with the cache its rows are still valid exact-dot lists."""
    knng = knng_mod
    x = synth.mixture(20000, 1024, 200, seed=32)
    with knng.Context(join_mode=knng.JOIN_INPLACE, join_cache=1) as ctx:
        k, dd, st = ctx.build(x)
    assert st.iterations >= 2
    _check_export(x, k, dd)


def test_build_rejects_bad_shapes(knng_mod):
    knng = knng_mod
    with knng.Context() as ctx:
        with pytest.raises(knng.KnngError) as e1:
            ctx.build(np.zeros((1, 1024), np.float32))
        assert e1.value.status == -1
        with pytest.raises(knng.KnngError) as e2:
            ctx.build(np.zeros((100, 100), np.float32))
        assert e2.value.status == -2
    with pytest.raises(knng.KnngError):
        knng.Context(k_build=65)


def test_build_one_million_properties(knng_mod):
    """1M x 1024 (the single-build configuration): properties on sampled rows and
    recall on 1,000 rows against exact brute force computed on the GPU."""
    import torch

    knng = knng_mod
    n, d = 1_000_000, 1024
    x = synth.mixture_torch(n, d, 10_000, seed=1001)
    with knng.Context() as ctx:
        knns, dists, st = ctx.build(x)
    assert st.iterations >= 1
    kh, dh = knns.cpu().numpy(), dists.cpu().numpy()
    ids = kh.astype(np.int64) - 1
    assert ids.min() >= 0 and ids.max() < n and not np.any(ids == np.arange(n)[:, None])
    assert np.all(np.diff(dh, axis=1) >= 0)
    rows = torch.randperm(n, generator=torch.Generator().manual_seed(7))[:1000].numpy()
    codes, _ = knng.quantize(x[torch.from_numpy(rows).cuda()])
    nb = torch.from_numpy(ids[rows]).cuda()
    qc = knng.quantize(x)[0]
    exact = torch.einsum("id,ikd->ik", codes.int().double(), qc[nb].int().double()).cpu().numpy()
    np.testing.assert_array_equal(dh[rows], exact.astype(np.float32))
    xs = x[torch.from_numpy(rows).cuda()].double()
    sims = xs @ x.double().T
    sims[torch.arange(len(rows)), torch.from_numpy(rows).cuda()] = -np.inf
    gt = sims.topk(15, dim=1).indices.cpu().numpy()
    rec = synth.recall_at_k(kh, gt, rows=rows)
    # sanity floor only: recall relative to the reference algorithm on these
    # same rows is tests/test_gpu_parity_scale.py
    assert rec > 0.3, rec


@pytest.mark.parametrize("fuse", [1, 0])
def test_build_degenerate_duplicates(knng_mod, fuse):
    """All-identical rows: no pivot separates them (every split peels one row, as in
    the reference), the forest's depth valve cuts the tail into leaves, and the
    graph is still a valid list of ids with exact scores.

    Among the identical rows every score ties, and the reference's initial list
    keeps an id twice when a random fill repeats a leaf candidate that a tied
    entry separates from it (it drops only adjacent repeats, src/main.cpp:295-302);
    no later visit can replace a tied entry.  The reference algorithm (the
    oracle's restatement) leaves repeated ids in about 1 % of these rows, so the
    ids are required distinct in the mixture half only."""
    knng = knng_mod
    x = np.tile(synth.mixture(1, 256, 1, seed=3), (5000, 1))
    x[:2500] = synth.mixture(2500, 256, 25, seed=4)  # half duplicates, half mixture
    with knng.Context(forest_fuse=fuse) as ctx:
        knns, dists, st = ctx.build(np.ascontiguousarray(x))
    _check_export(x, knns, dists, unique_rows=np.arange(5000) < 2500)


def _oracle_random_build(x, max_iter=30):
    """Random init (archive/nndescent_optimized.cpp) + the reference's iteration and
    early stop, in the oracle's double-buffered stable-tie mode."""
    prm = oracle.params(threads=1, tie_mode=oracle.TIE_STABLE, jacobi=1)
    codes, sk = oracle.quantize(x)
    ids, sc = oracle.init_random(codes, prm)
    n, K = ids.shape
    prev, it = np.float32(1.0), 0
    for it in range(max_iter):
        up = oracle.join_iter(codes, sk, ids, sc, prm)
        rate = np.float32(up) / np.float32(n * K)
        if rate < np.float32(0.04) or (it > 0 and (prev - rate) < np.float32(0.01)):
            it += 1
            break
        prev = rate
    else:
        it = max_iter
    k, d = oracle.export(ids, sc)
    return k, d, it


@pytest.mark.parametrize("iters", [0, 30])
def test_random_init_matches_oracle(knng_mod, iters):
    knng = knng_mod
    x = synth.mixture(4000, 768, 40, seed=61)
    with knng.Context(init_mode=knng.INIT_RANDOM, max_iterations=iters) as ctx:
        k, dd, st = ctx.build(x)
    kr, dr, itr = _oracle_random_build(x, iters)
    assert st.iterations == itr
    np.testing.assert_array_equal(k, kr)
    np.testing.assert_array_equal(dd, dr)


def _oracle_block_build(x, max_iter, block_size, bridges, k_build=50):
    """Block-partitioned hybrid init (archive/nndescent_hybrid.cpp) + the
    reference's iteration and early stop, oracle double-buffered stable ties."""
    prm = oracle.params(threads=1, tie_mode=oracle.TIE_STABLE, jacobi=1, k_build=k_build)
    codes, sk = oracle.quantize(x)
    ids, sc = oracle.init_block(codes, prm, block_size=block_size, bridges=bridges)
    n, K = ids.shape
    prev, it = np.float32(1.0), 0
    for it in range(max_iter):
        up = oracle.join_iter(codes, sk, ids, sc, prm)
        rate = np.float32(up) / np.float32(n * K)
        if rate < np.float32(0.04) or (it > 0 and (prev - rate) < np.float32(0.01)):
            it += 1
            break
        prev = rate
    else:
        it = max_iter
    k, d = oracle.export(ids, sc)
    return k, d, it


@pytest.mark.parametrize("iters", [0, 30])
def test_block_init_matches_oracle(knng_mod, iters):
    knng = knng_mod
    x = synth.mixture(4000, 768, 40, seed=62)
    with knng.Context(init_mode=knng.INIT_BLOCK, block_size=700, bridges=2, max_iterations=iters) as ctx:
        k, dd, st = ctx.build(x)
    kr, dr, itr = _oracle_block_build(x, iters, 700, 2)
    assert st.iterations == itr
    np.testing.assert_array_equal(k, kr)
    np.testing.assert_array_equal(dd, dr)


def test_block_init_archive_shape_and_batches(knng_mod):
    """The archive's own shape (K = 15, two bridges, equal blocks) at a small
    size, and a batch of two block-init jobs equal to the jobs alone."""
    knng = knng_mod
    x = synth.mixture(6000, 1024, 60, seed=63)
    y = synth.mixture(2500, 1024, 25, seed=64)
    kw = dict(init_mode=knng.INIT_BLOCK, block_size=1000, bridges=2, k_build=15, k_eval=15)
    with knng.Context(**kw) as ctx:
        kx, dx, sx = ctx.build(x)
        ky, dy, _ = ctx.build(y)
        res, _ = ctx.build_batch([x, y])
    kr, dr, itr = _oracle_block_build(x, 30, 1000, 2, k_build=15)
    assert sx.iterations == itr
    np.testing.assert_array_equal(kx, kr)
    np.testing.assert_array_equal(dx, dr)
    np.testing.assert_array_equal(res[0][0], kx)
    np.testing.assert_array_equal(res[1][0], ky)
    np.testing.assert_array_equal(res[1][1], dy)


def test_block_init_rejects_small_blocks(knng_mod):
    knng = knng_mod
    x = synth.mixture(1000, 384, 10, seed=65)
    with knng.Context(init_mode=knng.INIT_BLOCK, block_size=40) as ctx:  # 25 blocks of 40 < k_build + 1
        with pytest.raises(knng.KnngError) as e:
            ctx.build(x)
        assert e.value.status == -1
    with pytest.raises(knng.KnngError):
        knng.Context(init_mode=knng.INIT_BLOCK, bridges=51)
