"""CUDA path against the oracle, stage by stage, through the libknng C ABI.

Bit-exact: int8 codes, sign sketches, forest leaf order (replaying the
reference's own std::mt19937 pivots), initial graph ids and scores, each
NN-Descent iteration (double-buffered, ties ordered by (hamming desc,
sequence position asc) in both), export.  Whole builds are evaluated by
recall@15 against exact float64 brute force, next to the reference binary's
recall on the same input (tests/golden), within 0.5 points.
"""
import numpy as np
import pytest

import oracle
import synth

pytestmark = pytest.mark.gpu
RECALL_TOL = 0.005  # recall@15 may be at most 0.5 points below the reference's


@pytest.fixture(scope="module")
def torch_dev():
    import torch

    assert torch.cuda.is_available(), "the gpu tests need a CUDA device"
    import knng

    knng.lib()  # fails loudly if libknng.so is missing
    return torch, torch.device("cuda:0")


def _stable(**kw):
    return oracle.params(threads=1, tie_mode=oracle.TIE_STABLE, jacobi=1, **kw)


def _edge_rows(n, d, seed):
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal((n, d)) * rng.choice([0.01, 0.03, 0.3, 2.0], size=(n, 1))).astype(np.float32)
    vals = np.array([0.5 / 127, -0.5 / 127, 1.0, -1.0, 1.02, -1.5, 127.4 / 127, -128.6 / 127, 0.0, -0.0,
                     2.9 / 127, -2.9 / 127, 1e-40, -1e-40, 3.0, -3.0, np.inf, -np.inf], np.float32)
    cols = rng.integers(0, d, size=(n, 32))
    np.put_along_axis(x, cols, vals[rng.integers(0, len(vals), size=(n, 32))], axis=1)
    return x


@pytest.mark.parametrize("d", [128, 384, 768, 1024])
@pytest.mark.parametrize("mode", [oracle.QUANT_TRUNC, oracle.QUANT_ROUND])
def test_quantize_bit_exact(torch_dev, d, mode):
    torch, dev = torch_dev
    import knng

    x = _edge_rows(1537, d, seed=d + mode)
    codes_ref, sk_ref = oracle.quantize(x, mode)
    codes, sk = knng.quantize(torch.from_numpy(x).to(dev), mode)
    np.testing.assert_array_equal(codes.cpu().numpy(), codes_ref)
    np.testing.assert_array_equal(sk.cpu().numpy().view(np.uint64), sk_ref)


@pytest.mark.parametrize("n,d,c,leaf,trees", [(3000, 1024, 30, 64, 16), (5000, 384, 50, 64, 16),
                                               (4000, 768, 400, 16, 4), (70, 1024, 2, 64, 16),
                                               (64, 1024, 2, 64, 16), (2, 1024, 1, 64, 16)])
def test_forest_replay_matches_reference_pivots(torch_dev, n, d, c, leaf, trees):
    torch, dev = torch_dev
    import knng

    x = synth.mixture(n, d, c, seed=n + d)
    codes_ref, _ = oracle.quantize(x)
    prm = _stable(leaf_size=leaf, num_trees=trees)
    perm_ref, lf_ref, piv = oracle.forest(codes_ref, prm, log_pivots=True)
    with knng.Context(leaf_size=leaf, num_trees=trees) as ctx:
        perm, lf = ctx.forest(torch.from_numpy(codes_ref).to(dev), replay=piv)
    np.testing.assert_array_equal(perm.cpu().numpy(), perm_ref)
    np.testing.assert_array_equal(lf.cpu().numpy(), lf_ref)


def test_forest_replay_rejects_wrong_table(torch_dev):
    torch, dev = torch_dev
    import knng

    x = synth.mixture(3000, 1024, 30, seed=3)
    codes_ref, _ = oracle.quantize(x)
    _, _, piv = oracle.forest(codes_ref, _stable(), log_pivots=True)
    bad = piv.copy()
    bad[5, 3] += 1  # wrong node size
    with knng.Context() as ctx:
        with pytest.raises(knng.KnngError) as ei:
            ctx.forest(torch.from_numpy(codes_ref).to(dev), replay=bad)
        assert ei.value.status == -7


def _check_forest_invariants(perm, lf, n, leaf):
    for t in range(perm.shape[0]):
        assert np.array_equal(np.sort(perm[t]), np.arange(n))
        starts = np.flatnonzero(lf[t])
        assert starts[0] == 0
        sizes = np.diff(np.append(starts, n))
        assert sizes.min() >= 1 and sizes.max() <= leaf


@pytest.mark.parametrize("fuse", [1, 0])
@pytest.mark.parametrize("n,d", [(20000, 1024), (3000, 384), (120000, 128)])
def test_forest_native_invariants_and_init(torch_dev, n, d, fuse):
    """Native pivots, three levels per pass (fuse = 1: two fused rounds and the
    per-level tail at 20000 rows, more rounds at 120000) or one level per pass."""
    torch, dev = torch_dev
    import knng

    x = synth.mixture(n, d, n // 100, seed=7)
    codes_ref, _ = oracle.quantize(x)
    codes = torch.from_numpy(codes_ref).to(dev)
    with knng.Context(forest_fuse=fuse) as ctx:
        perm, lf = ctx.forest(codes)
        perm_h, lf_h = perm.cpu().numpy(), lf.cpu().numpy()
        _check_forest_invariants(perm_h, lf_h, n, 64)
        # the init merge from the GPU's own forest equals the oracle's on that forest
        ids_ref, sc_ref = oracle.init_graph(codes_ref, perm_h, lf_h, _stable())
        ids, sc = ctx.init_graph(codes, perm, lf)
    np.testing.assert_array_equal(sc.cpu().numpy(), sc_ref)
    np.testing.assert_array_equal(ids.cpu().numpy(), ids_ref)


@pytest.mark.parametrize("n,d,c,leaf,trees", [(3000, 1024, 30, 64, 16), (2500, 768, 25, 64, 16),
                                               (40, 1024, 4, 64, 16), (2, 1024, 1, 64, 16),
                                               (3000, 1024, 300, 8, 3)])
def test_init_graph_bit_exact(torch_dev, n, d, c, leaf, trees):
    torch, dev = torch_dev
    import knng

    x = synth.mixture(n, d, c, seed=n + 1)
    codes_ref, _ = oracle.quantize(x)
    prm = _stable(leaf_size=leaf, num_trees=trees)
    perm_ref, lf_ref, _ = oracle.forest(codes_ref, prm)
    ids_ref, sc_ref = oracle.init_graph(codes_ref, perm_ref, lf_ref, prm)
    with knng.Context(leaf_size=leaf, num_trees=trees) as ctx:
        ids, sc = ctx.init_graph(torch.from_numpy(codes_ref).to(dev), torch.from_numpy(perm_ref).to(dev),
                                 torch.from_numpy(lf_ref).to(dev))
    np.testing.assert_array_equal(sc.cpu().numpy(), sc_ref)
    np.testing.assert_array_equal(ids.cpu().numpy(), ids_ref)
    # Rows whose leaves give at least K distinct candidates need no random fill;
    # there the reference's own (unstable) tie order gives the same score vectors.
    # (With fills, adjacent-duplicate removal depends on the sort's tie order.)
    _, sc_tie = oracle.init_graph(codes_ref, perm_ref, lf_ref, oracle.params(threads=1, leaf_size=leaf,
                                                                              num_trees=trees))
    union = [set() for _ in range(n)]
    for t in range(trees):
        starts = np.append(np.flatnonzero(lf_ref[t]), n)
        for a, b in zip(starts[:-1], starts[1:]):
            members = perm_ref[t, a:b].tolist()
            for i in members:
                union[i].update(members)
    no_fill = np.array([len(u) - 1 >= prm.k_build for u in union])
    np.testing.assert_array_equal(sc.cpu().numpy()[no_fill], sc_tie[no_fill])


@pytest.mark.parametrize("n,d,c,k,mult", [(3000, 1024, 30, 50, 8), (6000, 1024, 600, 50, 8),
                                           (3000, 384, 30, 50, 8), (2000, 1024, 200, 20, 3),
                                           (40, 1024, 4, 50, 8)])
def test_join_iterations_bit_exact(torch_dev, n, d, c, k, mult):
    torch, dev = torch_dev
    import knng

    x = synth.mixture(n, d, c, seed=n + 2)
    codes_ref, sk_ref = oracle.quantize(x)
    prm = _stable(k_build=k, k_eval=min(15, k), rerank_mult=mult)
    perm_ref, lf_ref, _ = oracle.forest(codes_ref, prm)
    ids_ref, sc_ref = oracle.init_graph(codes_ref, perm_ref, lf_ref, prm)
    codes = torch.from_numpy(codes_ref).to(dev)
    sk = torch.from_numpy(sk_ref.view(np.int64)).to(dev)
    ids = torch.from_numpy(ids_ref.copy()).to(dev)
    sc = torch.from_numpy(sc_ref.copy()).to(dev)
    with knng.Context(k_build=k, k_eval=min(15, k), rerank_mult=mult) as ctx:
        for it in range(3):
            up_ref = oracle.join_iter(codes_ref, sk_ref, ids_ref, sc_ref, prm)
            ids, sc, up = ctx.join_iter(codes, sk, ids, sc)
            assert up == up_ref, f"iteration {it}"
            np.testing.assert_array_equal(sc.cpu().numpy(), sc_ref)
            np.testing.assert_array_equal(ids.cpu().numpy(), ids_ref)


def test_join_inplace_keeps_lists_exact(torch_dev):
    torch, dev = torch_dev
    import knng

    n, d = 4000, 1024
    x = synth.mixture(n, d, 40, seed=9)
    codes_ref, sk_ref = oracle.quantize(x)
    prm = _stable()
    perm_ref, lf_ref, _ = oracle.forest(codes_ref, prm)
    ids_ref, sc_ref = oracle.init_graph(codes_ref, perm_ref, lf_ref, prm)
    codes = torch.from_numpy(codes_ref).to(dev)
    sk = torch.from_numpy(sk_ref.view(np.int64)).to(dev)
    ids = torch.from_numpy(ids_ref.copy()).to(dev)
    sc = torch.from_numpy(sc_ref.copy()).to(dev)
    with knng.Context(join_mode=knng.JOIN_INPLACE) as ctx:
        for _ in range(2):
            ids, sc, up = ctx.join_iter(codes, sk, ids, sc, ids, sc)
            assert up > 0
    ids_h, sc_h = ids.cpu().numpy(), sc.cpu().numpy()
    assert np.all(np.diff(sc_h, axis=1) <= 0)  # each row sorted by score
    exact = np.einsum("id,ikd->ik", codes_ref.astype(np.int32), codes_ref[ids_h].astype(np.int32))
    np.testing.assert_array_equal(sc_h, exact)  # every score is the exact int8 dot
    for row in ids_h:
        assert len(np.unique(row)) == len(row)


def test_export_bit_exact(torch_dev):
    torch, dev = torch_dev
    import knng

    rng = np.random.default_rng(1)
    ids = rng.integers(0, 1000, size=(1000, 50)).astype(np.int32)
    sc = np.sort(rng.integers(-2 ** 24, 2 ** 24, size=(1000, 50)), axis=1)[:, ::-1].astype(np.int32)
    sc[:, -3:] = np.iinfo(np.int32).min
    kr, dr = oracle.export(ids, np.ascontiguousarray(sc), 15)
    k, dd = knng.export(torch.from_numpy(ids).to(dev), torch.from_numpy(np.ascontiguousarray(sc)).to(dev), 15)
    np.testing.assert_array_equal(k.cpu().numpy(), kr)
    np.testing.assert_array_equal(dd.cpu().numpy(), dr)


@pytest.mark.parametrize("k,mult", [(50, 8), (20, 3)])
def test_join_on_random_graph_bit_exact(torch_dev, k, mult):
    """Random neighbour lists (as after an init of tiny leaves): nearly every one of
    the K*K two-hop candidates is a distinct id, the worst case for the join's
    per-row tables."""
    torch, dev = torch_dev
    import knng

    n, d = 20000, 1024
    x = synth.mixture(n, d, 200, seed=41)
    codes_ref, sk_ref = oracle.quantize(x)
    rng = np.random.default_rng(5)
    ids_ref = np.empty((n, k), np.int32)
    for i in range(n):
        row = rng.choice(n - 1, size=k, replace=False)
        ids_ref[i] = row + (row >= i)
    c32 = codes_ref.astype(np.int32)
    sc_ref = np.einsum("id,ikd->ik", c32, c32[ids_ref]).astype(np.int32)
    o = np.argsort(-sc_ref, axis=1, kind="stable")
    ids_ref = np.ascontiguousarray(np.take_along_axis(ids_ref, o, axis=1))
    sc_ref = np.ascontiguousarray(np.take_along_axis(sc_ref, o, axis=1))
    prm = _stable(k_build=k, k_eval=min(15, k), rerank_mult=mult)
    codes = torch.from_numpy(codes_ref).to(dev)
    sk = torch.from_numpy(sk_ref.view(np.int64)).to(dev)
    ids = torch.from_numpy(ids_ref.copy()).to(dev)
    sc = torch.from_numpy(sc_ref.copy()).to(dev)
    with knng.Context(k_build=k, k_eval=min(15, k), rerank_mult=mult) as ctx:
        for _ in range(2):
            up_ref = oracle.join_iter(codes_ref, sk_ref, ids_ref, sc_ref, prm)
            ids, sc, up = ctx.join_iter(codes, sk, ids, sc)
            assert up == up_ref
            np.testing.assert_array_equal(sc.cpu().numpy(), sc_ref)
            np.testing.assert_array_equal(ids.cpu().numpy(), ids_ref)
