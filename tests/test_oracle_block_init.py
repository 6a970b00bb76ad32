"""The oracle's restatement of the archived block-partitioned hybrid init
(archive/nndescent_hybrid.cpp:98-144), on CPU: every row keeps the best rows
of its own block except for the bridge entries, lists are sorted by score,
scores are the exact int8 dots, and the result does not depend on the thread
count (the archive's per-thread generator made it do so)."""
import numpy as np

import synth


def test_block_init_properties(oracle_mod):
    x = synth.mixture(3000, 384, 30, seed=5)
    codes, _ = oracle_mod.quantize(x)
    prm = oracle_mod.params(threads=1)
    ids, sc = oracle_mod.init_block(codes, prm, block_size=500, bridges=2)
    n, K = ids.shape
    nb = 6  # round(3000 / 500)
    q = np.arange(n) * nb // n
    lo, hi = q * n // nb, (q + 1) * n // nb
    inside = (ids >= lo[:, None]) & (ids < hi[:, None])
    assert np.all(inside.sum(axis=1) >= K - 2)  # only the two bridges may leave the block
    assert np.all(np.diff(sc.astype(np.int64), axis=1) <= 0)
    assert not np.any(ids == np.arange(n)[:, None])
    c = codes.astype(np.int32)
    exact = np.einsum("id,ikd->ik", c, c[ids])
    np.testing.assert_array_equal(sc, exact)
    # the in-block entries are the block's K - 2 best at least
    i = 123
    block = [j for j in range(lo[i], hi[i]) if j != i]
    best = sorted(block, key=lambda j: (-int(c[i] @ c[j]), j))[: K - 2]
    assert set(best) <= set(ids[i].tolist())
    ids4, sc4 = oracle_mod.init_block(codes, oracle_mod.params(threads=4), block_size=500, bridges=2)
    np.testing.assert_array_equal(ids, ids4)
    np.testing.assert_array_equal(sc, sc4)
