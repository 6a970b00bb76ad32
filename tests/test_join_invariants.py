"""Invariants the GPU join relies on, checked on the oracle's restatement of the
reference iteration (src/main.cpp:320-440), on CPU.

* A row's pool threshold (its K-th score) never falls from one iteration to
  the next: the row changes only by its own insertions of better candidates.
  The candidate cache keeps "dot <= threshold" rejections across iterations
  on the strength of this.
* A row's pool stays sorted by score, descending, with distinct ids: the rank
  counting insertion needs a sorted pool.
Both the double-buffered schedule (the GPU default) and the reference's
in-place schedule (single-threaded oracle) are checked.
"""
import numpy as np
import pytest

import synth


@pytest.mark.parametrize("jacobi", [1, 0])
def test_threshold_never_falls_and_pools_stay_sorted(oracle_mod, jacobi):
    x = synth.mixture(3000, 384, 30, seed=41)
    prm = oracle_mod.params(threads=1, tie_mode=oracle_mod.TIE_STABLE, jacobi=jacobi)
    codes, sk = oracle_mod.quantize(x)
    perm, lf, _ = oracle_mod.forest(codes, prm)
    ids, sc = oracle_mod.init_graph(codes, perm, lf, prm)
    K = ids.shape[1]
    prev = sc[:, K - 1].copy()
    for it in range(6):
        updates = oracle_mod.join_iter(codes, sk, ids, sc, prm)
        assert np.all(sc[:, K - 1] >= prev), f"a threshold fell in iteration {it}"
        assert np.all(np.diff(sc.astype(np.int64), axis=1) <= 0), "a pool is not sorted"
        srt = np.sort(ids, axis=1)
        assert not np.any(srt[:, 1:] == srt[:, :-1]), "a pool repeats an id"
        prev = sc[:, K - 1].copy()
        if updates == 0:
            break
