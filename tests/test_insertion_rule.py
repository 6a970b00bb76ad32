"""The join's rank-counting insertion equals the reference's shift-insert loop.

The reference visits the reranked candidates in order and, for each one whose
dot beats the pool's last score, shift-inserts it after every entry with a
score >= its dot, dropping the last entry (src/main.cpp:411-418).  The GPU join
(stage G/H of csrc/join.cu) decides the same thing without the sequential
loop:

* survivor t is inserted iff fewer than K of {starting scores} and {dots of
  survivors visited before t} are >= its dot;
* the final pool is the best K of (starting entries, inserted survivors),
  ordered by score, ties first to starting entries (in pool order), then to
  earlier visits.

This test checks that rule against the loop on random sorted pools and
survivor sequences with many ties (small value ranges), pure Python.
"""
import random

import pytest


def shift_insert(pool_ids, pool_sc, survivors):
    """The reference's loop (survivor ids are distinct and not in the pool)."""
    ids, sc = list(pool_ids), list(pool_sc)
    K = len(ids)
    for sid, dot in survivors:
        if not dot > sc[K - 1]:
            continue
        pos = sum(1 for k in range(K - 1) if sc[k] >= dot)
        ids[pos + 1:] = ids[pos:K - 1]
        sc[pos + 1:] = sc[pos:K - 1]
        ids[pos], sc[pos] = sid, dot
    return ids, sc


def rank_rule(pool_ids, pool_sc, survivors):
    """The kernel's rule: acceptance by counting, then ranks over the union."""
    K = len(pool_ids)
    acc = []
    for t, (sid, dot) in enumerate(survivors):
        ge = sum(1 for s in pool_sc if s >= dot) + sum(1 for _, d in survivors[:t] if d >= dot)
        acc.append(ge < K)
    out_ids, out_sc = [None] * K, [None] * K
    for k in range(K):  # starting entry k: earlier entries, plus inserted survivors with a larger dot
        rank = k + sum(1 for a, (_, d) in zip(acc, survivors) if a and d > pool_sc[k])
        if rank < K:
            out_ids[rank], out_sc[rank] = pool_ids[k], pool_sc[k]
    for t, (sid, dot) in enumerate(survivors):
        if not acc[t]:
            continue
        rank = sum(1 for s in pool_sc if s >= dot)
        rank += sum(1 for q, (a, (_, d)) in enumerate(zip(acc, survivors)) if a and (d > dot or (d == dot and q < t)))
        if rank < K:
            out_ids[rank], out_sc[rank] = sid, dot
    assert None not in out_ids  # the ranks fill every position exactly once
    return out_ids, out_sc


@pytest.mark.parametrize("seed", range(8))
def test_rank_rule_equals_shift_insert(seed):
    rng = random.Random(seed)
    for _ in range(400):
        K = rng.choice([1, 2, 3, 5, 8, 15, 50])
        span = rng.choice([3, 10, 1000])  # small spans force ties
        pool_sc = sorted((rng.randrange(span) for _ in range(K)), reverse=True)
        pool_ids = list(range(K))
        thr0 = pool_sc[-1]
        P = rng.randrange(0, 3 * K + 3)
        # survivors: distinct new ids with dots above the starting threshold
        survivors = [(1000 + t, thr0 + 1 + rng.randrange(span)) for t in range(P)]
        assert rank_rule(pool_ids, pool_sc, survivors) == shift_insert(pool_ids, pool_sc, survivors)


def test_rejected_survivors_do_not_move_the_threshold():
    # A survivor rejected at its visit has a dot <= the last score then, so
    # counting it among the earlier values never changes a later decision.
    pool_ids, pool_sc = [0, 1, 2], [9, 7, 5]
    survivors = [(10, 8), (11, 6), (12, 6), (13, 7), (14, 9)]
    assert rank_rule(pool_ids, pool_sc, survivors) == shift_insert(pool_ids, pool_sc, survivors)
    assert shift_insert(pool_ids, pool_sc, survivors) == ([0, 14, 10], [9, 9, 8])
