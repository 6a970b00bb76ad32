"""The initial graph's batched merge keeps the K best distinct keys.

The reference builds a row's initial list from the union of the row's leaves
in all trees, de-duplicated, best K by score (src/main.cpp:234-314).  The GPU
merge (init_merge in csrc/init.cu) holds the row's list in a warp, two keys per
lane (positions lane and 32 + lane, 0 = empty), and merges 32 candidates at a
time (merge_batch):

* candidates above the list's K-th key find their rank in the list by binary
  search; a candidate equal to a listed key is dropped;
* each remaining candidate's final rank is that position plus the number of
  remaining candidates with a larger key; each list entry moves down by the
  number of remaining candidates larger than it;
* everything is written at its rank in one scatter; ranks >= K drop out.

This test restates that step lane by lane in pure Python, checks that every
list position is written by exactly one lane (the scatter has no write
conflicts, so the kernel needs no atomics), and that after any sequence of
leaf halves the list equals the K best distinct keys seen, for every K the
library accepts and with keys repeated across trees as leaf-mates are.
"""
import random

import pytest


def merge_batch(kA, kB, keys, thr, K):
    """One merge of 32 lane keys into the list (kA: positions 0-31, kB: 32-63)."""
    want = [k > thr for k in keys]
    if not any(want):
        return kA, kB, thr
    sl = kA + kB
    lo = [0] * 32
    for lane in range(32):
        if want[lane]:
            a, b = 0, K
            while a < b:
                mid = (a + b) // 2
                if sl[mid] > keys[lane]:
                    a = mid + 1
                else:
                    b = mid
            lo[lane] = a
            if a < K and sl[a] == keys[lane]:
                want[lane] = False
    chosen = [lane for lane in range(32) if want[lane]]
    writes = {}
    for lane in range(32):
        above = sum(1 for s in chosen if keys[s] > keys[lane])
        c_a = sum(1 for s in chosen if keys[s] > kA[lane])
        c_b = sum(1 for s in chosen if keys[s] > kB[lane])
        if lane < K and lane + c_a < K:
            writes.setdefault(lane + c_a, []).append(kA[lane])
        if 32 + lane < K and 32 + lane + c_b < K:
            writes.setdefault(32 + lane + c_b, []).append(kB[lane])
        if want[lane] and lo[lane] + above < K:
            writes.setdefault(lo[lane] + above, []).append(keys[lane])
    new = list(sl)
    for pos, vals in writes.items():
        assert len(vals) == 1, (pos, vals)  # one writer per position
        new[pos] = vals[0]
    kA = [new[lane] if lane < K else 0 for lane in range(32)]
    kB = [new[32 + lane] if 32 + lane < K else 0 for lane in range(32)]
    thr = kA[K - 1] if K - 1 < 32 else kB[K - 33]
    return kA, kB, thr


@pytest.mark.parametrize("K", [1, 2, 15, 31, 32, 33, 50, 63, 64])
def test_batched_merge_keeps_the_k_best_distinct_keys(K):
    rng = random.Random(1000 + K)
    for _ in range(150):
        # a row's leaf-mates: a pool of distinct keys, each tree's leaf a
        # sample of it, so keys recur across trees as they do on the GPU
        pool = rng.sample(range(1, 500), 220)
        kA, kB, thr = [0] * 32, [0] * 32, 0
        seen = set()
        for _tree in range(rng.randint(1, 16)):
            m = rng.randint(1, 64)
            leaf = rng.sample(pool, m)
            for half in range(2):
                keys = [leaf[lane + 32 * half] if lane + 32 * half < m else 0 for lane in range(32)]
                kA, kB, thr = merge_batch(kA, kB, keys, thr, K)
                seen.update(k for k in keys if k)
        want = sorted(seen, reverse=True)[:K]
        want += [0] * (K - len(want))
        assert (kA + kB)[:K] == want


def test_batched_merge_of_a_full_list_with_no_candidate_above_it_changes_nothing():
    K = 50
    kA, kB, thr = [0] * 32, [0] * 32, 0
    kA, kB, thr = merge_batch(kA, kB, list(range(300, 268, -1)), thr, K)
    kA, kB, thr = merge_batch(kA, kB, list(range(268, 236, -1)), thr, K)
    before = (list(kA), list(kB), thr)
    kA, kB, thr = merge_batch(kA, kB, [thr] * 16 + list(range(1, 17)), thr, K)
    assert (kA, kB, thr) == before
