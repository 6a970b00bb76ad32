"""The oracle's 128-bit random-hyperplane sketch against a numpy restatement.

The reference's README describes 128-bit random-hyperplane sketches
(README.md:33-34) but src/main.cpp keeps a coordinate-sign sketch, so the
optional hyperplane mode has no reference output to pin it.  Its definition is
restated here independently -- SplitMix64 plane values, a sum of four
uniform bytes per coordinate, the exact int32 projection of the int8 codes and
the strict `> 0` sign rule -- and the oracle (the checker of the CUDA kernel)
must agree bit for bit, including on codes at the int8 extremes.
"""
import numpy as np

import synth

M64 = (1 << 64) - 1


def _splitmix64(x):
    x = (x + 0x9E3779B97F4A7C15) & M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M64
    return x ^ (x >> 31)


def _planes(seed, d):
    g = np.empty((128, d), np.int64)
    for k in range(128):
        for j in range(d):
            h = _splitmix64(((seed << 32) ^ ((k << 10) | j)) & M64)
            g[k, j] = sum(((h >> (8 * b)) & 0xFF) // 4 - 32 for b in range(4))
    return g


def _sketch(codes, planes):
    dots = codes.astype(np.int64) @ planes.T
    bits = dots > 0
    words = np.zeros((codes.shape[0], 2), np.uint64)
    for k in range(128):
        words[:, k // 64] |= bits[:, k].astype(np.uint64) << np.uint64(k % 64)
    return words


def test_plane_values_match_numpy(oracle_mod):
    g = _planes(1337, 128)
    assert g.min() >= -128 and g.max() <= 124
    for k in (0, 1, 63, 64, 127):
        for j in (0, 5, 127):
            assert oracle_mod.plane_value(1337, k, j) == g[k, j]
    # close to a zero-mean bell: mean ~ -2 (the byte offset), spread ~ 37
    assert abs(g.mean() + 2) < 1.5 and 33 < g.std() < 41


def test_hyperplane_sketch_matches_numpy(oracle_mod):
    for d, seed in ((128, 1337), (384, 7)):
        x = synth.mixture(300, d, 6, seed=d)
        codes, _ = oracle_mod.quantize(x)
        codes[:20] = -128  # extremes: |dot| up to d * 128 * 128
        codes[20:40] = 127
        codes[40:45] = 0   # all-zero rows: every dot is 0, no bit set
        sk = oracle_mod.hyperplane_sketch(codes, seed)
        np.testing.assert_array_equal(sk, _sketch(codes, _planes(seed, d)))
        assert not sk[40:45].any()


def test_hyperplane_sketch_separates_neighbours(oracle_mod):
    """Close rows share more bits than random pairs (the point of the sketch)."""
    x = synth.mixture(2000, 1024, 20, seed=3)
    codes, _ = oracle_mod.quantize(x)
    sk = oracle_mod.hyperplane_sketch(codes)
    pc = np.vectorize(lambda v: bin(int(v)).count("1"))
    ham = lambda a, b: pc(sk[a, 0] ^ sk[b, 0]) + pc(sk[a, 1] ^ sk[b, 1])
    c32 = codes.astype(np.int32)
    best = np.argmax(c32[:50] @ c32.T - 10 ** 9 * np.eye(50, 2000, dtype=np.int64), axis=1)
    rand = np.random.default_rng(0).integers(0, 2000, 50)
    assert ham(np.arange(50), best).mean() < ham(np.arange(50), rand).mean() - 10
