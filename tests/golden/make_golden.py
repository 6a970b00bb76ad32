"""Regenerate the golden fixtures in this folder from the reference binary.

Each fixture is the output of the unmodified reference src/main.cpp (compiled
by oracle/Makefile into oracle/_ref/ against the container-file H5Cpp shim) run
with OMP_NUM_THREADS=1, which makes it deterministic, on a seeded synthetic
input.  The inputs themselves are not stored: the file keeps the generator
arguments and the SHA-256 of the float32 bytes, and the tests regenerate them.

Run from the repository root after `make -C oracle all ref`:
    python tests/golden/make_golden.py [NAME ...]      # all fixtures, or the named ones
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "sisap-2026-task1_gb300"))
import oracle as O  # noqa: E402
import synth  # noqa: E402

# name: (kind, n, d, centres or subspace dimension, seed)
CASES = {
    "mix_n2000_d1024": ("mixture", 2000, 1024, 20, 11),
    "mix_n3000_d384": ("mixture", 3000, 384, 30, 12),
    "mix_n2500_d768": ("mixture", 2500, 768, 25, 13),
    "mix_n6000_d1024_c600": ("mixture", 6000, 1024, 600, 14),
    "edge_n300_d1024": ("edge", 300, 1024, 3, 15),
    "tiny_n40_d1024": ("mixture", 40, 1024, 4, 16),
    "tiny_n2_d1024": ("mixture", 2, 1024, 1, 17),
    # low intrinsic dimension (synth.subspace): the reference reaches high recall
    "sub_n8000_d1024_m32": ("subspace", 8000, 1024, 32, 18),
    "sub_n6000_d768_m48": ("subspace", 6000, 768, 48, 19),
}

# Values at the quantiser's corners (src/main.cpp:184-190): sub-code positives
# (code 0, sign bit 1), sub-code negatives, exact +-1, beyond the clamp on both
# sides, signed zeros, values that truncate rather than round, and subnormals
# (read as zero by the reference's -ffast-math build).
EDGE_VALUES = np.array([0.5 / 127, -0.5 / 127, 1.0, -1.0, 1.02, -1.5, 127.4 / 127, -128.6 / 127,
                        0.0, -0.0, 2.9 / 127, -2.9 / 127, 126.99 / 127, -127.99 / 127, 3.0, -3.0,
                        1e-40, -1e-40],
                       dtype=np.float32)


def make_input(kind, n, d, centres, seed):
    if kind == "subspace":
        return synth.subspace(n, d, centres, seed)
    x = synth.mixture(n, d, centres, seed)
    if kind == "edge":
        rng = np.random.Generator(np.random.PCG64(seed + 1))
        cols = rng.integers(0, d, size=(n, 24))
        vals = EDGE_VALUES[rng.integers(0, len(EDGE_VALUES), size=(n, 24))]
        np.put_along_axis(x, cols, vals, axis=1)
    return x


def digest(x):
    return hashlib.sha256(np.ascontiguousarray(x, dtype=np.float32).tobytes()).hexdigest()


def main(names=None):
    for name, (kind, n, d, c, seed) in CASES.items():
        if names and name not in names:
            continue
        x = make_input(kind, n, d, c, seed)
        knns, dists, attrs, out = O.run_reference(x, threads=1)
        iters = sum(1 for ln in out.splitlines() if "-> Iteration" in ln)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), knns=knns, dists=dists,
                            sha256=np.array(digest(x)), iterations=np.array(iters),
                            params=np.array(attrs["params"]), algo=np.array(attrs["algo"]))
        print(name, knns.shape, "iterations", iters)


if __name__ == "__main__":
    main(sys.argv[1:])
