"""The oracle (CPU restatement) against fixtures made by the reference binary.

tests/golden/*.npz hold knns/dists written by the unmodified reference
src/main.cpp run single-threaded (tests/golden/make_golden.py).  With one
thread and the reference tie rules the restatement must reproduce them bit for
bit; this pins every stage of the oracle (quantiser, sketch, forest RNG,
leaf init, NN-Descent, export) before it is used to check the CUDA path.
"""
import glob
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def _load_case(path):
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    name = os.path.basename(path)[:-4]
    x = mg.make_input(*mg.CASES[name])
    return x, np.load(path), mg.digest


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_oracle_matches_reference_fixture(oracle_mod, path):
    x, g, digest = _load_case(path)
    assert digest(x) == str(g["sha256"]), "synthetic generator no longer reproduces the fixture input"
    knns, dists, st = oracle_mod.build_graph(x, oracle_mod.params(threads=1))
    assert st.iterations == int(g["iterations"])
    np.testing.assert_array_equal(knns, g["knns"])
    np.testing.assert_array_equal(dists, g["dists"])


def test_fixture_set_complete():
    assert len(FIXTURES) >= 7


def test_fixture_params_are_reference_defaults():
    g = np.load(FIXTURES[0])
    assert str(g["params"]) == "K_BUILD=50, RERANK=8, TREES=16, LEAF=64, STOP=0.04, DIFF=0.01"
    assert str(g["algo"]) == "Apex Hardware SIMD"
