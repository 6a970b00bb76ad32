"""The bounds-checked build (libknng_checked.so, compiled with -DKNNG_CHECKS).

Every index a kernel derives from its inputs (graph ids, permutation entries,
leaf positions, id maps) is checked before it addresses memory; a failed check
sets an error flag that the call returns as KNNG_E_BOUNDS.  No check traps.

The checked library runs in a child process (KNNG_LIBRARY selects it), on
small cases:
* with valid inputs its stages equal the oracle bit for bit, and a whole build
  equals the default library's build of the same rows;
* inputs with an id, a permutation entry or an id-map index outside its array
  return KNNG_E_BOUNDS (every such index is checked before use, so the bad
  value is never dereferenced), and the context builds correctly afterwards.
"""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sisap-2026-task1_gb300")
E_BOUNDS = -11

CHILD = textwrap.dedent(
    """
    import sys
    sys.path[:0] = [{pkg!r}, {orc!r}]
    import numpy as np
    import torch

    import knng
    import oracle
    import synth

    assert knng.LIB_PATH.endswith("libknng_checked.so"), knng.LIB_PATH
    E_BOUNDS = -11
    dev = torch.device("cuda:0")
    ref = np.load({npz!r})
    x = ref["x"]
    n, d = x.shape

    def expect_bounds(fn):
        try:
            fn()
        except knng.KnngError as e:
            assert e.status == E_BOUNDS, e
            return
        raise AssertionError("no KNNG_E_BOUNDS")

    codes_ref, sk_ref = oracle.quantize(x)
    codes, sk = knng.quantize(torch.from_numpy(x).to(dev))
    assert np.array_equal(codes.cpu().numpy(), codes_ref)
    prm_o = oracle.params(threads=1, tie_mode=oracle.TIE_STABLE, jacobi=1)
    perm_ref, lf_ref, piv = oracle.forest(codes_ref, prm_o, log_pivots=True)
    ids_ref, sc_ref = oracle.init_graph(codes_ref, perm_ref, lf_ref, prm_o)
    ids1_ref, sc1_ref = ids_ref.copy(), sc_ref.copy()
    up_ref = oracle.join_iter(codes_ref, sk_ref, ids1_ref, sc1_ref, prm_o)
    for gram in (0, 1):
        with knng.Context(gram_mode=gram) as ctx:
            perm, lf = ctx.forest(codes, replay=piv)
            assert np.array_equal(perm.cpu().numpy(), perm_ref)
            ids, sc = ctx.init_graph(codes, perm, lf)
            assert np.array_equal(ids.cpu().numpy(), ids_ref) and np.array_equal(sc.cpu().numpy(), sc_ref)
            ids1, sc1, up = ctx.join_iter(codes, sk, ids, sc)
            assert up == up_ref
            assert np.array_equal(ids1.cpu().numpy(), ids1_ref) and np.array_equal(sc1.cpu().numpy(), sc1_ref)
            # a permutation entry outside [0, n), then a negative one
            for bad_val in (n + 7, -5):
                bad = perm.clone()
                bad[3, 17] = bad_val
                expect_bounds(lambda: ctx.init_graph(codes, bad, lf))
            # graph ids outside [0, n): a neighbour of row 5 and a two-hop id
            for r, k, bad_val in ((5, 3, n + 5), (9, 0, -2)):
                bad = ids.clone()
                bad[r, k] = bad_val
                expect_bounds(lambda: ctx.join_iter(codes, sk, bad, sc))
            # the context is still usable and exact
            ids2, sc2 = ctx.init_graph(codes, perm, lf)
            assert np.array_equal(ids2.cpu().numpy(), ids_ref) and np.array_equal(sc2.cpu().numpy(), sc_ref)
            ids3, sc3, up3 = ctx.join_iter(codes, sk, ids2, sc2)
            assert up3 == up_ref and np.array_equal(ids3.cpu().numpy(), ids1_ref)
    # export: an id outside the id map
    idm = torch.arange(n, dtype=torch.int32, device=dev)
    k_ok, d_ok = knng.export(ids1, sc1, 15, id_map=idm)
    k_plain, _ = knng.export(ids1, sc1, 15)
    assert torch.equal(k_ok, k_plain)
    bad = ids1.clone()
    bad[7, 2] = n + 100
    expect_bounds(lambda: knng.export(bad, sc1, 15, id_map=idm))
    # a whole build equals the default library's build of the same rows
    with knng.Context() as ctx:
        kk, dd, st = ctx.build(x)
    assert np.array_equal(kk, ref["knns"]) and np.array_equal(dd, ref["dists"])
    print("checked ok")
    """
)


@pytest.fixture(scope="module")
def checked_lib():
    import importlib.util

    spec = importlib.util.spec_from_file_location("knng_build_script", os.path.join(PKG, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return b.build_checked()


@pytest.mark.gpu
def test_checked_build_exact_and_reports_bad_indices(checked_lib, tmp_path):
    import knng
    import synth

    x = synth.mixture(3000, 1024, 30, seed=11)
    with knng.Context() as ctx:
        kk, dd, _ = ctx.build(x)
    npz = str(tmp_path / "ref.npz")
    np.savez(npz, x=x, knns=kk, dists=dd)
    code = CHILD.format(pkg=PKG, orc=os.path.join(ROOT, "oracle"), npz=npz)
    env = dict(os.environ, KNNG_LIBRARY=checked_lib)
    r = subprocess.run([sys.executable, "-c", code], env=env, cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and "checked ok" in r.stdout, r.stdout[-3000:] + r.stderr[-3000:]
