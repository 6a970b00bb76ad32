"""Every NN-Descent kernel variant the autotuner can pick, bit for bit.

The join is compiled as six variants (3 or 4 resident CTAs per SM x 2, 4 or 8
Hamming candidates in flight per 8-lane group); the autotuner picks one per
(d, size) bucket and phase.  Each is forced here through the context's
join_ctas_per_sm / join_cblock and checked against the oracle's
double-buffered, stable-tie restatement of src/main.cpp:320-440:

* one iteration at a time through knng_join_iter (no candidate cache);
* whole builds with the candidate cache on, from the GPU's own initial graph
  (itself bit-exact against the oracle on the same forest) through the
  reference's early stop (src/main.cpp:432-439) to the exported knns/dists.
  These builds also copy unchanged rows through (a row whose list and
  neighbours' lists did not change in the previous iteration); the oracle
  computes every row, so the comparison covers that skip too.
"""
import os

import numpy as np
import pytest

import oracle
import synth

pytestmark = pytest.mark.gpu
VARIANTS = [(c, b) for c in (3, 4) for b in (2, 4, 8)]
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def env():
    import torch

    assert torch.cuda.is_available(), "the gpu tests need a CUDA device"
    import knng

    knng.lib()
    return torch, knng


def _stable(**kw):
    # double-buffered iterations are independent of the thread count
    return oracle.params(threads=THREADS, tie_mode=oracle.TIE_STABLE, jacobi=1, **kw)


def _oracle_from_init(codes, sk, ids, sc, prm, max_iter=30):
    """The reference's iteration loop and early stop from a given initial graph."""
    ids, sc = ids.copy(), sc.copy()
    n, K = ids.shape
    prev, it, ups = np.float32(1.0), 0, []
    for it in range(max_iter):
        up = oracle.join_iter(codes, sk, ids, sc, prm)
        ups.append(up)
        rate = np.float32(up) / np.float32(n * K)
        if rate < np.float32(prm.early_stop_rate) or (it > 0 and (prev - rate) < np.float32(prm.rate_diff_tol)):
            it += 1
            break
        prev = rate
    else:
        it = max_iter
    k, d = oracle.export(ids, sc, prm.k_eval)
    return k, d, it, ups


@pytest.fixture(scope="module")
def iter_case():
    n, d = 6000, 1024
    x = synth.mixture(n, d, 600, seed=n + 2)
    codes, sk = oracle.quantize(x)
    prm = _stable()
    perm, lf, _ = oracle.forest(codes, prm)
    ids0, sc0 = oracle.init_graph(codes, perm, lf, prm)
    steps = []
    ids, sc = ids0.copy(), sc0.copy()
    for _ in range(3):
        up = oracle.join_iter(codes, sk, ids, sc, prm)
        steps.append((up, ids.copy(), sc.copy()))
    return codes, sk, ids0, sc0, steps


@pytest.mark.parametrize("ctas,cblock", VARIANTS)
def test_join_variant_iterations_bit_exact(env, iter_case, ctas, cblock):
    torch, knng = env
    codes_h, sk_h, ids0, sc0, steps = iter_case
    codes = torch.from_numpy(codes_h).cuda()
    sk = torch.from_numpy(sk_h.view(np.int64)).cuda()
    ids = torch.from_numpy(ids0.copy()).cuda()
    sc = torch.from_numpy(sc0.copy()).cuda()
    with knng.Context(join_ctas_per_sm=ctas, join_cblock=cblock) as ctx:
        for it, (up_ref, ids_ref, sc_ref) in enumerate(steps):
            ids, sc, up = ctx.join_iter(codes, sk, ids, sc)
            assert up == up_ref, f"iteration {it}"
            np.testing.assert_array_equal(sc.cpu().numpy(), sc_ref)
            np.testing.assert_array_equal(ids.cpu().numpy(), ids_ref)


@pytest.fixture(scope="module")
def build_case(env):
    torch, knng = env
    n, d = 16000, 1024
    x = synth.mixture(n, d, 160, seed=77)
    codes_h, sk_h = oracle.quantize(x)
    codes = torch.from_numpy(codes_h).cuda()
    with knng.Context() as ctx:  # the build's own forest and initial graph (native pivots)
        perm, lf = ctx.forest(codes)
        ids0, sc0 = ctx.init_graph(codes, perm, lf)
    ids0, sc0 = ids0.cpu().numpy(), sc0.cpu().numpy()
    ids_ref, sc_ref = oracle.init_graph(codes_h, perm.cpu().numpy(), lf.cpu().numpy(), _stable())
    np.testing.assert_array_equal(ids0, ids_ref)
    np.testing.assert_array_equal(sc0, sc_ref)
    ref = _oracle_from_init(codes_h, sk_h, ids0, sc0, _stable())
    assert ref[2] >= 3  # enough iterations for the cache to serve most candidates
    return x, ref


@pytest.mark.parametrize("ctas,cblock", VARIANTS)
def test_build_variant_with_cache_bit_exact(env, build_case, ctas, cblock):
    torch, knng = env
    x, (k_ref, d_ref, it_ref, ups_ref) = build_case
    with knng.Context(join_ctas_per_sm=ctas, join_cblock=cblock, join_cache=1) as ctx:
        st = knng.Stats()
        k, dd, _ = ctx.build(x, None, None, st)
    assert st.join_ctas_per_sm == ctas and st.join_cblock == cblock
    assert st.iterations == it_ref
    assert list(st.updates[: st.iterations]) == ups_ref
    # every row counts as changed before the first iteration; later, rows whose
    # inputs did not change are copied through
    assert st.join_skipped[0] == 0
    assert sum(st.join_skipped[: st.iterations]) > 0
    np.testing.assert_array_equal(k, k_ref)
    np.testing.assert_array_equal(dd, d_ref)


def test_forced_variant_rejects_bad_values(env):
    _, knng = env
    for ctas, cb in [(5, 4), (4, 3), (2, 2)]:
        with pytest.raises(knng.KnngError) as e:
            knng.Context(join_ctas_per_sm=ctas, join_cblock=cb)
        assert e.value.status == -1
