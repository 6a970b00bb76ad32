"""The optional 128-bit random-hyperplane sketch mode, CUDA against the oracle.

src/main.cpp keeps one sign bit per coordinate; its README describes 128-bit
random-hyperplane sketches (README.md:33-34).  That variant is built as
sketch_mode = KNNG_SKETCH_HYPERPLANE and, since the reference has no code for
it, pinned to the oracle's restatement (itself checked against numpy in
tests/test_oracle_hyperplane.py):

* the sketch kernel, bit for bit, at every supported d and at code extremes;
* NN-Descent iterations scoring the 2-word sketches, bit for bit;
* a whole build in that mode from the GPU's own initial graph, bit for bit
  through the reference's early stop and export.
"""
import os

import numpy as np
import pytest

import oracle
import synth

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def env():
    import torch

    assert torch.cuda.is_available(), "the gpu tests need a CUDA device"
    import knng

    knng.lib()
    return torch, knng


def _stable(**kw):
    return oracle.params(threads=THREADS, tie_mode=oracle.TIE_STABLE, jacobi=1, **kw)


@pytest.mark.parametrize("n,d,seed", [(1000, 1024, 1337), (777, 384, 5), (130, 128, 99), (64, 768, 1)])
def test_hyperplane_sketch_bit_exact(env, n, d, seed):
    torch, knng = env
    x = synth.mixture(n, d, max(1, n // 50), seed=n)
    codes, _ = oracle.quantize(x)
    codes[: n // 10] = -128
    codes[n // 10: n // 5] = 127
    codes[n // 5: n // 5 + 3] = 0
    ref = oracle.hyperplane_sketch(codes, seed)
    sk = knng.sketch_hyperplane(torch.from_numpy(codes).cuda(), seed)
    np.testing.assert_array_equal(sk.cpu().numpy().view(np.uint64), ref)


def test_hyperplane_join_iterations_bit_exact(env):
    torch, knng = env
    n, d = 6000, 1024
    x = synth.mixture(n, d, 600, seed=8)
    codes_h, _ = oracle.quantize(x)
    sk_h = oracle.hyperplane_sketch(codes_h)
    prm = _stable(sketch_mode=1)
    perm, lf, _ = oracle.forest(codes_h, prm)
    ids_ref, sc_ref = oracle.init_graph(codes_h, perm, lf, prm)
    codes = torch.from_numpy(codes_h).cuda()
    sk = torch.from_numpy(sk_h.view(np.int64)).cuda()
    ids = torch.from_numpy(ids_ref.copy()).cuda()
    sc = torch.from_numpy(sc_ref.copy()).cuda()
    with knng.Context(sketch_mode=knng.SKETCH_HYPERPLANE) as ctx:
        for it in range(3):
            up_ref = oracle.join_iter(codes_h, sk_h, ids_ref, sc_ref, prm)
            ids, sc, up = ctx.join_iter(codes, sk, ids, sc)
            assert up == up_ref, f"iteration {it}"
            np.testing.assert_array_equal(sc.cpu().numpy(), sc_ref)
            np.testing.assert_array_equal(ids.cpu().numpy(), ids_ref)


def test_hyperplane_build_bit_exact_from_gpu_init(env):
    torch, knng = env
    n, d = 12000, 768
    x = synth.mixture(n, d, 120, seed=9)
    codes_h, _ = oracle.quantize(x)
    codes = torch.from_numpy(codes_h).cuda()
    with knng.Context(sketch_mode=knng.SKETCH_HYPERPLANE) as ctx:
        perm, lf = ctx.forest(codes)
        ids0, sc0 = ctx.init_graph(codes, perm, lf)
        st = knng.Stats()
        k, dd, _ = ctx.build(x, None, None, st)
    ids, sc = ids0.cpu().numpy(), sc0.cpu().numpy()
    prm = _stable(sketch_mode=1)
    sk_h = oracle.hyperplane_sketch(codes_h)
    prev, it, ups = np.float32(1.0), 0, []
    for it in range(30):
        up = oracle.join_iter(codes_h, sk_h, ids, sc, prm)
        ups.append(up)
        rate = np.float32(up) / np.float32(n * 50)
        if rate < np.float32(0.04) or (it > 0 and (prev - rate) < np.float32(0.01)):
            it += 1
            break
        prev = rate
    kr, dr = oracle.export(ids, sc)
    assert st.iterations == it and list(st.updates[:it]) == ups
    np.testing.assert_array_equal(k, kr)
    np.testing.assert_array_equal(dd, dr)
