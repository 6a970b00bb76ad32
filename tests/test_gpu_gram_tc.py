"""The tcgen05 (f16 tensor-core) leaf Gram against the dp4a one and the oracle.

int8 codes are exact in f16 and every partial sum of a Gram entry is an
integer of magnitude <= d * 128^2 <= 2^24, exact in fp32, so the tensor-core
Gram must reproduce the int32 dots bit for bit -- including rows of extreme
codes (all -128: dot = 1024 * 16384 = 2^24 exactly) and leaves of every size.
"""
import numpy as np
import pytest

import oracle
import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def knng_mod():
    import torch

    assert torch.cuda.is_available(), "the gpu tests need a CUDA device"
    import knng

    knng.lib()
    return knng


def _extreme_rows(n, d, seed):
    rng = np.random.default_rng(seed)
    x = rng.choice(np.array([-2.0, 2.0, -1.0, 1.0, 0.0, 0.5 / 127], np.float32), size=(n, d))
    x[: n // 8] = -2.0  # codes -128 everywhere
    x[n // 8: n // 4] = 2.0  # codes 127 everywhere
    return x.astype(np.float32)


@pytest.mark.parametrize("n,d,kind", [(3000, 1024, "mix"), (5000, 384, "mix"), (2500, 768, "mix"),
                                      (700, 1024, "extreme"), (900, 128, "extreme"), (37, 1024, "mix")])
def test_tc_init_graph_bit_exact(knng_mod, n, d, kind):
    import torch

    knng = knng_mod
    x = synth.mixture(n, d, max(1, n // 100), seed=n + d) if kind == "mix" else _extreme_rows(n, d, n)
    codes_ref, _ = oracle.quantize(x)
    prm = oracle.params(threads=1, tie_mode=oracle.TIE_STABLE, jacobi=1)
    perm_ref, lf_ref, _ = oracle.forest(codes_ref, prm)
    ids_ref, sc_ref = oracle.init_graph(codes_ref, perm_ref, lf_ref, prm)
    codes = torch.from_numpy(codes_ref).cuda()
    with knng.Context(gram_mode=knng.GRAM_TCGEN05) as ctx:
        ids, sc = ctx.init_graph(codes, torch.from_numpy(perm_ref).cuda(), torch.from_numpy(lf_ref).cuda())
    np.testing.assert_array_equal(sc.cpu().numpy(), sc_ref)
    np.testing.assert_array_equal(ids.cpu().numpy(), ids_ref)


def test_tc_full_build_equals_dp4a(knng_mod):
    knng = knng_mod
    x = synth.mixture(30000, 1024, 300, seed=77)
    with knng.Context(gram_mode=knng.GRAM_DP4A) as a, knng.Context(gram_mode=knng.GRAM_TCGEN05) as b:
        ka, da, sa = a.build(x)
        kb, db, sb = b.build(x)
    np.testing.assert_array_equal(ka, kb)
    np.testing.assert_array_equal(da, db)
    assert sa.iterations == sb.iterations


@pytest.mark.parametrize("d", [1024, 256])
def test_tc_wait_timeout_reports_and_context_recovers(knng_mod, d):
    """The tensor-core Gram's mbarrier waits are bounded.  With the limit set to
    give up at once every wait for tensor-core work fails (d = 1024: in the
    staging loop, d = 256: at the end of each tile); the kernel flags the
    timeout, the whole block stops, the committed MMAs are drained with the
    full limit and tensor memory is freed.  The call returns KNNG_E_TIMEOUT,
    and builds afterwards -- in a new context and in the same process -- are
    exact again."""
    import torch

    knng = knng_mod
    x = synth.mixture(3000, d, 30, seed=91)
    codes_ref, _ = oracle.quantize(x)
    prm = oracle.params(threads=1, tie_mode=oracle.TIE_STABLE, jacobi=1)
    perm_ref, lf_ref, _ = oracle.forest(codes_ref, prm)
    ids_ref, sc_ref = oracle.init_graph(codes_ref, perm_ref, lf_ref, prm)
    codes = torch.from_numpy(codes_ref).cuda()
    perm, lf = torch.from_numpy(perm_ref).cuda(), torch.from_numpy(lf_ref).cuda()
    with knng.Context(gram_mode=knng.GRAM_TCGEN05, wait_limit=-1) as ctx:
        with pytest.raises(knng.KnngError) as e:
            ctx.init_graph(codes, perm, lf)
        assert e.value.status == -5  # KNNG_E_TIMEOUT
        with pytest.raises(knng.KnngError) as e2:
            ctx.build(x)
        assert e2.value.status == -5
    torch.cuda.synchronize()  # the device is still usable
    with knng.Context(gram_mode=knng.GRAM_TCGEN05) as ctx:
        ids, sc = ctx.init_graph(codes, perm, lf)
        np.testing.assert_array_equal(sc.cpu().numpy(), sc_ref)
        np.testing.assert_array_equal(ids.cpu().numpy(), ids_ref)
        k, dd, st = ctx.build(x)
        assert st.iterations >= 1 and k.min() >= 1
