"""Host memory in and out of knng_build.

Rows and results may live in pageable host memory (numpy, std::vector), in
pinned host memory or on the device.  Pageable memory goes through the
context's pinned buffers, copied by host threads in chunks of 65,536 rows, so
the test uses several chunks and a ragged last one; every form must give the
same graph bit for bit."""
import numpy as np
import pytest

import synth


@pytest.mark.gpu
def test_pageable_pinned_and_device_rows_give_the_same_graph():
    import torch

    import knng

    n, d = 150_000, 1024  # chunks of 65,536 + 65,536 + 18,928 rows
    x = synth.mixture(n, d, 1500, seed=77)
    prm = knng.params(max_iterations=2)
    with knng.Context(prm) as ctx:
        k_page, d_page, _ = ctx.build(x)  # pageable in, pageable out
        xd = torch.from_numpy(x).cuda()
        k_dev, d_dev, _ = ctx.build(xd)  # device in, device out
        xp = torch.from_numpy(x).pin_memory()
        kp = torch.empty((n, prm.k_eval), dtype=torch.int32).pin_memory()
        dp = torch.empty((n, prm.k_eval), dtype=torch.float32).pin_memory()
        ctx.build(xp, kp, dp)  # pinned in, pinned out
        k_mix = np.full((n, prm.k_eval), -7, np.int32)
        d_mix = np.full((n, prm.k_eval), -7, np.float32)
        ctx.build(xp.numpy(), k_mix, d_mix)  # pinned in, pageable out
        k_pg2, d_pg2, _ = ctx.build(x)  # pageable again: the slots are reused
    np.testing.assert_array_equal(k_page, k_dev.cpu().numpy())
    np.testing.assert_array_equal(d_page, d_dev.cpu().numpy())
    np.testing.assert_array_equal(k_page, kp.numpy())
    np.testing.assert_array_equal(d_page, dp.numpy())
    np.testing.assert_array_equal(k_page, k_mix)
    np.testing.assert_array_equal(d_page, d_mix)
    np.testing.assert_array_equal(k_page, k_pg2)
    np.testing.assert_array_equal(d_page, d_pg2)
    assert k_page.min() >= 1 and k_page.max() <= n


@pytest.mark.gpu
def test_batch_with_pageable_rows_equals_plain_builds():
    import knng

    xs = [synth.mixture(n, d, max(1, n // 100), seed=80 + j)
          for j, (n, d) in enumerate([(70_000, 768), (3_000, 1024), (66_000, 1024)])]
    prm = knng.params(max_iterations=2)
    with knng.Context(prm) as ctx:
        res, _ = ctx.build_batch(xs)
        for x, (k, dd, _) in zip(xs, res):
            k1, d1, _ = ctx.build(x)
            np.testing.assert_array_equal(k, k1)
            np.testing.assert_array_equal(dd, d1)


@pytest.mark.gpu
def test_device_rows_passed_as_host_rows_are_read_in_place():
    """A caller that passes device memory with rows_on_device = 0 gets the same
    graph as with the flag set: the library looks at the pointer and reads
    device rows in place instead of copying them as host memory."""
    import ctypes as C

    import torch

    import knng

    n, d = 20_000, 1024
    x = synth.mixture(n, d, 200, seed=78)
    xd = torch.from_numpy(x).cuda()
    prm = knng.params(max_iterations=2)
    with knng.Context(prm) as ctx:
        k_ref, d_ref, _ = ctx.build(x)
        k_out = np.empty((n, prm.k_eval), np.int32)
        d_out = np.empty((n, prm.k_eval), np.float32)
        torch.cuda.synchronize()
        st = knng.Stats()
        rc = knng.lib().knng_build(ctx.h, C.c_void_p(xd.data_ptr()), n, d, 0, k_out.ctypes.data_as(C.c_void_p),
                                   d_out.ctypes.data_as(C.c_void_p), 0, C.byref(st))
    assert rc == 0
    np.testing.assert_array_equal(k_out, k_ref)
    np.testing.assert_array_equal(d_out, d_ref)
