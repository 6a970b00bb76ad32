"""The serving loop (knng_server): jobs submitted while others run are admitted
by memory footprint, batched and overlapped on the device, and each result is
the same as the job built alone (bit for bit: the batch keeps per-job pivots,
fills and early stop, and the update is double-buffered)."""
import threading
import time

import numpy as np
import pytest

import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def knng_mod():
    import torch

    assert torch.cuda.is_available(), "the gpu tests need a CUDA device"
    import knng

    knng.lib()
    return knng


def test_served_results_equal_alone(knng_mod):
    import torch

    knng = knng_mod
    specs = [(20000, 1024, 200), (3000, 1024, 30), (9000, 1024, 900), (500, 1024, 5), (15000, 1024, 150),
             (7000, 1024, 70), (1200, 1024, 12), (30000, 1024, 300)]
    xs = [synth.mixture(n, d, c, seed=300 + k) for k, (n, d, c) in enumerate(specs)]
    with knng.Context() as ctx:
        solo = [ctx.build(x)[:2] for x in xs]
    dev_x = {k: torch.from_numpy(x).cuda() for k, x in enumerate(xs) if k % 2}
    with knng.Server(slots=1) as sv:
        # all arrive while the first build runs on the single slot: they are
        # admitted together as the next batch; half the inputs are on the device
        tickets = [sv.submit(dev_x.get(k, x)) for k, x in enumerate(xs)]
        outs = [sv.wait(t) for t in tickets]
    batched = 0
    for (k, dd, r), (ks, ds) in zip(outs, solo):
        assert r.status == 0 and r.latency_s >= r.run_s >= 0
        batched += r.batch_jobs > 1
        k = k.cpu().numpy() if hasattr(k, "cpu") else k
        dd = dd.cpu().numpy() if hasattr(dd, "cpu") else dd
        np.testing.assert_array_equal(k, ks)
        np.testing.assert_array_equal(dd, ds)
    assert batched > 0  # jobs that arrived while a batch ran were batched together


def test_admission_by_footprint(knng_mod):
    knng = knng_mod
    big = synth.mixture(60000, 1024, 600, seed=9)
    small = synth.mixture(2000, 1024, 20, seed=10)
    budget_gb = 1.5 * knng.lib().knng_footprint_bytes(None, 2000, 1024, 0) / 1e9
    with knng.Server(slots=1, mem_budget_gb=budget_gb) as sv:
        tb = sv.submit(big)
        ts = sv.submit(small)
        _, _, rb = sv.wait(tb)
        ks, ds, rs = sv.wait(ts)
    assert rb.status == -4  # larger than the whole budget: refused
    assert rs.status == 0 and ks.min() >= 1


def test_poll_and_concurrent_submitters(knng_mod):
    knng = knng_mod
    xs = [synth.mixture(4000, 768, 40, seed=20 + k) for k in range(6)]
    with knng.Context() as ctx:
        solo = [ctx.build(x)[:2] for x in xs]
    with knng.Server(slots=3) as sv:
        tickets = [None] * len(xs)

        def submit(k):
            tickets[k] = sv.submit(xs[k])

        ths = [threading.Thread(target=submit, args=(k,)) for k in range(len(xs))]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        done = {}
        deadline = time.time() + 120
        while len(done) < len(xs) and time.time() < deadline:
            for k, t in enumerate(tickets):
                if k not in done:
                    r = sv.poll(t)
                    if r is not None:
                        done[k] = r
            time.sleep(0.005)
    assert len(done) == len(xs)
    for k, (kn, dd, r) in done.items():
        np.testing.assert_array_equal(kn, solo[k][0])
        np.testing.assert_array_equal(dd, solo[k][1])


def test_admission_backfills_past_a_job_that_does_not_fit(knng_mod):
    """Two slots; a long job runs; the next queued job needs the whole budget,
    so it must wait for the memory to free up, and a small job queued behind it
    is admitted on the idle slot meanwhile instead of waiting behind it."""
    knng = knng_mod
    fp = knng.lib().knng_footprint_bytes
    first = synth.mixture(40000, 1024, 400, seed=41)   # runs first, on slot 0
    big = synth.mixture(60000, 1024, 600, seed=42)     # fits only when nothing else runs
    small = synth.mixture(1500, 1024, 15, seed=43)     # fits next to the first job
    b_big, b_first, b_small = fp(None, 60000, 1024, 0), fp(None, 40000, 1024, 0), fp(None, 1500, 1024, 0)
    budget = b_big + 1  # the big job runs alone; the first and the small job fit together
    assert b_first + b_small <= budget and b_small + b_big > budget
    with knng.Context() as ctx:
        solo_small = ctx.build(small)[:2]
    with knng.Server(slots=2, mem_budget_gb=budget / 1e9) as sv:
        t0 = time.perf_counter()
        tf = sv.submit(first)
        time.sleep(0.05)  # the first job is admitted and running
        tb = sv.submit(big)
        t_big = time.perf_counter()
        ts = sv.submit(small)
        t_small = time.perf_counter()
        _, _, rf = sv.wait(tf)
        _, _, rb = sv.wait(tb)
        ks, ds, rs = sv.wait(ts)
    assert rf.status == rb.status == rs.status == 0
    big_start = t_big + rb.queued_s
    small_done = t_small + rs.latency_s
    assert small_done <= big_start + 1e-3, (small_done - t0, big_start - t0)
    np.testing.assert_array_equal(ks, solo_small[0])
    np.testing.assert_array_equal(ds, solo_small[1])
