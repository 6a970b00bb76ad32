"""Throughput of the GB300 kNN-graph build (vectors/s) on synthetic SISAP-shaped data.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config full|1m|small]
    python bench.py --impl reference ...     # the reference's CPU path: its binary where it
                                             # runs (x86, built here), else the oracle port

A step is one whole graph build of one synthetic dataset (quantise, RP forest,
leaf init, NN-Descent to the reference's early stop, export): the stages
Aftab5550/SISAP-2026-task1 src/main.cpp:179-457 runs.  `value` is vectors/s
with the float32 rows already in HBM (device-timed with CUDA events on the
library's stream); `e2e` is the same build through knng_build with pinned host
rows in and host knns/dists out, timed by a host wall clock around the call,
so the copies and the host-side set-up are inside the timed region.  The inputs
(26 GB at 6.35M x 1024) are far larger than L2, so no flush is needed.

At N = 1 the line also carries `batched` (64 independent jobs in one
knng_build_batch call against the same jobs built one after another) and
`serving` (Poisson arrivals through the serving loop: jobs/s, p50/p99
latency); `--config batched|serving` prints either as a line of its own.

Several GPUs run independent replicas (the build does not shard): each rank
builds its own dataset of the configured size; value = all ranks' vectors /
max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "sisap-2026-task1_gb300")
sys.path.insert(0, PKG)

CONFIGS = {
    # name: (n, d, centres, description)
    "full": (6_350_000, 1024, 50_000, "full-scale single build 6.35M x 1024, 50k centres"),
    "1m": (1_000_000, 1024, 10_000, "single build 1M x 1024, 10k centres"),
    "300k": (300_000, 1024, 3_000, "profiling case 300k x 1024, 3k centres (codes+sketches 0.34 GB > L2)"),
    "small": (100_000, 1024, 1_000, "plain small 100k x 1024, 1k centres"),
}
CPU_SAMPLE = (100_000, 1024, 1_000)  # bounded CPU sample (the 100k small config), ~10-30 s of CPU work
METRIC = "vectors/s (kNN-graph build, recall@15-checked)"
GRAM = {"dp4a": 0, "tc": 1}
# DRAM read + write bytes per row of one working NN-Descent launch: the mean
# over the working join launches of one 300k x 1024 build (3k centres), from
# the one-pass ncu capture summarised in profiles/join_kernel_dram_300k.md.
JOIN_DRAM_BYTES_PER_ROW_300K = 22251.0
JOIN_TRAFFIC_SOURCE = ("profiles/join_kernel_dram_300k.md: mean DRAM bytes per row of a 300k build's working "
                       "join launches (ncu), times this workload's rows")


def workload_config(name, ws, prm=None):
    """The `config` object both arms print: the workload and the reference-default
    algorithm parameters it is built with (src/main.cpp:19-29), nothing about
    either implementation, so the two lines name the same configuration."""
    n, d, centres, desc = CONFIGS[name]
    p = {"k": 15, "k_build": 50, "trees": 16, "leaf": 64, "rerank": 8}
    if prm is not None:
        p = {"k": prm.k_eval, "k_build": prm.k_build, "trees": prm.num_trees, "leaf": prm.leaf_size,
             "rerank": prm.rerank_mult}
    return {"workload": desc, "n": n, "d": d, "centres": centres, **p,
            "l2": "inputs (n x d float32) far larger than L2; no flush", "parallelism": f"replicas x{ws}"}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Group:
    """Barrier and max-over-ranks for N independent replicas (no data-path collective)."""

    def __init__(self, backend):
        self.ws, self.rank, self.local = dist_env()
        self.dist = None
        if self.ws > 1:
            import torch.distributed as dist

            dist.init_process_group(backend=backend)
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, v, device=None):
        if not self.dist:
            return v
        import torch

        t = torch.tensor([float(v)], dtype=torch.float64, device=device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


def recall_sample(x, knns, rows=10_000, seed=7):
    """recall@15 of exported knns on a seeded row sample vs exact fp64 brute force (GPU)."""
    import torch

    import evaluate
    import synth

    n = x.shape[0]
    g = torch.Generator().manual_seed(seed)
    idx = torch.randperm(n, generator=g)[: min(rows, n)].numpy()
    gt = evaluate.sample_knn(x, idx, 15)
    kh = knns.cpu().numpy() if hasattr(knns, "cpu") else knns
    return synth.recall_at_k(kh, gt, rows=idx)


def cpu_port_step(threads, sample=CPU_SAMPLE, seed=4242, want=False):
    """One reference-algorithm build (oracle port, OpenMP, reference tie rules and
    in-place race) on the bounded sample; returns (s, n[, x, knns])."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    import synth

    n, d, c = sample
    x = synth.mixture(n, d, c, seed=seed)
    prm = oracle.params(threads=threads)
    t0 = time.perf_counter()
    knns, _, _ = oracle.build_graph(x, prm)
    el = time.perf_counter() - t0
    return (el, n, x, knns) if want else (el, n)


def recall_parity(x_np, ref_knns, dev):
    """recall@15 (all rows, exact fp64) of the reference port's graph and of the
    GPU build of the same rows: the parity measure (recall@15 within 0.5 pt)."""
    import torch

    import knng

    x = torch.from_numpy(x_np).to(dev)
    with knng.Context() as ctx:
        kg, _, _ = ctx.build(x)
    r_ref = recall_sample(x, torch.from_numpy(ref_knns), rows=x.shape[0])
    r_gpu = recall_sample(x, kg, rows=x.shape[0])
    return {"n": int(x.shape[0]), "reference_port": r_ref, "gpu": r_gpu, "gap_pt": 100 * (r_ref - r_gpu)}


def same_sample_gpu(dev, steps, warmup, sample=CPU_SAMPLE, seed=4242):
    """The GPU build timed on exactly the rows the reference arm builds (the
    bounded CPU sample: same generator, size and seed): device-resident
    vectors/s and, through knng_build with pinned host rows in and host
    knns/dists out, end-to-end vectors/s.  Same N on both sides, so the ratio
    to the reference arm is like for like."""
    import torch

    import knng
    import synth

    n, d, c = sample
    xh_np = synth.mixture(n, d, c, seed=seed)
    x = torch.from_numpy(xh_np).to(dev)
    xh = torch.from_numpy(xh_np).pin_memory()
    kh = torch.empty((n, 15), dtype=torch.int32, pin_memory=True)
    dh = torch.empty((n, 15), dtype=torch.float32, pin_memory=True)
    dev_s, e2e_s = [], []
    with knng.Context() as ctx:
        for _ in range(warmup):
            ctx.build(x)
            ctx.build(xh, kh, dh)
        for _ in range(steps):
            st = knng.Stats()
            ctx.build(x, None, None, st)
            dev_s.append(st.device_s)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ctx.build(xh, kh, dh)  # returns once the host outputs are written
            e2e_s.append(time.perf_counter() - t0)
    return {"value": n / statistics.mean(dev_s), "e2e": n / statistics.mean(e2e_s), "unit": "vectors/s",
            "sample": f"{n} x {d} rows, {c} centres, seed {seed}: the reference arm's own sample", "steps": steps}


def reference_recall_same_rows(x, knns, rows):
    """The reference algorithm (the oracle's restatement of src/main.cpp, its
    own tie rules and in-place race, every host thread) on exactly the rows the
    GPU built: recall@15 of both graphs on the same seeded sample against exact
    float64 brute force, and the CPU build time."""
    import torch

    import evaluate
    import synth

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    threads = os.cpu_count() or 1
    xh = x.cpu().numpy()
    t0 = time.perf_counter()
    kr, _, st = oracle.build_graph(xh, oracle.params(threads=threads))
    cpu_s = time.perf_counter() - t0
    del xh
    n = x.shape[0]
    idx = torch.randperm(n, generator=torch.Generator().manual_seed(7))[: min(rows, n)].numpy()
    gt = evaluate.sample_knn(x, idx, 15)
    r_ref = synth.recall_at_k(kr, gt, rows=idx)
    r_gpu = synth.recall_at_k(knns.cpu().numpy(), gt, rows=idx)
    return {"n": int(n), "sample_rows": int(len(idx)), "reference_port": r_ref, "gpu": r_gpu,
            "gap_pt": 100 * (r_ref - r_gpu), "reference_iterations": int(st.iterations),
            "reference_build_s": float(st.build_s), "reference_wall_s": cpu_s, "threads": threads}


def cpu_ref_step(threads, sample=CPU_SAMPLE, seed=4242):
    """One build by the unmodified reference binary (oracle/_ref/main: src/main.cpp
    compiled with its own flags against the container-file H5Cpp shim) on the
    bounded sample; returns (buildtime s, process wall s, n), or None when the
    binary is absent or cannot run on this host."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    import synth

    n, d, c = sample
    if oracle.ref_binary(d) is None:
        return None
    x = synth.mixture(n, d, c, seed=seed)
    t0 = time.perf_counter()
    try:
        _, _, attrs, _ = oracle.run_reference(x, threads=threads)
    except (OSError, subprocess.CalledProcessError):
        return None  # e.g. an x86 build on an Arm host
    wall = time.perf_counter() - t0
    # buildtime: src/main.cpp's own timer, after quantisation to after NN-Descent
    return float(np.asarray(attrs["buildtime"]).reshape(-1)[0]), wall, n


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    cfg_name = args.config if args.config in CONFIGS else "full"
    sample = (f"bounded sample of the workload: {CPU_SAMPLE[0]} x {CPU_SAMPLE[1]} rows, {CPU_SAMPLE[2]} centres, "
              "same generator; one whole build per step")
    kind, times, walls = "reference", [], []
    for k in range(args.warmup + args.steps):
        r = cpu_ref_step(threads, CPU_SAMPLE)
        if r is None:
            kind = "port"
            break
        if k >= args.warmup:
            times.append(r[0])
            walls.append(r[1])
    if kind == "port":
        times = []
        for k in range(args.warmup + args.steps):
            s, _ = cpu_port_step(threads, CPU_SAMPLE)
            if k >= args.warmup:
                times.append(s)
        walls = times
    v = CPU_SAMPLE[0] / statistics.mean(times)
    if kind == "reference":
        note = ("the unmodified reference binary (oracle/_ref/main, src/main.cpp with its own flags) with "
                "OMP_NUM_THREADS = all host threads; value from its buildtime attribute")
    else:
        note = ("oracle/_ref is an x86 build of the reference made where its sources are, so it is absent or "
                "cannot run on this host; its restatement (oracle/knng_oracle.cpp, pinned bit-exact to the "
                "reference binary) runs with OpenMP")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "vectors/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int8/int32",
        "data": "synthetic", "config": workload_config(cfg_name, ws),
        "cpu_baseline": {"value": v, "unit": "vectors/s", "cores": threads, "kind": kind, "sample": sample},
        "e2e": {"value": v, "unit": "vectors/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "process_wall_s": statistics.mean(walls),
        "note": note,
    }
    print(json.dumps(line), flush=True)
    return 0


def _job_specs(count, lo, hi, dims, seed):
    """Seeded (n, d) of `count` jobs: n log-uniform in [lo, hi], d drawn from dims."""
    import numpy as np

    rng = np.random.Generator(np.random.PCG64(seed))
    ns = np.exp(rng.uniform(np.log(lo), np.log(hi), size=count)).astype(np.int64)
    ds = rng.choice(np.asarray(dims), size=count)
    return [(int(n), int(d)) for n, d in zip(ns, ds)]


def measure_batched(steps, warmup, seq_passes):
    """64 independent jobs (n log-uniform in [5k, 200k], d in {384, 768, 1024}):
    one knng_build_batch call per step against the same jobs as 64 plain
    knng_build calls one after another.  jobs/s of both forms by the host wall
    clock around the calls (what a caller waits for: host set-up, launches and
    the device work); the device-event spans are reported beside them.  Every
    job's output is checked bit-identical between the two."""
    import torch

    import knng
    import synth

    dev = torch.device("cuda", 0)
    specs = _job_specs(64, 5_000, 200_000, (384, 768, 1024), seed=4003)
    xs = [synth.mixture_torch(n, d, max(1, n // 100), seed=4000 + j, device=dev) for j, (n, d) in enumerate(specs)]
    torch.cuda.synchronize()
    rows = sum(n for n, _ in specs)
    with knng.Context() as ctx:
        for _ in range(warmup):
            res, _ = ctx.build_batch(xs)
        bt, bw = [], []
        launches = 0
        stages = ("quantize_s", "forest_s", "init_s", "join_s", "export_s")
        with ClockSampler(0) as clk:
            for _ in range(steps):
                st = knng.Stats()
                t0 = time.perf_counter()
                res, st = ctx.build_batch(xs, st)
                bw.append(time.perf_counter() - t0)
                bt.append(st.device_s)
                launches += st.kernel_launches
        b_stage = {k[:-2]: getattr(st, k) for k in stages}  # summed over the batch's dimension groups
        for x in xs:
            ctx.build(x)  # warm the plain path too (autotune buckets, buffers)
        seq, seq_w = [], []
        same = True
        s_stage = {}
        outs = []
        for _ in range(seq_passes):
            tot = 0.0
            s_stage = {k[:-2]: 0.0 for k in stages}
            outs = []
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for j, x in enumerate(xs):
                k, d_, st1 = ctx.build(x)
                outs.append((k, d_))
                tot += st1.device_s
                for k2 in stages:
                    s_stage[k2[:-2]] += getattr(st1, k2)
            seq_w.append(time.perf_counter() - t0)
            seq.append(tot)
        for j, (k, d_) in enumerate(outs):  # compared outside the timed loop
            same &= bool(torch.equal(k, res[j][0]) and torch.equal(d_, res[j][1]))
    del xs
    torch.cuda.empty_cache()
    b_js = 64 / statistics.mean(bw)
    s_js = 64 / statistics.mean(seq_w)
    return {"workload": "64 jobs, n log-uniform [5k, 200k], d in {384, 768, 1024}", "rows": rows,
            "jobs_per_s": b_js, "ms_per_step": 1e3 * statistics.mean(bw), "steps": steps,
            "sequential_plain_jobs_per_s": s_js, "batched_over_sequential": b_js / s_js,
            "timer": "host wall clock around the calls",
            "device_span": {"batched_jobs_per_s": 64 / statistics.mean(bt),
                            "sequential_jobs_per_s": 64 / statistics.mean(seq),
                            "batched_over_sequential": statistics.mean(seq) / statistics.mean(bt)},
            "identical_to_plain": same, "vectors_per_s": rows / statistics.mean(bw), "clocks": clk.summary(),
            "gpu_launches": launches,
            "stage_s": {"batched (sum over dimension groups, which run concurrently)": b_stage,
                        "sequential (sum over the 64 builds)": s_stage}}


def run_batched(args):
    b = measure_batched(args.steps, args.warmup, max(1, args.steps // 2))
    line = {"metric": "jobs/s (64 independent kNN-graph builds, batched)", "value": b["jobs_per_s"], "unit": "jobs/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": b["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int8/int32",
            "data": "synthetic (seeded Gaussian mixtures, one per job)",
            "config": {"workload": "batched builds: " + b["workload"], "rows": b["rows"],
                       "l2": "inputs far larger than L2"},
            "sequential_plain_jobs_per_s": b["sequential_plain_jobs_per_s"],
            "batched_over_sequential": b["batched_over_sequential"], "identical_to_plain": b["identical_to_plain"],
            "vectors_per_s": b["vectors_per_s"], "clocks": b["clocks"], "gpu_launches": b["gpu_launches"]}
    print(json.dumps(line), flush=True)
    return 0


def measure_serving(count, slots):
    """Poisson arrivals (mean 4 jobs/s) of builds with n log-uniform in [10k, 2M],
    d = 1024, rows resident in HBM; the server admits them by footprint against
    180 GB and batches them continuously.  Returns jobs/s and p50/p99 latency
    next to the same jobs built one after another."""
    import numpy as np
    import torch

    import knng
    import synth

    dev = torch.device("cuda", 0)
    specs = _job_specs(count, 10_000, 2_000_000, (1024,), seed=5003)
    xs = [synth.mixture_torch(n, d, max(1, n // 100), seed=5000 + j, device=dev) for j, (n, d) in enumerate(specs)]
    torch.cuda.synchronize()
    rng = np.random.Generator(np.random.PCG64(5))
    gaps = rng.exponential(1.0 / 4.0, size=count)
    with knng.Context() as ctx:  # warm-up + sequential reference
        ctx.build(xs[0])
        solo = {}
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for j, x in enumerate(xs):  # back to back, host wall clock
            k, d_, st = ctx.build(x)
            if j < 4:
                solo[j] = (k, d_)
        seq_s = time.perf_counter() - t0
    with knng.Server(slots=slots, mem_budget_gb=180.0) as sv:
        sv.wait(sv.submit(xs[0]))  # warm the workers
        tickets = [None] * count
        t0 = time.perf_counter()
        with ClockSampler(0) as clk:
            for j in range(count):
                time.sleep(gaps[j])
                tickets[j] = sv.submit(xs[j])
            outs = [sv.wait(t, 1200.0) for t in tickets]
            t_end = time.perf_counter()
    lat = sorted(r.latency_s for _, _, r in outs)
    mean_batch = float(np.mean([r.batch_jobs for _, _, r in outs]))
    same = all(torch.equal(outs[j][0], solo[j][0]) and torch.equal(outs[j][1], solo[j][1]) for j in solo)
    del xs, outs
    torch.cuda.empty_cache()
    return {"workload": f"{count} jobs, Poisson mean 4/s, n log-uniform [10k, 2M], d = 1024, 180 GB budget",
            "slots": slots, "rows": int(sum(n for n, _ in specs)), "arrival_span_s": float(np.sum(gaps)),
            "jobs_per_s": count / (t_end - t0), "wall_s": t_end - t0,
            "p50_latency_s": lat[len(lat) // 2], "p99_latency_s": lat[min(len(lat) - 1, int(0.99 * len(lat)))],
            "mean_batch_jobs": mean_batch, "sequential_plain_jobs_per_s": count / seq_s, "identical_to_plain": same,
            "clocks": clk.summary()}


def run_serving(args):
    sv = measure_serving(args.serve_jobs, args.slots)
    line = {"metric": "jobs/s (serving, Poisson 4 jobs/s, n log-uniform [10k, 2M])", "value": sv["jobs_per_s"],
            "unit": "jobs/s", "n_gpus": 1, "steps": 1, "warmup": 1, "ms_per_step": 1e3 * sv["wall_s"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int8/int32",
            "data": "synthetic (seeded Gaussian mixtures, one per job)",
            "config": {"workload": "serving loop: " + sv["workload"], "slots": sv["slots"], "rows": sv["rows"],
                       "arrival_span_s": sv["arrival_span_s"]},
            "p50_latency_s": sv["p50_latency_s"], "p99_latency_s": sv["p99_latency_s"],
            "mean_batch_jobs": sv["mean_batch_jobs"], "sequential_plain_jobs_per_s": sv["sequential_plain_jobs_per_s"],
            "identical_to_plain": sv["identical_to_plain"], "clocks": sv["clocks"]}
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    import torch

    import knng
    import synth

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    grp = Group("nccl" if ws > 1 else "gloo")
    n, d, centres, desc = CONFIGS[args.config]
    dev = torch.device("cuda", local)
    x = synth.mixture_torch(n, d, centres, seed=1000 * 2 + rank, device=dev)
    torch.cuda.synchronize()
    # the pinned host copy of the rows for the end-to-end leg, pinned up front as
    # a caller would (pinned late in the process, after the device work, the
    # quantise kernel read it at 93 GB/s instead of 112)
    xh = None
    if not args.skip_e2e:
        xh = torch.empty((n, d), dtype=torch.float32, pin_memory=True)
        xh.copy_(x)
    prm = knng.params(device=local, gram_mode=GRAM[args.gram], join_cache=args.join_cache,
                      forest_fuse=args.forest_fuse)
    ctx = knng.Context(prm)
    knns = torch.empty((n, prm.k_eval), dtype=torch.int32, device=dev)
    dists = torch.empty((n, prm.k_eval), dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        ctx.build(x, knns, dists)
    # ---- device-resident timed region
    stats = []
    grp.barrier()
    torch.cuda.synchronize()
    launches = 0
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            st = knng.Stats()
            ctx.build(x, knns, dists, st)
            stats.append(st)
            launches += st.kernel_launches
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    grp.barrier()
    dev_s = sum(s.device_s for s in stats)
    t_max = grp.max(dev_s, device=dev)
    ms_per_step = 1e3 * t_max / args.steps
    value = ws * n * args.steps / t_max
    # ---- end to end: pinned host rows in, host knns/dists out
    e2e = None
    if not args.skip_e2e:
        kh = torch.empty((n, prm.k_eval), dtype=torch.int32, pin_memory=True)
        dh = torch.empty((n, prm.k_eval), dtype=torch.float32, pin_memory=True)
        ctx.build(xh, kh, dh)  # warm the host-input path
        grp.barrier()
        torch.cuda.synchronize()
        # host wall clock around the public call: argument checks, buffer
        # set-up, the job table and every copy are inside it (knng_build
        # returns once the host outputs are written)
        t0 = time.perf_counter()
        e2e_dev = 0.0
        e2e_stats = []
        for _ in range(args.steps):
            st = knng.Stats()
            ctx.build(xh, kh, dh, st)
            e2e_dev += st.device_s
            e2e_stats.append(st)
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
        e2e_max = grp.max(e2e_s, device=dev)
        e2e = {"value": ws * n * args.steps / e2e_max, "unit": "vectors/s", "h2d_bytes_per_step": n * d * 4,
               "d2h_bytes_per_step": n * prm.k_eval * 8, "timer": "host wall clock around knng_build",
               "device_span_vectors_per_s": n * args.steps / e2e_dev,
               # quantize reads the pinned host rows over the host link; the
               # export stage includes the device-to-host copy of knns/dists
               "stage_s": {f: statistics.mean(getattr(q, f + "_s") for q in e2e_stats)
                           for f in ("quantize", "forest", "init", "join", "export")}}
        del xh
    # ---- roofline of the dominant kernel (NN-Descent join launches)
    # Algorithmic bytes per row of one iteration of the reference algorithm:
    # every one of the K*K two-hop candidates reads its id and its sketch,
    # R = K*rerank candidates are reranked against their d-byte rows (plus a
    # 4-byte id), and the row's list is read and written (K * 16).
    last = stats[-1]
    it = last.iterations
    join_ms = [last.join_ms[i] for i in range(it)]
    K = prm.k_build
    W8 = d // 8
    R = K * prm.rerank_mult
    row_alg = K * K * (4 + W8) + R * (d + 4) + K * 16
    # What the kernel itself moves (its own counters): distinct sketches scored
    # (deduplicated, candidate cache), reranked rows not known to be rejected,
    # the candidate cache read and write, lists and the own row.
    counted = []
    for i in range(it):
        rows_b = n * (K * 8 + K * K * 4 + d + W8 + K * 8)
        cache_b = 0
        if prm.join_cache:
            wr = min(last.join_distinct[i], 1536 * n)
            cache_b = 6 * (wr + (min(last.join_distinct[i - 1], 1536 * n) if i else 0))
        counted.append(rows_b + last.join_candidates[i] * W8 + last.join_dots[i] * d + cache_b)
    peak, peak_kind = load_peaks()
    secs = sum(join_ms) * 1e-3
    ms_launch = sum(join_ms) / max(1, it)
    # DRAM bytes actually moved per launch: the per-row mean of a 300k-row
    # build's working launches (ncu), times this workload's rows, unless the
    # caller passes a measured figure for this exact workload.
    if args.traffic_per_launch:
        traffic, t_src = args.traffic_per_launch, "--traffic-per-launch"
    else:
        traffic, t_src = JOIN_DRAM_BYTES_PER_ROW_300K * n, JOIN_TRAFFIC_SOURCE
    achieved = traffic / (ms_launch * 1e-3) / 1e9 if it else 0.0
    achieved_counted = sum(counted) / secs / 1e9 if it else 0.0
    nodedup_rate = n * row_alg * it / secs / 1e9 if it else 0.0
    roofline = {"kernel": "join_kernel (NN-Descent iteration)", "bound": "hbm", "achieved": achieved,
                "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "traffic_source": t_src, "ms_per_launch": ms_launch,
                "counted_bytes_per_launch": sum(counted) / max(1, it), "counted_achieved": achieved_counted,
                "counted_frac": achieved_counted / peak,
                "nodedup_bytes_per_launch": n * row_alg, "nodedup_bytes_per_row": row_alg,
                "nodedup_rate_over_peak": nodedup_rate / peak,
                "note": "achieved/frac: DRAM bytes moved per launch / launch time; counted_*: the bytes the "
                        "kernel's own counters say its algorithm must touch (distinct sketches scored, rows "
                        "reranked, lists, candidate cache); nodedup_*: every two-hop candidate's id and "
                        "sketch plus R rows per row, an upper bound the kernel avoids by deduplicating"}
    # ---- recall on a seeded sample
    rec = recall_sample(x, knns, rows=args.recall_rows) if args.recall_rows > 0 and rank == 0 else None
    # ---- the reference algorithm on these very rows (optional: minutes of CPU
    #      time at full size): recall@15 of both graphs on the same sample
    full_parity = None
    if args.reference_recall and rank == 0:
        full_parity = reference_recall_same_rows(x, knns, args.recall_rows)
    # ---- the same build on the reference arm's own sample rows (like-for-like N)
    # (part of the CPU-baseline leg: --skip-cpu leaves both out)
    same = same_sample_gpu(dev, args.steps, max(1, args.warmup)) if rank == 0 and ws == 1 and not args.skip_cpu else None
    # ---- CPU baseline (rank 0, N=1 only)
    cpu = None
    parity = None
    if rank == 0 and ws == 1 and not args.skip_cpu:
        threads = os.cpu_count() or 1
        s, ns, xs, ks = cpu_port_step(threads, want=True)
        parity = recall_parity(xs, ks, dev)
        cpu = {"value": ns / s, "unit": "vectors/s", "cores": threads, "kind": "port",
               "sample": f"{CPU_SAMPLE[0]} x {CPU_SAMPLE[1]} rows ({CPU_SAMPLE[2]} centres), one whole build, "
                         "oracle restatement of src/main.cpp with OpenMP"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "vectors/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int8/int32", "data": "synthetic (seeded Gaussian mixture, Zipf 1.1)",
            "config": workload_config(args.config, ws, prm),
            "implementation": {"join": "jacobi" if prm.join_mode == 0 else "inplace",
                               "leaf_gram": "tcgen05 f16" if prm.gram_mode == 1 else "dp4a",
                               "forest": "three levels per pass" if prm.forest_fuse else "one level per pass",
                               "candidate_cache": bool(prm.join_cache),
                               "join_tuned": {"ctas_per_sm": last.join_ctas_per_sm, "cblock": last.join_cblock,
                                              "cuda_graph": bool(last.graph_used)}},
            "build_s": last.build_s, "step_s": last.device_s, "iterations": it,
            "join_iterations": {"ms": [round(last.join_ms[i], 3) for i in range(it)],
                                "updates": [int(last.updates[i]) for i in range(it)],
                                "rows_skipped_unchanged": [int(last.join_skipped[i]) for i in range(it)],
                                "distinct_candidates": [int(last.join_distinct[i]) for i in range(it)],
                                "sketches_scored": [int(last.join_candidates[i]) for i in range(it)],
                                "rows_reranked": [int(last.join_dots[i]) for i in range(it)]},
            "stage_s": {"quantize": last.quantize_s, "forest": last.forest_s, "init": last.init_s,
                        "join": last.join_s, "export": last.export_s},
            "recall@15": rec, "recall_rows": args.recall_rows, "recall_parity_100k": parity,
            "value_same_config": same["value"] if same else None, "same_config": same,
            "recall_parity_same_rows": full_parity,
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
            "clocks": clk.summary(), "gpu_launches": launches, "wall_s": wall,
        }
    ctx.close()
    del x, knns, dists
    torch.cuda.empty_cache()
    # ---- the batched and served forms (one GPU: rank 0 at N = 1)
    if rank == 0 and ws == 1 and not args.skip_forms:
        line["batched"] = measure_batched(min(args.steps, 5), 2, 1)
        line["serving"] = measure_serving(args.serve_jobs, args.slots)
    if rank == 0:
        print(json.dumps(line), flush=True)
    grp.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--config", default="full", choices=sorted(CONFIGS) + ["batched", "serving"])
    ap.add_argument("--gram", default="tc", choices=["tc", "dp4a"],
                    help="leaf Gram: tcgen05 f16 tensor cores or dp4a")
    ap.add_argument("--join-cache", type=int, default=1, choices=[0, 1],
                    help="per-row candidate cache in the NN-Descent join (identical results; 1 = default)")
    ap.add_argument("--forest-fuse", type=int, default=1, choices=[0, 1],
                    help="RP forest: three levels per pass over large nodes (1 = default) or one level per pass")
    ap.add_argument("--serve-jobs", type=int, default=32)
    ap.add_argument("--slots", type=int, default=3)
    ap.add_argument("--recall-rows", type=int, default=10_000)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--reference-recall", action="store_true",
                    help="also build the same rows with the reference algorithm on the CPU (minutes at full size) "
                         "and report both recalls on the same sample")
    ap.add_argument("--skip-forms", action="store_true",
                    help="leave the batched and serving measurements out of the default line")
    ap.add_argument("--traffic-per-launch", type=float, default=None,
                    help="dram read+write bytes per join launch from an ncu capture, scaled to this workload")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gpu":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "batched":
        return run_batched(args)
    if args.config == "serving":
        return run_serving(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
