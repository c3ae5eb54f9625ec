"""Benchmark: batched jet clustering on one GB300 (events/s).

Default workload (one "step"): 4096 events, particle counts log-uniform in
[50, 2000] (seeded generator, Poisson(3)+1 hard axes), anti-kt R=0.4 in FP64,
clustered in one batched call (one persistent kernel per size bucket).
``--workload pileup``: 64 pile-up-like events of 10k-60k particles (soft pT
Exp(0.6 GeV), eta U[-4, 4], 2-6 hard axes), anti-kt R=0.4, with kt R=0.6
reported beside it (the tiled kernel).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload mixed|pileup]

Prints one JSON line.  ``value`` is events/s with the inputs resident in HBM,
timed with CUDA events on the library's stream around each step, L2 flushed
(256 MiB write) between steps; each step is one launch of a CUDA graph that
holds the batch call, after the autotuner has picked the launch configuration
(``--no-graph`` / ``--no-tune`` turn either off).  ``e2e`` is the same metric through the
host-memory entry point (pinned host buffers; H2D copy of the inputs, the
kernels, D2H copy of the outputs and a synchronisation inside each step).
``--impl reference`` times the CPU clustering that stands in for the
reference (the reference has no CPU path; see oracle/) on all host cores.
Under torchrun one batch of N x 4096 events is split across the ranks by
estimated cost (replicas.balance; no collective during clustering); rank 0
prints the max-over-ranks time.

The default (mixed) line also carries, measured in the same run:
``latency`` (µs per merge step of lone events, fitted into the per-step
critical path that does not scale with the event and the scan cost per active
pseudojet), ``served`` (1000 requests of the serving mix through the
continuous-batching server at 2k and 20k events/s offered: p50/p99 overall and
for events of at most 2000 particles, and lone requests), ``pileup`` (64
events of 10k-60k particles, anti-kt R=0.4 and kt R=0.6, and end to end) and
``reference_gpu_per_event`` (the reference's own tri_matrix and grid backends,
one event per call through its driver).  ``--no-legs`` skips them.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from fastjet_gpu_gb300 import events as E  # noqa: E402

ALGO, RADIUS = -1, 0.4
WORKLOADS = {
    "mixed": dict(
        events=4096, make=lambda n: E.mixed_batch(n, 50, 2000, seed=3), flush=True, cpu_start=64,
        per_event_sample=256, second=None, dominant=(1024, 2048, "k_cluster_smem, events of 1025-2048 particles"),
        metric="events/s, batched anti-kt R=0.4 clustering of 4096 events (50-2000 particles)",
        workload="4096 events, particle counts log-uniform in [50, 2000], anti-kt R=0.4, FP64, one batched call"),
    "pileup": dict(
        events=64, make=lambda n: E.pileup_batch(n, 10000, 60000, seed=4), flush=True, cpu_start=16,
        per_event_sample=4, second=(1, 0.6), dominant=None,
        metric="events/s, batched anti-kt R=0.4 clustering of 64 pile-up events (10k-60k particles)",
        workload="64 pile-up-like events, 10k-60k particles, anti-kt R=0.4 (kt R=0.6 beside it), FP64, "
                 "one batched call"),
}
WORKLOADS["serving"] = dict(
    events=3000, make=lambda n: E.serving_mix(n, seed=5)[0], flush=False, cpu_start=32, per_event_sample=64,
    second=None, dominant=None,
    metric="events/s served, open-loop Poisson arrivals of single events (lognormal sizes, median 1500), "
           "with p50/p99 latency",
    workload="served requests: sizes lognormal (median 1500, sigma 0.8) clipped to [100, 20000]; anti-kt R=0.4 "
             "70%, kt R=0.6 15%, C/A R=0.8 15%; Poisson arrivals at 2k-200k events/s (20k-200k as specified, 2k and 4k below capacity)")
SERVING_RATES = (2000, 4000, 20000, 50000, 100000, 200000)  # the first two below capacity
# DRAM bytes per particle of a shared-memory clustering launch (read + write):
# one ncu capture of the dominant launch of this workload measured 59.9 MB of
# dram__bytes_read.sum + dram__bytes_write.sum for 1,071,102 particles
TRAFFIC_B_PER_PARTICLE = 55.9
# the same for the tiled kernel: 4.8 MB for a two-event launch of 103,475 particles
TRAFFIC_TILED_B_PER_PARTICLE = 46.4
W = WORKLOADS["mixed"]
N_EVENTS = W["events"]
METRIC = W["metric"]
WORKLOAD = W["workload"]


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[3 + k].lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def fp64_peak_tflops(dev):
    """FP64 peak measured here: cuBLAS DGEMM 4096^3 (2 n^3 flops), best of 5, CUDA events."""
    import torch
    n = 4096
    g = torch.Generator(device=dev).manual_seed(0)
    a = torch.rand((n, n), dtype=torch.float64, device=dev, generator=g)
    b = torch.rand((n, n), dtype=torch.float64, device=dev, generator=g)
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(5):
        s_, e_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s_.record()
        torch.matmul(a, b)
        e_.record()
        e_.synchronize()
        best = min(best, s_.elapsed_time(e_))
    del a, b
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def pair_evaluations(batch, cores, sample=None):
    """Algorithmic pair evaluations E_pairs of the batch, counted by the CPU
    nearest-neighbour oracle on the same inputs: N(N-1)/2 initial distances,
    then per step the new jet against the n_s active pseudojets and one scan of
    n_s for every pseudojet whose neighbour was merged.  With `sample`, only the
    `sample` smallest events are counted and the count is scaled by sum N^2."""
    import oracle
    sizes = batch.sizes().astype(np.float64)
    if sample is None or sample >= batch.n_events:
        return float(oracle.cluster_batch(batch.particles, batch.offsets, ALGO, RADIUS, threads=cores,
                                          want_history=False)[-1]), "counted"
    idx = np.argsort(sizes)[:sample]
    sub = E._batch_from([batch.event(int(e)) for e in idx])
    ev = oracle.cluster_batch(sub.particles, sub.offsets, ALGO, RADIUS, threads=cores, want_history=False)[-1]
    return float(ev) * float((sizes ** 2).sum() / (sizes[idx] ** 2).sum()), \
        f"counted on the {sample} smallest events, scaled by sum N^2"


def cpu_cluster_rate(batch, threads, target_s=10.0, max_events=None, algo=None, radius=None):
    """Oracle events/s on `threads` host threads over a bounded prefix sample."""
    import oracle
    algo = ALGO if algo is None else algo
    radius = RADIUS if radius is None else radius
    n = min(W["cpu_start"], batch.n_events)
    while True:
        off = batch.offsets[: n + 1]
        t0 = time.perf_counter()
        oracle.cluster_batch(batch.particles[: off[-1]], off, algo, radius, threads=threads, want_history=False)
        dt = time.perf_counter() - t0
        if dt >= target_s or n >= batch.n_events or (max_events and n >= max_events):
            return n / dt, n, dt
        n = min(batch.n_events, max(n * 2, int(n * target_s / max(dt, 1e-3))))


def run_reference(args, rank):
    if rank != 0:
        return
    batch = W["make"](N_EVENTS)
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_cluster_rate(batch, cores, target_s=0.5)
    vals, samples = [], []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        v, n, dt = cpu_cluster_rate(batch, cores, target_s=5.0)
        vals.append(v)
        samples.append(n)
    total = time.perf_counter() - t_all
    value = float(np.mean(vals))
    line = {"metric": METRIC, "value": value, "unit": "events/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "events": N_EVENTS, "algorithm": "anti-kt", "R": RADIUS,
                       "l2": "n/a (host CPU)"},
            "cpu_baseline": {"value": value, "unit": "events/s", "cores": cores, "kind": "port",
                             "sample": f"first {min(samples)}-{max(samples)} events of the batch per step "
                                       f"(the reference has no CPU clustering; the oracle restatement, "
                                       f"nearest-neighbour form, one event per thread)"},
            "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _pct(x, q):
    return float(np.percentile(x, q)) if len(x) else None


def serving_leg(ctx, local_rank, n_events=1000, rates=(2000, 20000), lone_n=48):
    """Requests through the continuous-batching server, bounded for the default
    run: the first `n_events` requests of the serving mix (lognormal sizes,
    median 1500, sigma 0.8, clipped to [100, 20000]; anti-kt R=0.4 70%, kt
    R=0.6 15%, C/A R=0.8 15%) replayed open-loop with Poisson arrivals at each
    offered rate (latency: scheduled arrival to observed completion), then
    `lone_n` requests of at most 2000 particles one at a time."""
    import fastjet_gpu_gb300 as F
    batch, algo, radius = E.serving_mix(n_events, seed=5)
    sizes = batch.sizes()
    small = sizes <= 2000
    srv = F.Server(ctx)
    try:
        k = min(128, n_events)
        srv.replay(batch.particles[: batch.offsets[k]], batch.offsets[: k + 1], algo[:k], radius[:k],
                   np.arange(k) * 50.0)
        gaps = np.random.default_rng(17).exponential(1.0, n_events)
        launches0 = srv.launches
        rows = []
        with ClockSampler(local_rank) as clk:
            for rate in rates:
                arrival = np.cumsum(gaps) * (1e6 / rate)
                lat, wall = srv.replay(batch.particles, batch.offsets, algo, radius, arrival)
                lat = lat / 1e3
                rows.append({"offered": rate, "served": n_events / (wall * 1e-6),
                             "p50_ms": _pct(lat, 50), "p99_ms": _pct(lat, 99),
                             "p50_ms_le2000": _pct(lat[small], 50), "p99_ms_le2000": _pct(lat[small], 99)})
        launches = srv.launches - launches0
        pick = np.flatnonzero(small)
        pick = pick[np.linspace(0, pick.size - 1, min(lone_n, pick.size)).astype(int)]
        lone = []
        for e in pick:
            t0 = time.perf_counter()
            srv.submit(batch.event(int(e)), int(algo[e]), float(radius[e]))
            got = []
            while not got:
                got = srv.poll(1, timeout_us=1000000)
            lone.append(1e3 * (time.perf_counter() - t0))
    finally:
        srv.close()
    return {"requests_per_rate": n_events, "rates": rows, "gpu_launches": launches, "clocks": clk.summary(),
            "lone_request_ms_le2000": {"p50": _pct(lone, 50), "p99": _pct(lone, 99), "requests": len(lone),
                                       "sizes": [int(sizes[pick].min()), int(sizes[pick].max())]},
            "l2": "not flushed: each request's momenta arrive from host memory as it is submitted",
            "workload": "served requests: the first 1000 of the serving mix (sizes lognormal, median 1500, "
                        "in [100, 20000]; anti-kt 0.4 / kt 0.6 / C/A 0.8 at 70/15/15 %), Poisson arrivals"}


def pileup_leg(ctx, dev, stream, flush, steps=2):
    """64 pile-up-like events of 10k-60k particles (soft pT Exp(0.6 GeV), eta
    U[-4, 4], 2-6 hard axes) in one batched call on the tiled kernel: anti-kt
    R=0.4 and kt R=0.6, inputs resident and L2 flushed between steps, then
    end to end through the host entry point (pinned buffers)."""
    import torch
    batch = E.pileup_batch(64, 10000, 60000, seed=4)
    total = int(batch.offsets[-1])
    ne = batch.n_events
    p4 = torch.from_numpy(batch.particles).to(dev)
    off = torch.from_numpy(batch.offsets).to(dev)
    out = {"jets": torch.empty((total, 4), dtype=torch.float64, device=dev),
           "jet_label": torch.empty(total, dtype=torch.int32, device=dev),
           "n_jets": torch.empty(ne, dtype=torch.int32, device=dev)}
    res = {}
    for name, algo, radius, k in (("anti-kt R=0.4", -1, 0.4, steps), ("kt R=0.6", 1, 0.6, 1)):
        with torch.cuda.stream(stream):
            ctx.cluster_batch_device(p4, off, algo, radius, total=total, out=out)
        ctx.check()
        ms = []
        with torch.cuda.stream(stream):
            for i in range(k):
                flush.fill_(float(i))
                s_, e_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s_.record(stream)
                ctx.cluster_batch_device(p4, off, algo, radius, total=total, out=out)
                e_.record(stream)
                e_.synchronize()
                ms.append(s_.elapsed_time(e_))
        ctx.check()
        res[name] = {"value": ne * k / (sum(ms) / 1e3), "unit": "events/s", "ms_per_step": float(np.mean(ms)),
                     "steps": k}
    del p4, off, out
    p4_h = torch.from_numpy(batch.particles).pin_memory().numpy()
    off_h = torch.from_numpy(batch.offsets).pin_memory().numpy()
    out_h = {"jets": torch.empty((total, 4), dtype=torch.float64).pin_memory().numpy(),
             "jet_label": torch.empty(total, dtype=torch.int32).pin_memory().numpy(),
             "n_jets": torch.empty(ne, dtype=torch.int32).pin_memory().numpy()}
    t0 = time.perf_counter()
    ctx.cluster_batch(p4_h, off_h, -1, 0.4, out=out_h)
    e2e = ne / (time.perf_counter() - t0)
    return {"workload": f"{ne} pile-up-like events, 10k-60k particles ({total} in all), one batched call",
            "events": ne, "particles": total, "l2": "flushed between steps (256 MiB write)",
            "anti-kt R=0.4": res["anti-kt R=0.4"], "kt R=0.6": res["kt R=0.6"],
            "e2e": {"value": e2e, "unit": "events/s", "h2d_bytes_per_step": int(batch.particles.nbytes
                                                                               + batch.offsets.nbytes),
                    "d2h_bytes_per_step": int(total * 36 + ne * 4)}}


def reference_gpu_leg(batch, n_sample=12, repeat=20):
    """The reference's own GPU backends, one event per cluster() call through
    its own driver (main.cc:269-335, `--repeat 20 --csv`: the mean cudaEvent time
    of the H2D copy, cluster() -- which allocates and frees its scratch on every
    call -- and the D2H copy), built from the reference sources by
    oracle/ref/Makefile: the 354- and 808-particle events of the parity set and
    a size-spread sample of this batch's events.  Context for the batched
    number: the reference has no batched or served mode."""
    import re
    bindir = os.path.join(ROOT, "oracle", "_ref", "bin")
    if not all(os.access(os.path.join(bindir, b), os.X_OK) for b in ("tri_matrix", "grid")):
        return {"unavailable": "reference backends not built (oracle/ref/Makefile needs the staged sources)"}
    golden = os.path.join(ROOT, "tests", "golden", "inputs")
    with open(os.path.join(golden, "synth_354.txt")) as f:
        t354 = f.read()
    with open(os.path.join(golden, "synth_808.txt")) as f:
        t808 = f.read()
    sizes = batch.sizes()
    order = np.argsort(sizes, kind="stable")
    pick = order[np.linspace(0, order.size - 1, min(n_sample, order.size)).astype(int)]
    tmix = E.write_events([batch.event(int(e)) for e in pick])
    cases = [("354 particles, anti-kt R=0.4, ptmin 1", t354, ["-antikt", "-r", "0.4", "-p", "1.0"]),
             ("808 particles, kt R=1.0", t808, ["-kt", "-r", "1.0"]),
             ("808 particles, anti-kt R=0.4", t808, ["-antikt", "-r", "0.4"]),
             ("808 particles, C/A R=0.8", t808, ["-cam", "-r", "0.8"]),
             (f"{pick.size} events of this batch, {int(sizes[pick].min())}-{int(sizes[pick].max())} particles, "
              "anti-kt R=0.4", tmix, ["-antikt", "-r", "0.4", "-p", "1.0"])]
    line = re.compile(r"^(\d+),(\d+),([0-9.eE+-]+)")
    out = {"how": f"reference driver --repeat {repeat} --csv, per event: mean ms of H2D + cluster() + D2H",
           "cases": []}
    for backend in ("tri_matrix", "grid"):
        for name, text, argv in cases:
            try:
                r = subprocess.run([os.path.join(bindir, backend)] + argv + ["--repeat", str(repeat), "--csv"],
                                   input=text, capture_output=True, text=True, timeout=600)
            except subprocess.TimeoutExpired:
                out["cases"].append({"backend": backend, "case": name, "unavailable": "timed out"})
                continue
            ms = [(int(m.group(1)), float(m.group(3))) for m in map(line.match, r.stdout.split("\n")) if m]
            if r.returncode != 0 or not ms:
                out["cases"].append({"backend": backend, "case": name, "unavailable": f"exit {r.returncode}"})
                continue
            tot = sum(t for _, t in ms)
            out["cases"].append({"backend": backend, "case": name, "events": len(ms),
                                 "ms_per_event": tot / len(ms), "events_per_s": 1e3 * len(ms) / tot,
                                 "per_event": [[n, t] for n, t in ms]})
    return out


def latency_leg(ctx, dev, sizes=(1100, 1400, 1700, 2000), repeat=5):
    """Per merge step latency of lone events on the plain path (one event per
    launch, CUDA events), all in the 1025-2048-particle bucket so that one
    kernel shape runs them.  An event of N particles takes N steps over
    N, N-1, ..., 1 active pseudojets, so its time per step is fitted as
    c0 + c1 * (N + 1) / 2: c0 is the part of a step that does not grow with
    the event (the argmin reductions and barriers, the new jet's FP64
    kinematics, the neighbour resolution) -- the latency floor of this design
    for one event -- and c1 the cost of scanning one active pseudojet."""
    import torch
    rows = []
    for k, n in enumerate(sizes):
        ev = torch.from_numpy(E.single_event(n, 3, seed=500 + k)).to(dev)
        ctx.cluster_event(ev, ALGO, RADIUS)
        ms = []
        for _ in range(repeat):
            s_, e_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s_.record()
            ctx.cluster_event(ev, ALGO, RADIUS)
            e_.record()
            e_.synchronize()
            ms.append(s_.elapsed_time(e_))
        rows.append((n, float(np.median(ms))))
    n = np.array([r[0] for r in rows], dtype=np.float64)
    us_step = np.array([1e3 * r[1] / r[0] for r in rows])
    c1, c0 = np.polyfit((n + 1) / 2, us_step, 1)
    return {"events": [{"particles": int(a), "ms": b, "us_per_step": 1e3 * b / a} for a, b in rows],
            "floor_us_per_step": float(c0), "us_per_active_pseudojet": float(c1),
            "floor_share_at_2000": float(c0 / us_step[-1]),
            "note": "one event per launch, anti-kt R=0.4, bucket 1025-2048 (one kernel shape); per-step time "
                    "fitted as c0 + c1 * mean active pseudojets; c0 = the per-step critical path that does not "
                    "scale with the event"}


def run_ours(args, rank, world, local_rank):
    import torch

    import fastjet_gpu_gb300 as F

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    if world > 1:
        # replicas: one batch of world x N_EVENTS events split across the ranks
        # by estimated cost (N^2 per event), no exchange during clustering
        from fastjet_gpu_gb300 import replicas as RP
        full = W["make"](N_EVENTS * world)
        mine = RP.balance(full.sizes(), world)[rank]
        batch = E.Batch(*RP.subset(full.particles, full.offsets, mine))
        del full
    else:
        batch = W["make"](N_EVENTS)
    n_local = batch.n_events
    total = int(batch.offsets[-1])
    ctx = F.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    p4 = torch.from_numpy(batch.particles).to(dev)
    off = torch.from_numpy(batch.offsets).to(dev)
    out = {"jets": torch.empty((total, 4), dtype=torch.float64, device=dev),
           "jet_label": torch.empty(total, dtype=torch.int32, device=dev),
           "n_jets": torch.empty(n_local, dtype=torch.int32, device=dev)}
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    tuning = None
    if not args.no_tune:
        # per-bucket kernel shape and CTAs per SM (and the tile side when the
        # workload has events above 2048 particles), timed on synthetic events
        tuning = ctx.autotune(ALGO, RADIUS, skip_large=int(batch.sizes().max()) <= 2048)
    graph = None if args.no_graph else ctx.capture_batch(p4, off, ALGO, RADIUS, total=total, out=out)

    def step(algo=ALGO, radius=RADIUS):
        if graph is not None and (algo, radius) == (ALGO, RADIUS):
            graph.launch()
        else:
            ctx.cluster_batch_device(p4, off, algo, radius, total=total, out=out)

    def check():
        ctx.check()
        if graph is not None:
            graph.check()

    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            step()
    check()
    n_jets_total = int(out["n_jets"].sum().item())

    def timed_steps(k_steps, algo=ALGO, radius=RADIUS):
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(k_steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(k_steps)]
        with torch.cuda.stream(stream):  # the library's stream: its kernels, the flush and the events
            for k in range(k_steps):
                if W["flush"]:
                    flush.fill_(float(k))  # evict L2 between steps (the inputs, 70-80 MB, fit in the 129 MB L2)
                torch.cuda.nvtx.range_push("timed_step")
                starts[k].record(stream)
                step(algo, radius)
                ends[k].record(stream)
                torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        return [s_.elapsed_time(e_) for s_, e_ in zip(starts, ends)]

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clk:
        t_wall = time.perf_counter()
        step_ms = timed_steps(args.steps)
        t_wall = time.perf_counter() - t_wall
    check()
    barrier()
    dev_s = sum(step_ms) / 1e3
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([dev_s], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_s = float(t.item())
    value = world * N_EVENTS * args.steps / dev_s

    # end to end through the host-memory entry point (pinned buffers)
    p4_h = torch.from_numpy(batch.particles).pin_memory().numpy()
    off_h = torch.from_numpy(batch.offsets).pin_memory().numpy()
    out_h = {"jets": torch.empty((total, 4), dtype=torch.float64).pin_memory().numpy(),
             "jet_label": torch.empty(total, dtype=torch.int32).pin_memory().numpy(),
             "n_jets": torch.empty(n_local, dtype=torch.int32).pin_memory().numpy()}
    for _ in range(2):
        ctx.cluster_batch(p4_h, off_h, ALGO, RADIUS, out=out_h)
    barrier()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 5))
    for _ in range(e2e_steps):
        res = ctx.cluster_batch(p4_h, off_h, ALGO, RADIUS, out=out_h)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    assert int(res["n_jets"].sum()) == n_jets_total
    h2d = batch.particles.nbytes + batch.offsets.nbytes

    # the plain path: one event per launch, synchronous (the per-event-launch
    # comparator), on an evenly spaced sample of the same events
    idx = np.linspace(0, n_local - 1, min(W["per_event_sample"], n_local)).astype(int)
    sample = [torch.from_numpy(batch.event(int(e))).to(dev) for e in idx]
    ctx.cluster_event(sample[0], ALGO, RADIUS)
    lat = []
    for ev in sample:
        t0 = time.perf_counter()
        ctx.cluster_event(ev, ALGO, RADIUS)
        lat.append(time.perf_counter() - t0)
    sizes = batch.sizes()
    # event sizes are drawn independently of their position, so an evenly
    # spaced sample follows the batch's size distribution
    per_event = {"value": len(lat) / sum(lat) if sum(lat) > 0 else None, "unit": "events/s",
                 "p50_ms": 1e3 * float(np.percentile(lat, 50)), "p99_ms": 1e3 * float(np.percentile(lat, 99)),
                 "sample": f"{len(lat)} events evenly spaced in the batch (sizes {int(sizes[idx].min())}-"
                           f"{int(sizes[idx].max())}), fjg_cluster_event, synchronous, device inputs"}
    second = None
    if W["second"] is not None:
        a2, r2 = W["second"]
        with torch.cuda.stream(stream):
            step(a2, r2)
        ctx.check()
        ms2 = timed_steps(max(1, min(args.steps, 3)), a2, r2)
        second = {"algorithm": {1: "kt", 0: "cambridge-aachen", -1: "anti-kt"}[a2], "R": r2,
                  "value": n_local * len(ms2) / (sum(ms2) / 1e3), "unit": "events/s",
                  "ms_per_step": float(np.mean(ms2))}
    d2h = total * 32 + total * 4 + n_local * 4

    # roofline.  Primary: algorithmic FP64 work of the dominant kernel (9 flops
    # per pair evaluation, pair evaluations counted by the CPU oracle on the
    # same events) per launch / its launch time, against the FP64 peak measured
    # here with DGEMM.  Secondary: shared-memory bytes of the same work (24 B
    # per pair evaluation: rap, phi, w of the partner) against the nominal
    # shared-memory bandwidth, and the HBM staging bytes of the whole step.
    alg_bytes = 32 * total + 8 * (n_local + 1) + 36 * n_jets_total + 4 * n_local
    step_s = dev_s / args.steps
    peak, peak_kind = _peaks()
    achieved = alg_bytes / step_s / 1e9
    cores = os.cpu_count() or 1
    dom = W.get("dominant")
    if dom is not None:
        lo_n, hi_n, dom_name = dom
        sizes_all = batch.sizes()
        sel = np.flatnonzero((sizes_all > lo_n) & (sizes_all <= hi_n))
        dom_batch = E._batch_from([batch.event(int(e)) for e in sel])
        p4_d = torch.from_numpy(dom_batch.particles).to(dev)
        off_d = torch.from_numpy(dom_batch.offsets).to(dev)
        with torch.cuda.stream(stream):
            for _ in range(2):
                ctx.cluster_batch_device(p4_d, off_d, ALGO, RADIUS)
        ctx.check()
        dms = []
        with torch.cuda.stream(stream):
            for k in range(3):
                flush.fill_(float(k))
                s_, e_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                torch.cuda.nvtx.range_push("dominant_kernel")  # profilers can select these launches
                s_.record(stream)
                ctx.cluster_batch_device(p4_d, off_d, ALGO, RADIUS)
                e_.record(stream)
                torch.cuda.nvtx.range_pop()
                e_.synchronize()
                dms.append(s_.elapsed_time(e_))
        ctx.check()
        dom_s = float(np.mean(dms)) / 1e3
        e_pairs, e_how = pair_evaluations(dom_batch, cores)
        dom_desc = f"{dom_name} ({dom_batch.n_events} events, {int(dom_batch.offsets[-1])} particles), " \
                   f"timed alone on its events (CUDA events, 3 launches)"
        dom_particles = int(dom_batch.offsets[-1])
    else:
        dom_s = step_s
        e_pairs, e_how = pair_evaluations(batch, cores, sample=4 if n_local > 512 or total > 10 ** 6 else None)
        dom_desc = "k_cluster_tiled (every event of the batch: one launch per step)"
        dom_particles = total
    fp64_peak = fp64_peak_tflops(dev)
    fp64_ach = 9.0 * e_pairs / dom_s / 1e12
    smem_peak = 128.0 * 152 * 2.07e9 / 1e12  # TB/s, nominal: 128 B per clock per SM at 2070 MHz
    fp32_peak = 128.0 * 152 * 2.07e9 / 1e12  # T operations/s, nominal: 128 FP32 lanes per SM
    # DRAM bytes per particle of the shared-memory kernels from an ncu capture
    # of the same kernel on the same workload, scaled to this launch
    traffic = (TRAFFIC_B_PER_PARTICLE if dom is not None else TRAFFIC_TILED_B_PER_PARTICLE) * dom_particles
    line = {"metric": METRIC, "value": value, "unit": "events/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": 1e3 * step_s, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "events": N_EVENTS, "particles": total, "algorithm": "anti-kt",
                       "R": RADIUS, "l2": "flushed between steps (256 MiB write)" if W["flush"] else "not flushed",
                       "parallelism": f"replicas{world}", "cuda_graph": graph is not None,
                       "tuning": tuning},
            "per_event_launch": per_event,
            "e2e": {"value": world * N_EVENTS / e2e_s, "unit": "events/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "roofline": {"bound": "fp64", "kind": "FP64-equivalent", "kernel": dom_desc, "achieved": fp64_ach,
                         "peak": fp64_peak, "unit": "TFLOP/s", "frac": fp64_ach / fp64_peak, "traffic": traffic,
                         "pair_evaluations": e_pairs, "pair_evaluations_how": e_how,
                         "launch_ms": 1e3 * dom_s,
                         "note": "FP64-equivalent: achieved = 9 flops x E_pairs (oracle count) / launch time, "
                                 "against the FP64 rate measured here (cuBLAS DGEMM 4096^3): how fast an "
                                 "implementation bound by FP64 arithmetic would have to be to match.  The "
                                 "kernels take most pair decisions in FP32 with a proven error bound, so this "
                                 "is not the resource that binds; the pipes they use are in 'secondary', and "
                                 "the per-step critical path that does bind is in 'latency'",
                         "secondary": [
                             {"bound": "fp32", "achieved": 12.0 * e_pairs / dom_s / 1e12, "peak": fp32_peak,
                              "unit": "TFLOP/s", "frac": 12.0 * e_pairs / dom_s / 1e12 / fp32_peak,
                              "note": "12 FP32 operations per pair evaluation (the filter distance and its "
                                      "bound); peak nominal (128 lanes x 152 SMs x 2070 MHz, one operation "
                                      "per lane and clock)"},
                             {"bound": "smem", "achieved": 24.0 * e_pairs / dom_s / 1e12, "peak": smem_peak,
                              "unit": "TB/s", "frac": 24.0 * e_pairs / dom_s / 1e12 / smem_peak,
                              "note": "24 B per pair evaluation; peak nominal (128 B/clk/SM, 152 SMs, 2070 MHz)"},
                             {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                              "frac": achieved / peak,
                              "note": f"whole step, staging only ({alg_bytes} B per step); peak {peak_kind}"}]},
            "gpu_launches": args.steps * 12,  # 2 input checks, 4 bucketing kernels, the tiled kernel, 5 buckets
            "clocks": clk.summary(),
            "wall_s": t_wall}
    if second is not None:
        line["config"]["second"] = second
    if rank == 0 and not args.no_legs and args.workload == "mixed":
        line["latency"] = latency_leg(ctx, dev)
        line["served"] = serving_leg(ctx, local_rank)
        line["pileup"] = pileup_leg(ctx, dev, stream, flush)
        line["reference_gpu_per_event"] = reference_gpu_leg(batch)
    if rank == 0 and not args.no_cpu_baseline:
        v, n, dt = cpu_cluster_rate(batch, cores, target_s=10.0)
        v1, n1, dt1 = cpu_cluster_rate(batch, 1, target_s=5.0)
        line["cpu_baseline"] = {"value": v, "unit": "events/s", "cores": cores, "kind": "port",
                                "sample": f"first {n} of the {n_local} events ({dt:.1f} s), oracle "
                                          f"nearest-neighbour clustering, one event per thread",
                                "single_thread": {"value": v1, "unit": "events/s", "cores": 1,
                                                  "sample": f"first {n1} events ({dt1:.1f} s)"}}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if graph is not None:
        graph.close()
    ctx.close()


def run_serving(args, rank, world, local_rank):
    """Open-loop serving: each offered rate replays the same request trace
    (one event per request) through the server; latency runs from each
    request's scheduled arrival to its completion being observed."""
    import torch

    import fastjet_gpu_gb300 as F

    if rank != 0:
        return
    torch.cuda.set_device(local_rank)
    batch, algo, radius = E.serving_mix(N_EVENTS, seed=5)
    sizes = batch.sizes()
    small = sizes <= 2000
    ctx = F.Context(local_rank)
    tuning = None if args.no_tune else ctx.autotune(-1, 0.4)
    srv = F.Server(ctx)
    rng = np.random.default_rng(17)
    gaps = rng.exponential(1.0, N_EVENTS)
    # warm-up: the first requests of the trace, well spaced
    for _ in range(max(args.warmup, 3)):
        k = min(256, N_EVENTS)
        srv.replay(batch.particles[: batch.offsets[k]], batch.offsets[: k + 1], algo[:k], radius[:k],
                   np.arange(k) * 50.0)
    rates = []
    launches0 = srv.launches
    with ClockSampler(local_rank) as clk:
        for rate in SERVING_RATES:
            arrival = np.cumsum(gaps) * (1e6 / rate)
            lat, wall = srv.replay(batch.particles, batch.offsets, algo, radius, arrival)
            rates.append({"offered": rate, "served": N_EVENTS / (wall * 1e-6), "wall_s": wall * 1e-6,
                          "p50_ms": float(np.percentile(lat, 50)) / 1e3, "p99_ms": float(np.percentile(lat, 99)) / 1e3,
                          "p50_ms_le2000": float(np.percentile(lat[small], 50)) / 1e3,
                          "p99_ms_le2000": float(np.percentile(lat[small], 99)) / 1e3})
    launches = srv.launches - launches0
    # lightly loaded: requests one at a time (latency of a lone event)
    lone_idx = np.linspace(0, N_EVENTS - 1, 64).astype(int)
    lone = []
    for e in lone_idx:
        t0 = time.perf_counter()
        srv.submit(batch.event(int(e)), int(algo[e]), float(radius[e]))
        got = []
        while not got:
            got = srv.poll(1, timeout_us=1000000)
        lone.append(1e3 * (time.perf_counter() - t0))
    lone = np.array(lone)
    lone_small = lone[sizes[lone_idx] <= 2000]
    srv.close()
    # the same events as one batch, and one event per launch
    dev = torch.device("cuda", local_rank)
    p4 = torch.from_numpy(batch.particles).to(dev)
    off = torch.from_numpy(batch.offsets).to(dev)
    a_t = torch.from_numpy(algo).to(dev)
    r_t = torch.from_numpy(radius).to(dev)
    ctx.cluster_batch_device(p4, off, a_t, r_t)
    torch.cuda.synchronize()
    ctx.check()
    t0 = time.perf_counter()
    ctx.cluster_batch_device(p4, off, a_t, r_t)
    torch.cuda.synchronize()
    batched = N_EVENTS / (time.perf_counter() - t0)
    ctx.check()
    sample = [torch.from_numpy(batch.event(int(e))).to(dev) for e in lone_idx[:16]]
    t0 = time.perf_counter()
    for k, ev in enumerate(sample):
        e = int(lone_idx[k])
        ctx.cluster_event(ev, int(algo[e]), float(radius[e]))
    per_event = len(sample) / (time.perf_counter() - t0)
    top = rates[-1]
    h2d = int(batch.particles.nbytes)
    line = {"metric": METRIC, "value": top["served"], "unit": "events/s", "n_gpus": 1, "steps": len(SERVING_RATES),
            "warmup": max(args.warmup, 3), "ms_per_step": 1e3 * float(np.mean([r["wall_s"] for r in rates])),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "requests_per_rate": N_EVENTS, "particles": int(batch.offsets[-1]),
                       "l2": "not flushed: each request's momenta are copied in from host memory as it arrives",
                       "rates": rates, "tuning": tuning,
                       "lone_request_ms": {"p50": float(np.percentile(lone, 50)), "p99": float(np.percentile(lone, 99)),
                                           "p50_le2000": float(np.percentile(lone_small, 50)),
                                           "p99_le2000": float(np.percentile(lone_small, 99)),
                                           "sample": f"{len(lone)} requests one at a time"},
                       "batched_same_events": batched, "per_event_launch": per_event},
            "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"],
            "e2e": {"value": top["served"], "unit": "events/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": 0},
            "gpu_launches": launches, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-legs", action="store_true",
                    help="mixed workload: skip the latency, served, pile-up and reference-GPU legs")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch configuration")
    ap.add_argument("--no-graph", action="store_true", help="launch through the API instead of a CUDA graph")
    ap.add_argument("--workload", default="mixed", choices=sorted(WORKLOADS))
    ap.add_argument("--events", type=int, default=None,
                    help="events per step (default: the workload's; smaller only for profiling captures)")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    globals().update(W=w, N_EVENTS=args.events or w["events"], METRIC=w["metric"], WORKLOAD=w["workload"])
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.workload == "serving":
        run_serving(args, rank, world, local_rank)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    try:
        run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
