#!/usr/bin/env python
"""Voxel-steps/s of the Voxelyze3 soft-body step on GB300.

Default run (N=1) prints one JSON line whose value is the batched
plain-physics configuration — 512 independent seeded creatures (cubic
lattice side U{6..20}, fill U(0.3, 0.9), largest 6-connected component, four
materials with E log-uniform in [1e5, 1e7] Pa, rho=1000, nu=0.35, one or two
actuated at 5 Hz), gravity and floor on, no self-collision, FP64, all creatures
packed into shared launches.  A "step" is one physics step of the whole batch.
The batch's device state (~1 GB) is larger than L2, so no flush is needed
between timed iterations.  The first steps of the fresh batch are timed on
their own (config.fresh_batch); after 256 more settling steps the launch shape
is picked by the autotuner (vx3_autotune, recorded in config.tuning) and the
line's K steps are timed (config.timed_window): the configuration's runs are
35,000-56,000 steps long, nearly all of them in that settled regime.

The same line carries, under "modes":
  plain_vs_batched  the one-simulation-per-launch form against the batched form on
                    the same sample of creatures;
  serve             the serving stream: Poisson arrivals at 50, 200 and 2,000 req/s
                    of creatures with V log-uniform in [100, 1e5] and horizons
                    U[1e3, 5e4] steps, 20% with self-collision, through the
                    continuous-batching loop (vx3_submit / vx3_poll), against the
                    plain per-simulation path on the same requests;
  collide           64 creatures of 40^3 at fill 0.5 with self-collision, all in one
                    batch, for a bounded share of their 20,000 steps;
  slab              the single 200x200x100 body (4M voxels) for its 2,000 steps
                    (or a bounded share), with its HBM and FP64 rooflines.

Other workloads (--workload): slab, collide, plain (one 10^3 creature) as the
line's value, serve (the serving block alone, more requests).

--impl reference times the reference's CPU implementation of the step on this
machine's host cores: the reference compiled from its own sources
(oracle/_ref) where present, otherwise the oracle's C restatement.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_PEAK_FALLBACK = 6800.0
FP64_INSTR_PEAK = 505.8e9          # measured DFMA/DADD/DMUL issue rate on this machine's GB300 (instructions/s)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", HBM_PEAK_FALLBACK)), "measured"
    return HBM_PEAK_FALLBACK, "fallback"


# FP64-pipe thread instructions (DADD/DMUL/DFMA, compares, conversions; predicated-on lanes)
# per link (k_links) and per voxel (k_voxels) of one step, read by ncu per workload in the
# steps the workload's value is timed over (sm__thread_inst_executed_pipe_fp64_pred_on.sum /
# links or voxels); the lanes a warp's FP64 instruction keeps busy on average (that sum /
# sm__inst_executed_pipe_fp64.sum: the pipe costs the same per warp instruction whatever
# its active lanes); and DRAM bytes per link of one k_links launch (dram__bytes_read.sum +
# dram__bytes_write.sum / links).  profiles/fp64_counts_by_workload.md has the captures.
FP64_COUNTS = {
    # batch of 512 creatures, step 288 (the settled window the line's value is timed over)
    "batch": dict(per_link=655165600 / 1627115, per_voxel=195889184 / 844972,
                  lanes_link=655165600 / 21707472, lanes_voxel=195889184 / 6829054,
                  traffic_per_link=764864000 / 1627115, source="ncu, 512-creature batch, step 288"),
    # 8 of the 64 collision creatures, mean of steps 201, 1001 and 1901 (the 2,000 timed steps)
    "collide": dict(per_link=(149924800 + 139983552 + 137419616) / 3 / 373621,
                    per_voxel=(64035808 + 59213696 + 58503680) / 3 / 249183,
                    lanes_link=(149924800 + 139983552 + 137419616) / (5079772 + 4651183 + 4567875),
                    lanes_voxel=(64035808 + 59213696 + 58503680) / (2291351 + 2149824 + 2144277),
                    traffic_per_link=(180225280 + 181382912 + 181297408) / 3 / 373621,
                    source="ncu, 8 collision creatures 40^3, mean of steps 201, 1001, 1901"),
    # a 100x100x50 slab, mean of steps 201, 1001 and 1901
    "slab": dict(per_link=(695043520 + 694503200 + 694274368) / 3 / 1480000,
                 per_voxel=(117620192 + 117357888 + 117292448) / 3 / 500000,
                 lanes_link=(695043520 + 694503200 + 694274368) / (22570878 + 22544145 + 22522796),
                 lanes_voxel=(117620192 + 117357888 + 117292448) / (3896502 + 3879244 + 3875868),
                 traffic_per_link=(420665344 + 421070336 + 421153792) / 3 / 1480000,
                 source="ncu, 100x100x50 slab, mean of steps 201, 1001, 1901"),
}
# steps a whole run of each workload takes (the batch: 0.5 s simulated at its creatures' time steps)
RUN_STEPS = {"batch": "35,000-56,000", "collide": "20,000", "slab": "2,000", "plain": "10,000"}
FP64_INSTR_PER_LINK = FP64_COUNTS["batch"]["per_link"]
FP64_INSTR_PER_VOXEL = FP64_COUNTS["batch"]["per_voxel"]
LINK_TRAFFIC_PER_LINK = FP64_COUNTS["batch"]["traffic_per_link"]


def fp64_peak_fma_per_s(device=0):
    """FP64 FMA throughput of this GPU, measured live with a cuBLAS DGEMM (4096^3, best of 3):
    the denominator of the FP64 roofline, as the HBM copy and the bf16 GEMM are for the others."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=f"cuda:{device}")
    b = torch.randn(n, n, dtype=torch.float64, device=f"cuda:{device}")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    torch.cuda.empty_cache()
    return n ** 3 / best


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------- workloads
def make_workload(name, rank=0, n_batch=512, n_collide=64, slab_dims=(200, 200, 100)):
    from gpuvoxels_gb300 import synth
    if name == "batch":
        cs = synth.config1_batch(n_batch, seed=1 + 1000 * rank, sim_time=0.5)
        desc = dict(workload="batched plain physics: %d creatures, side U{6..20}, fill U(0.3,0.9), 4 materials E log-uniform "
                    "[1e5,1e7] Pa, nu=0.35, 5 Hz actuation, 0.01 m voxels, gravity+floor, no self-collision" % len(cs))
    elif name == "slab":
        X, Y, Z = slab_dims
        cs = [synth.slab(X, Y, Z, seed=3 + rank)]
        desc = dict(workload=f"single large body: solid {X}x{Y}x{Z} slab ({X * Y * Z} voxels), E=1e6, nu=0.35, "
                             "per-voxel CTE actuation")
    elif name == "collide":
        cs = synth.config2_batch(n_collide, seed=2 + rank)
        desc = dict(workload="collision-heavy: %d creatures 40^3 fill 0.5, 3 materials incl. E=1e5, self-collision on "
                    "(radius 0.75), contraction-only actuation at 5 Hz" % len(cs))
    elif name == "plain":
        cs = [synth.config0_creature(0)]
        desc = dict(workload="plain single creature: 10^3 lattice, fill 0.6, passive+active, 5 Hz +-39 C")
    else:
        raise ValueError(name)
    return cs, desc


def algorithmic_bytes(ctx, ids):
    """Compulsory DRAM bytes of one step: k_links reads and writes 284 B per link plus 73 B per
    endpoint voxel; k_voxels 249 B per voxel plus 52 B per link end (its force and moment slot)."""
    import gpuvoxels_gb300 as g
    link_b = vox_b = 0
    for i in ids:
        info = ctx.info(i)
        nv, nl = info.num_voxel, info.num_link
        link_b += nl * 284 + nv * 73
        vox_b += nv * (104 + 4 + 4 + 1 + 4 + 8 + 104 + 4 + 12 + 4) + 2 * nl * 52
    return link_b, vox_b


# ---------------------------------------------------------------------------- CPU baseline
def cpu_sample(cs, budget_s=12.0, threads=None, prefer_reference=True):
    """Times the CPU implementation on a bounded sample of the workload, one simulation
    per host thread.  Returns (voxel-steps/s, threads, kind, sample text)."""
    from oracle.oracle import OracleSim, RefSim, desc_from_vxa
    threads = threads or os.cpu_count() or 1
    kind = "reference" if (prefer_reference and RefSim.available()) else "port"
    picks = [cs[i % len(cs)] for i in range(threads)]
    # size the per-thread step count from a short probe so the sample takes ~budget_s
    def make(c):
        return RefSim(c.vxa) if kind == "reference" else OracleSim(desc_from_vxa(c.vxa))
    probe = make(picks[0])
    t0 = time.perf_counter()
    probe.step(20)
    per_vs = (time.perf_counter() - t0) / (20 * picks[0].num_voxel)
    mean_v = sum(c.num_voxel for c in picks) / len(picks)
    steps = max(20, int(budget_s / max(per_vs * mean_v, 1e-9)))
    sims = [make(c) for c in picks]
    for s in sims:
        s.step(2)

    def work(s):
        return s.step(steps)

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        done = list(ex.map(work, sims))
    dt = time.perf_counter() - t0
    vsteps = sum(d * c.num_voxel for d, c in zip(done, picks))
    return vsteps / dt, threads, kind, f"{threads} creatures of the workload x {steps} steps, one per host thread"


# ---------------------------------------------------------------------------- main arms
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist.get_rank(), ws, dist


def shard(items, rank, world):
    """Round-robin dealing of independent simulations to devices (vx3_node_worker.cu:91-93)."""
    return [x for i, x in enumerate(items) if i % world == rank]


def reduce_timing(dist, dev_s, vsteps):
    """Whole-job numbers: the slowest rank's time and the sum of every rank's voxel-steps."""
    if dist is None:
        return dev_s, vsteps
    import torch
    t = torch.tensor([dev_s, float(vsteps)], dtype=torch.float64)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    sm = t.clone()
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return float(mx[0]), int(sm[1])


def kernel_times(ctx, ids, reps=5):
    """Median per-kernel device times over `reps` profiled steps (one launch per kernel, CUDA
    events on the context's stream): (k_links ms, contacts ms, k_voxels ms)."""
    import gpuvoxels_gb300 as g
    ctx.set_profiling(True)
    lk, ck, vk = [], [], []
    for _ in range(reps):
        ctx.step(ids, 1, g.BATCHED)
        t = ctx.timing()
        lk.append(t["link_ms"]); ck.append(t["contact_ms"]); vk.append(t["voxel_ms"])
    ctx.set_profiling(False)
    return statistics.median(lk), statistics.median(ck), statistics.median(vk)


def rooflines(ctx, ids, workload, link_ms, con_ms, vox_ms, peak64):
    """HBM roofline of the dominant step kernel (algorithmic bytes over its event-timed duration
    against the measured copy bandwidth) and, beside it, the FP64-pipe roofline that binds."""
    link_b, vox_b = algorithmic_bytes(ctx, ids)
    dom = "k_links" if link_ms >= vox_ms else "k_voxels"
    dom_ms, dom_b = (link_ms, link_b) if dom == "k_links" else (vox_ms, vox_b)
    peak, peak_kind = measured_peaks()
    achieved = dom_b / (dom_ms / 1e3) / 1e9
    n_links = sum(ctx.info(i).num_link for i in ids)
    n_vox = sum(ctx.info(i).num_voxel for i in ids)
    counts = FP64_COUNTS.get(workload)
    if counts is None or peak64 is None:
        fp64 = {"unavailable": "no ncu count of FP64 instructions for this workload" if counts is None else "no DGEMM peak"}
    else:
        ach_l = counts["per_link"] * n_links / (link_ms / 1e3)
        ach_v = counts["per_voxel"] * n_vox / (vox_ms / 1e3)
        fp64 = {"bound": "fp64", "kernel": "k_links", "achieved": ach_l / 1e9, "peak": peak64 / 1e9,
                "unit": "G FP64 thread-instructions/s", "frac": ach_l / peak64,
                "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (FMA/s)",
                "instr_per_link": counts["per_link"], "k_voxels_achieved": ach_v / 1e9, "k_voxels_frac": ach_v / peak64,
                "instr_per_voxel": counts["per_voxel"], "counts_source": counts["source"],
                # the pipe's issue capacity in use: a warp instruction costs the same with idle lanes
                "lanes_per_instr": counts["lanes_link"], "pipe_frac": ach_l / peak64 * 32 / counts["lanes_link"],
                "k_voxels_lanes_per_instr": counts["lanes_voxel"],
                "k_voxels_pipe_frac": ach_v / peak64 * 32 / counts["lanes_voxel"]}
    traffic = counts["traffic_per_link"] * n_links if (counts and dom == "k_links" and counts.get("traffic_per_link")) else None
    return {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
            "algorithmic_bytes_per_launch": dom_b, "kernel_ms": dom_ms, "link_kernel_ms": link_ms, "voxel_kernel_ms": vox_ms,
            "contact_kernel_ms": con_ms, "traffic": traffic,
            "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum per k_links launch, per link "
                               f"({counts['source']}), times this run's links") if traffic else None,
            "fp64": fp64,
            "note": "the step kernels are bound by GB300's FP64 pipe, not by HBM: see roofline.fp64"}, n_links, n_vox


def measure_resident(ctx, ids, steps, warmup, dist=None, sample_clocks=True, device=0):
    """K batched steps of device-resident simulations, after W warm-up steps, timed with CUDA
    events on the context's stream; returns (device seconds, voxel-steps, launches, clocks, wall)."""
    import gpuvoxels_gb300 as g
    ctx.step(ids, warmup, g.BATCHED)
    if dist:
        dist.barrier()
    with ClockSampler(device) as clk:
        t0 = time.perf_counter()
        ctx.step(ids, steps, g.BATCHED)
        wall = time.perf_counter() - t0
    tm = ctx.timing()
    return tm["device_ms"] / 1e3, tm["voxel_steps"], tm["launches"], clk.summary(), wall


def workload_block(args, name, steps, full_steps, device, budget, peak64):
    """One more configuration measured in the same run: its own context, the autotuner's shape,
    W warm-up steps, then `steps` batched steps (a stated share of the configuration's
    `full_steps` when smaller), with its HBM and FP64 rooflines."""
    import gpuvoxels_gb300 as g
    t0 = time.perf_counter()
    cs, desc = make_workload(name, 0, args.batch)
    gen_s = time.perf_counter() - t0
    with g.Context(device, budget) as ctx:
        t0 = time.perf_counter()
        ids = ctx.load_many([c.vxa for c in cs], names=[f"{name}{i}" for i in range(len(cs))])
        ctx.step(ids, 1, g.BATCHED)
        load_s = time.perf_counter() - t0
        if not args.no_autotune:
            ctx.autotune(ids)
        dev_s, vsteps, launches, clocks, wall = measure_resident(ctx, ids, steps, args.warmup, device=device)
        link_ms, con_ms, vox_ms = kernel_times(ctx, ids)
        roof, n_links, n_vox = rooflines(ctx, ids, name, link_ms, con_ms, vox_ms, peak64)
        status = {}
        for i in ids:
            st = ctx.info(i).status
            status[st] = status.get(st, 0) + 1
        out = dict(workload=desc["workload"], simulations=len(cs), voxels=n_vox, links=n_links, value=vsteps / dev_s,
                   unit="voxel-steps/s", steps=steps, of_steps=full_steps,
                   share_note=(None if steps >= full_steps else
                               f"{steps} of the configuration's {full_steps} steps, timed as a bounded share of the run "
                               "(the per-step cost of a running simulation is steady)"),
                   ms_per_step=dev_s * 1e3 / steps, gpu_launches=launches, tuning=ctx.tuning(), roofline=roof,
                   clocks=clocks, status_counts={str(k): v for k, v in status.items()},
                   host_s=dict(generate=round(gen_s, 2), load_upload_first_step=round(load_s, 2)))
    return out


def serve_stream(args, device, budget, n_requests, rates):
    """The serving stream (seeded Poisson arrivals per offered rate) through the continuous-
    batching loop, and the plain per-simulation path on the same requests.

    Served: each request is parsed and loaded on arrival (vx3_load_vxa), queued with its horizon
    (vx3_submit) and advanced by vx3_poll, which admits queued requests as the context's HBM
    budget allows, advances every admitted one by --chunk-steps steps in one captured batch and
    retires finished ones.  Latency = completion (the poll that returned it) - arrival.
    Plain: one request at a time, in arrival order, each alone in PLAIN mode (one simulation
    per launch); every request is loaded and run for a bounded sample of its steps, and its
    service time is the measured load plus the measured per-step time times its horizon; the
    queue of the stream is then replayed first-come-first-served with those service times."""
    import itertools
    import gpuvoxels_gb300 as g
    from gpuvoxels_gb300 import synth
    t0 = time.perf_counter()
    reqs = synth.serving_requests(n_requests, seed=4)
    gen_s = time.perf_counter() - t0
    work = [c.num_voxel * h for c, h in reqs]
    # ---- plain arm: measured per-request service times
    service = []
    with g.Context(device, budget) as ctx:
        w = ctx.load_vxa(reqs[0][0].vxa, name="warm")
        ctx.step(w, 1, g.PLAIN)
        ctx.step(w, 32, g.PLAIN)
        ctx.free(w)
        for k, (c, h) in enumerate(reqs):
            a = time.perf_counter()
            sid = ctx.load_vxa(c.vxa, name=f"p{k}")
            ctx.step(sid, 1, g.PLAIN)
            b = time.perf_counter()
            n_s = max(1, min(h - 1, args.plain_sample_steps))
            ctx.step(sid, n_s, g.PLAIN)
            e = time.perf_counter()
            service.append((b - a) + (e - b) * (h - 1) / n_s)
            ctx.free(sid)
    pct = lambda xs, p: sorted(xs)[min(len(xs) - 1, int(round(p / 100.0 * (len(xs) - 1))))]
    out = []
    for ri, rate in enumerate(rates):
        rng = np.random.default_rng(5 + ri)
        arrivals = list(itertools.accumulate(rng.exponential(1.0 / rate, size=len(reqs))))
        # ---- served arm
        with g.Context(device, budget) as ctx:
            ctx.set_serving(args.serve_order, args.serve_cap_voxels)
            w = ctx.load_vxa(reqs[0][0].vxa, name="warm")
            ctx.submit(w, 256)
            while ctx.pending():
                for r in ctx.poll(args.chunk_steps):
                    ctx.free(r.id)
            lat, vsteps, k, arrival_of = [], 0, 0, {}
            t0 = time.perf_counter()
            last = t0
            while k < len(reqs) or ctx.pending():
                now = time.perf_counter() - t0
                while k < len(reqs) and arrivals[k] <= now:
                    c, horizon = reqs[k]
                    sid = ctx.load_vxa(c.vxa, name=f"r{k}")
                    ctx.submit(sid, horizon)
                    arrival_of[sid] = arrivals[k]
                    k += 1
                if ctx.pending():
                    done = ctx.poll(args.chunk_steps)
                    tnow = time.perf_counter() - t0
                    for r in done:
                        lat.append(tnow - arrival_of[r.id])
                        vsteps += r.num_voxel * r.steps
                        ctx.free(r.id)
                        last = time.perf_counter()
                elif k < len(reqs):
                    time.sleep(max(0.0, min(0.01, arrivals[k] - (time.perf_counter() - t0))))
            span = (last - t0) - arrivals[0]
        # ---- plain arm: the same arrivals, one request at a time in the same order policy
        free_at, plat, waiting, nxt = 0.0, [], [], 0
        while nxt < len(reqs) or waiting:
            if not waiting:
                free_at = max(free_at, arrivals[nxt])
            while nxt < len(reqs) and arrivals[nxt] <= free_at:
                waiting.append(nxt)
                nxt += 1
            # one request at a time: a lane for the longest changes nothing, so orders 1 and 2 are
            # the least work first
            pick = min(waiting, key=lambda i: (work[i], i)) if args.serve_order >= 1 else waiting[0]
            waiting.remove(pick)
            free_at += service[pick]
            plat.append(free_at - arrivals[pick])
        pspan = free_at - arrivals[0]
        served = vsteps / span
        plain = sum(work) / pspan
        out.append(dict(offered_req_per_s=rate, completed=len(lat), p50_latency_s=pct(lat, 50), p99_latency_s=pct(lat, 99),
                        served_voxel_steps_per_s=served, makespan_s=span,
                        plain_p50_latency_s=pct(plat, 50), plain_p99_latency_s=pct(plat, 99),
                        plain_voxel_steps_per_s=plain, plain_makespan_s=pspan, served_vs_plain=served / plain))
    vs = [c.num_voxel for c, _ in reqs]
    return dict(
        requests=len(reqs), voxels_min=min(vs), voxels_max=max(vs), voxel_steps_total=int(sum(work)),
        collide=int(sum(1 for c, _ in reqs if c.meta.get("collide"))), chunk_steps=args.chunk_steps,
        policy=dict(order={0: "first come first served", 1: "least voxels x horizon first",
                           2: "least voxels x horizon first, beside a lane for the most work queued"}[args.serve_order],
                    max_active_voxels=args.serve_cap_voxels, both_arms=True),
        stream=("Poisson arrivals at each offered rate (seeded); creatures with V log-uniform in [100, 1e5] (fill "
                "U(0.5, 0.9), 4 materials E log-uniform [1e5, 1e7] Pa), horizons U[1e3, 5e4] steps, 20% with "
                "self-collision; the same requests at every rate"),
        plain_arm=(f"each request alone in PLAIN mode (one simulation per launch): load + first step measured, then "
                   f"min(horizon, {args.plain_sample_steps}) steps measured and scaled to its horizon; the stream's "
                   "queue replayed with those service times, in the served arm's order (least work first for "
                   "orders 1 and 2, a lane being no use to one request at a time)"),
        plain_service_s_total=sum(service), generate_s=round(gen_s, 2), target_served_vs_plain=10.0, rates=out)


def run_ours(args):
    rank, ws, dist = dist_init()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import gpuvoxels_gb300 as g
    cs, desc = make_workload(args.workload, rank, args.batch)
    budget = int(args.budget_gb * (1 << 30))
    # ---- device-resident throughput
    ctx = g.Context(local, budget)
    prec = g.FMA if args.precision == "fma" else g.EXACT
    ctx.set_precision(prec)
    ids = [ctx.load_vxa(c.vxa, name=f"c{i}") for i, c in enumerate(cs)]
    ctx.step(ids, 1, g.BATCHED)                       # upload + first step
    if args.tuning:
        bl, bv, il, iv = (int(x) for x in args.tuning.split(","))
        ctx.set_tuning(bl, bv, il, iv, args.graph_steps)
    else:
        ctx.set_tuning(graph_steps=args.graph_steps)
    # a freshly loaded batch's first steps (creatures settling on the floor and starting to
    # move: many links change angle mode) are timed on their own; the line's value is timed
    # after `settle_steps` more, in the regime the rest of the run (tens of thousands of
    # steps for this configuration) stays in
    fdev_s, fvsteps, _, _, _ = measure_resident(ctx, ids, args.steps, args.warmup, dist, sample_clocks=False, device=local)
    fdev_s, fvsteps = reduce_timing(dist, fdev_s, fvsteps)
    fresh = dict(value=fvsteps / fdev_s, ms_per_step=fdev_s * 1e3 / args.steps,
                 window=f"steps {2 + args.warmup}-{1 + args.warmup + args.steps} of the run, launch shape before tuning")
    ctx.step(ids, args.settle_steps, g.BATCHED)
    if not args.tuning and not args.no_autotune:
        ctx.autotune(ids)                             # launch shape picked on the live batch
    tuning = ctx.tuning()
    first = 2 + 2 * args.warmup + args.steps + args.settle_steps
    dev_s, vsteps, launches, clocks, wall = measure_resident(ctx, ids, args.steps, args.warmup, dist, device=local)
    dev_s, vsteps = reduce_timing(dist, dev_s, vsteps)
    value = vsteps / dev_s
    link_ms, con_ms, vox_ms = kernel_times(ctx, ids)
    peak64 = None
    if args.precision == "exact":
        try:
            peak64 = fp64_peak_fma_per_s(local)
        except Exception:   # the FP64 roofline is reported beside the HBM one; its absence is not fatal
            peak64 = None
    roof, n_links, n_vox = rooflines(ctx, ids, args.workload, link_ms, con_ms, vox_ms, peak64)
    # ---- plain one-simulation-per-launch form against the batched form, on the same sample
    plain = None
    if args.workload == "batch" and rank == 0:
        sub = ids[:args.plain_sims]
        ctx.step(sub, 32, g.PLAIN)
        tp = ctx.timing()
        ctx.step(sub, 32, g.BATCHED)
        tb = ctx.timing()
        pv = tp["voxel_steps"] / (tp["device_ms"] / 1e3)
        bv = tb["voxel_steps"] / (tb["device_ms"] / 1e3)
        plain = dict(sample=f"first {len(sub)} creatures x 32 steps, both forms", plain_value=pv, batched_value=bv,
                     batched_vs_plain=bv / pv)
    ctx.close()
    # ---- end to end through the C ABI with host buffers: parse+load, upload, K steps, read back
    e2e = None
    if rank == 0:
        walls = []
        docs = [c.vxa.encode() for c in cs]      # the VXA files' bytes, as a caller holds them in host memory
        for _ in range(args.e2e_reps):           # each a fresh context: parse, upload, steps, read-back
            c2 = g.Context(local, budget)
            c2.set_precision(prec)
            c2.set_tuning(tuning["block_links"], tuning["block_voxels"], tuning["items_links"], tuning["items_voxels"],
                          tuning["graph_steps"])
            c2.set_claim_sizes(tuning["claim_links"], tuning["claim_voxels"])
            h0, d0 = c2.transfer_bytes()
            t0 = time.perf_counter()
            ids2 = c2.load_many(docs, names=[f"c{i}" for i in range(len(cs))])
            c2.step(ids2, args.steps, g.BATCHED)
            pos, q, fl, _ = c2.get_states(ids2)      # every creature's pose, one device pass and one copy
            walls.append(time.perf_counter() - t0)
            h1, d1 = c2.transfer_bytes()             # bytes the engine copied each way in the timed region
            h2d, d2h = h1 - h0, d1 - d0
            e2e_vs = sum(c2.info(i).num_voxel for i in ids2) * args.steps
            c2.close()
        e2e_wall = sorted(walls)[len(walls) // 2]
        e2e = dict(value=e2e_vs / e2e_wall, unit="voxel-steps/s", h2d_bytes_per_step=int(h2d / args.steps),
                   d2h_bytes_per_step=int(d2h / args.steps), runs_s=[round(w, 4) for w in walls],
                   note=f"median of {len(walls)} runs, each the wall clock of vx3_load_vxa_many (host VXA parse + "
                        "topology for every creature, on host threads), the upload, "
                        f"{args.steps} batched steps and vx3_get_states (every voxel's pose, one device pass and one copy)")
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    cpu = None
    if not args.no_cpu:
        v, cores, kind, sample = cpu_sample(cs, args.cpu_seconds)
        cpu = dict(value=v, unit="voxel-steps/s", cores=cores, kind=kind, sample=sample)
    modes = {}
    if plain:
        modes["plain_vs_batched"] = plain
    if args.workload == "batch" and ws == 1 and not args.no_modes:
        rates = [float(x) for x in args.serve_rates.split(",")]
        modes["serve"] = serve_stream(args, local, budget, args.serve_requests, rates)
        modes["collide"] = workload_block(args, "collide", args.collide_steps, 20000, local, budget, peak64)
        modes["slab"] = workload_block(args, "slab", args.slab_steps, 2000, local, budget, peak64)
    line = {
        "metric": "voxel-steps/sec (batched step of all simulations)",
        "value": value, "unit": "voxel-steps/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_s * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded creatures, no dataset)",
        "config": dict(desc, simulations=len(cs) * ws, voxels=n_vox * ws, links=n_links * ws, mode="batched",
                       kernel_build=args.precision, tuning=tuning,
                       tuning_source="vx3_autotune on the live batch" if not (args.tuning or args.no_autotune) else "set",
                       timed_window=f"steps {first}-{first + args.steps - 1} of the run (after {args.settle_steps} "
                                    f"settling steps; the configuration runs {RUN_STEPS.get(args.workload, 'more')})",
                       fresh_batch=fresh,
                       l2="device state larger than L2; no flush needed", parallelism=f"replicas x{ws} (no collective)"),
        "e2e": e2e,
        "gpu_launches": launches,
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "wall_s_timed": wall,
    }
    if modes:
        line["modes"] = modes
    print(json.dumps(line))


def run_serve(args):
    """The serving block alone (see serve_stream), as its own JSON line."""
    rates = [float(x) for x in args.serve_rates.split(",")]
    out = serve_stream(args, 0, int(args.budget_gb * (1 << 30)), args.serve_requests, rates)
    best = max(out["rates"], key=lambda r: r["served_voxel_steps_per_s"])
    line = {"metric": "served voxel-steps/s and completion latency (Poisson arrivals) vs the plain per-simulation path",
            "unit": "voxel-steps/s", "value": best["served_voxel_steps_per_s"], "n_gpus": 1, "higher_is_better": True,
            "dtype": "f64", "data": "synthetic (seeded creatures, no dataset)",
            "config": {"workload": f"serving stream: {out['requests']} requests per rate", "kernel_build": args.precision},
            "serve": out}
    print(json.dumps(line))


def profile_case(args):
    """A short, self-terminating run for ncu: the workload's kernels, one launch each per step."""
    import gpuvoxels_gb300 as g
    cs, desc = make_workload(args.workload, 0, args.batch, args.collide_sims, tuple(int(x) for x in args.slab_dims.split(",")))
    ctx = g.Context(0, int(args.budget_gb * (1 << 30)))
    ctx.set_precision(g.FMA if args.precision == "fma" else g.EXACT)
    ids = ctx.load_many([c.vxa for c in cs], names=[f"c{i}" for i in range(len(cs))])
    ctx.set_profiling(True)
    ctx.step(ids, args.profile_steps, g.BATCHED)
    t = ctx.timing()
    n_links = sum(ctx.info(i).num_link for i in ids)
    n_vox = sum(ctx.info(i).num_voxel for i in ids)
    print(json.dumps(dict(workload=desc["workload"], steps=args.profile_steps, voxels=n_vox, links=n_links,
                          link_ms=t["link_ms"], voxel_ms=t["voxel_ms"], contact_ms=t["contact_ms"])))
    ctx.close()


def run_reference(args):
    rank, ws, dist = dist_init()
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    cs, desc = make_workload(args.workload, 0, args.batch)
    threads = os.cpu_count() or 1
    vals = []
    for _ in range(min(args.steps, 3)):
        v, cores, kind, sample = cpu_sample(cs, args.cpu_seconds, threads)
        vals.append(v)
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": "voxel-steps/sec (batched step of all simulations)", "value": v,
            "unit": "voxel-steps/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded creatures, no dataset)",
            "config": dict(desc, simulations=len(cs)),
            "cpu_baseline": dict(value=v, unit="voxel-steps/s", cores=cores, kind=kind, sample=sample),
            "e2e": dict(value=v, unit="voxel-steps/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0)}
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--e2e-reps", type=int, default=3, help="end-to-end runs (fresh contexts); the median is reported")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch", choices=["batch", "slab", "collide", "plain", "serve"])
    ap.add_argument("--serve-requests", type=int, default=16, help="requests of the serving stream (per offered rate)")
    ap.add_argument("--serve-rates", default="50,200,2000", help="offered request rates (req/s) of the serving stream")
    ap.add_argument("--chunk-steps", type=int, default=64)
    ap.add_argument("--serve-order", type=int, default=1, choices=(0, 1, 2),
                    help="admission order: 0 first come first served, 1 least work first, 2 least work first beside a "
                         "lane for the most work queued")
    ap.add_argument("--serve-cap-voxels", type=int, default=150000,
                    help="most voxels in the running batch (0: the HBM budget decides); 150k voxels (~450k links) keep the "
                         "step kernels' resident warps busy several times over")
    ap.add_argument("--plain-sample-steps", type=int, default=256,
                    help="steps of each request measured in PLAIN mode for the plain arm of the serving stream")
    ap.add_argument("--collide-steps", type=int, default=2000, help="steps of the collision-heavy block (of 20,000)")
    ap.add_argument("--collide-sims", type=int, default=64, help="creatures of the collision workload for --profile-steps")
    ap.add_argument("--slab-steps", type=int, default=2000, help="steps of the single-body block (of 2,000)")
    ap.add_argument("--slab-dims", default="200,200,100", help="slab size X,Y,Z for --profile-steps (a smaller case for ncu)")
    ap.add_argument("--no-modes", action="store_true", help="skip the serving, collision and single-body blocks")
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--settle-steps", type=int, default=256,
                    help="untimed steps between the fresh-batch window and the timed window of the line's value")
    ap.add_argument("--budget-gb", type=float, default=64.0)
    ap.add_argument("--graph-steps", type=int, default=64)
    ap.add_argument("--tuning", default="", help="block_links,block_voxels,items_links,items_voxels (0 = keep); skips the autotuner")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--plain-sims", type=int, default=32)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--precision", default="exact", choices=["exact", "fma"])
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="profiling case for ncu: load the workload, run this many batched steps with one launch per "
                         "kernel (no graphs), print the per-kernel times and exit")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.profile_steps:
        profile_case(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
