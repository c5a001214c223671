#!/usr/bin/env python
"""Voxel-steps/s of the Voxelyze3 soft-body step on GB300.

Default workload (N=1): the batched plain-physics configuration — 512
independent seeded creatures (cubic lattice side U{6..20}, fill U(0.3, 0.9),
largest 6-connected component, four materials with E log-uniform in
[1e5, 1e7] Pa, rho=1000, nu=0.35, one or two actuated at 5 Hz), gravity and
floor on, no self-collision, FP64, all creatures packed into shared launches.
A "step" is one physics step of the whole batch.  The batch's device state
(~1 GB) is larger than L2, so no flush is needed between timed iterations.

Other workloads (--workload): slab (a solid 200x200x100 body, 4M voxels),
collide (40^3 creatures at fill 0.5 with self-collision), serve (Poisson
request stream through the serving loop), plain (one 10^3 creature).

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
# per link and per voxel of one step of the batch workload, read by ncu at step 205
# (sm__thread_inst_executed_pipe_fp64_pred_on.sum ÷ links or voxels; profiles/k_links_k_voxels_batch512_steady.md).
FP64_INSTR_PER_LINK = 684878336 / 1627115      # 420.9
FP64_INSTR_PER_VOXEL = 236663360 / 844972      # 280.1
# DRAM bytes per link of one k_links launch at the same step (ncu dram__bytes_read.sum +
# dram__bytes_write.sum = 410.2 MB + 358.0 MB for 1,627,115 links).
LINK_TRAFFIC_PER_LINK = (410284544 + 358874112) / 1627115


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
def make_workload(name, rank=0, n_batch=512):
    from gpuvoxels_gb300 import synth
    if name == "batch":
        cs = synth.config1_batch(n_batch, seed=1 + 1000 * rank, sim_time=0.5)
        desc = dict(workload="batched plain physics: %d creatures, side U{6..20}, fill U(0.3,0.9), 4 materials E log-uniform "
                    "[1e5,1e7] Pa, nu=0.35, 5 Hz actuation, 0.01 m voxels, gravity+floor, no self-collision" % len(cs))
    elif name == "slab":
        cs = [synth.slab(200, 200, 100, seed=3 + rank)]
        desc = dict(workload="single large body: solid 200x200x100 slab (4M voxels), E=1e6, nu=0.35, per-voxel CTE actuation")
    elif name == "collide":
        cs = synth.config2_batch(16, seed=2 + rank)
        desc = dict(workload="collision-heavy: 16 creatures 40^3 fill 0.5, 3 materials incl. E=1e5, self-collision on "
                    "(64 in the full configuration)")
    elif name == "plain":
        cs = [synth.config0_creature(0)]
        desc = dict(workload="plain single creature: 10^3 lattice, fill 0.6, passive+active, 5 Hz +-39 C")
    else:
        raise ValueError(name)
    return cs, desc


def algorithmic_bytes(ctx, ids):
    """Compulsory DRAM bytes of one step (the kernels' data model)."""
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
    if args.autotune:
        ctx.autotune(ids)
    if args.tuning:
        bl, bv, il, iv = (int(x) for x in args.tuning.split(","))
        ctx.set_tuning(bl, bv, il, iv, args.graph_steps)
    else:
        ctx.set_tuning(graph_steps=args.graph_steps)
    ctx.step(ids, args.warmup, g.BATCHED)
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        ctx.step(ids, args.steps, g.BATCHED)
        wall = time.perf_counter() - t0
    tm = ctx.timing()
    dev_s = tm["device_ms"] / 1e3
    vsteps = tm["voxel_steps"]
    launches = tm["launches"]
    dev_s, vsteps = reduce_timing(dist, dev_s, vsteps)
    value = vsteps / dev_s
    # ---- per-kernel times (profiled steps: one launch per kernel, events on the context stream)
    ctx.set_profiling(True)
    lk, ck, vk = [], [], []
    for _ in range(5):
        ctx.step(ids, 1, g.BATCHED)
        t = ctx.timing()
        lk.append(t["link_ms"]); ck.append(t["contact_ms"]); vk.append(t["voxel_ms"])
    ctx.set_profiling(False)
    link_ms, vox_ms, con_ms = statistics.median(lk), statistics.median(vk), statistics.median(ck)
    link_b, vox_b = algorithmic_bytes(ctx, ids)
    dom = "k_links" if link_ms >= vox_ms else "k_voxels"
    dom_ms, dom_b = (link_ms, link_b) if dom == "k_links" else (vox_ms, vox_b)
    peak, peak_kind = measured_peaks()
    achieved = dom_b / (dom_ms / 1e3) / 1e9
    n_links = sum(ctx.info(i).num_link for i in ids)
    n_vox = sum(ctx.info(i).num_voxel for i in ids)
    # ---- the FP64 roofline that actually bounds both step kernels
    fp64 = None
    if args.workload == "batch" and args.precision != "exact":
        fp64 = {"unavailable": "FP64 instructions per link were counted (ncu) for the exact build, the one measured by default"}
    elif args.workload == "batch":
        try:
            peak64 = fp64_peak_fma_per_s(local)
            ach_l = FP64_INSTR_PER_LINK * n_links / (link_ms / 1e3)
            ach_v = FP64_INSTR_PER_VOXEL * n_vox / (vox_ms / 1e3)
            fp64 = {"bound": "fp64", "kernel": "k_links", "achieved": ach_l / 1e9, "peak": peak64 / 1e9,
                    "unit": "G FP64 thread-instructions/s", "frac": ach_l / peak64,
                    "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (FMA/s)",
                    "instr_per_link": FP64_INSTR_PER_LINK, "k_voxels_achieved": ach_v / 1e9, "k_voxels_frac": ach_v / peak64,
                    "instr_per_voxel": FP64_INSTR_PER_VOXEL}
        except Exception as e:   # the FP64 roofline is reported beside the HBM one; its absence is not fatal
            fp64 = {"unavailable": str(e)[:200]}
    # ---- plain one-simulation-per-launch form of the same kernels, on a sample of the batch
    plain = None
    if args.workload == "batch" and rank == 0:
        sub = ids[:args.plain_sims]
        ctx.step(sub, 32, g.PLAIN)
        tp = ctx.timing()
        ctx.step(sub, 32, g.BATCHED)
        tb = ctx.timing()
        plain = dict(sample=f"first {len(sub)} creatures x 32 steps", plain_value=tp["voxel_steps"] / (tp["device_ms"] / 1e3),
                     batched_value_same_sample=tb["voxel_steps"] / (tb["device_ms"] / 1e3),
                     full_batch_vs_plain=value / (tp["voxel_steps"] / (tp["device_ms"] / 1e3)))
    ctx.close()
    # ---- end to end through the C ABI with host buffers: parse+load, upload, K steps, read back
    e2e = None
    if rank == 0:
        walls = []
        for _ in range(args.e2e_reps):           # each a fresh context: parse, upload, steps, read-back
            c2 = g.Context(local, budget)
            c2.set_precision(prec)
            h0, d0 = c2.transfer_bytes()
            t0 = time.perf_counter()
            ids2 = c2.load_many([c.vxa for c in cs], names=[f"c{i}" for i in range(len(cs))])
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
    line = {
        "metric": "voxel-steps/sec (batched step of all simulations)",
        "value": value, "unit": "voxel-steps/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_s * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded creatures, no dataset)",
        "config": dict(desc, simulations=len(cs) * ws, voxels=n_vox * ws, links=n_links * ws, mode="batched",
                       kernel_build=args.precision,
                       l2="device state larger than L2; no flush needed", parallelism=f"replicas x{ws} (no collective)"),
        "e2e": e2e,
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
                     "algorithmic_bytes_per_launch": dom_b, "kernel_ms": dom_ms,
                     "link_kernel_ms": link_ms, "voxel_kernel_ms": vox_ms, "contact_kernel_ms": con_ms,
                     "traffic": LINK_TRAFFIC_PER_LINK * n_links if dom == "k_links" else None,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per k_links launch at step 205, "
                                       "per link, times this run's links",
                     "fp64": fp64,
                     "note": "the step kernels are bound by GB300's FP64 pipe, not by HBM: see roofline.fp64"},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "wall_s_timed": wall,
    }
    if plain:
        line["modes"] = plain
    print(json.dumps(line))


def run_serve(args):
    """Serving: requests arrive as a Poisson stream; each is parsed and loaded on arrival
    (vx3_load_vxa), queued (vx3_submit) and advanced by vx3_poll in chunks of --chunk-steps
    alongside every other admitted request, within the context's HBM budget.  Per offered
    rate: completion latency p50/p99 (submit to finish) and served voxel-steps/s."""
    import itertools
    import numpy as np
    import gpuvoxels_gb300 as g
    from gpuvoxels_gb300 import synth
    reqs = synth.serving_requests(args.serve_requests, seed=4)
    ctx = g.Context(0, int(args.budget_gb * (1 << 30)))
    ctx.set_precision(g.FMA if args.precision == "fma" else g.EXACT)
    # warm the kernels and graphs with one small request
    w = ctx.load_vxa(reqs[0][0].vxa, name="warm")
    ctx.submit(w, 256)
    while ctx.pending():
        for r in ctx.poll(args.chunk_steps):
            ctx.free(r.id)
    rates = [float(x) for x in args.serve_rates.split(",")]
    rng = np.random.default_rng(5)
    out = []
    for rate in rates:
        arrivals = list(itertools.accumulate(rng.exponential(1.0 / rate, size=len(reqs))))
        lat, vsteps, k = [], 0, 0
        t0 = time.perf_counter()
        while k < len(reqs) or ctx.pending():
            now = time.perf_counter() - t0
            while k < len(reqs) and arrivals[k] <= now:
                c, horizon = reqs[k]
                sid = ctx.load_vxa(c.vxa, name=f"r{k}")
                ctx.submit(sid, horizon)
                k += 1
            if ctx.pending():
                for r in ctx.poll(args.chunk_steps):
                    lat.append(r.finish_time_s - r.submit_time_s)
                    vsteps += r.num_voxel * r.steps
                    ctx.free(r.id)
            elif k < len(reqs):
                time.sleep(max(0.0, min(0.01, arrivals[k] - (time.perf_counter() - t0))))
        span = time.perf_counter() - t0
        lat.sort()
        pct = lambda p: lat[min(len(lat) - 1, int(round(p / 100.0 * (len(lat) - 1))))]
        out.append(dict(offered_req_per_s=rate, completed=len(lat), p50_latency_s=pct(50), p99_latency_s=pct(99),
                        served_voxel_steps_per_s=vsteps / span, makespan_s=span))
    ctx.close()
    line = {"metric": "served voxel-steps/s and completion latency (Poisson arrivals)", "unit": "voxel-steps/s",
            "value": max(o["served_voxel_steps_per_s"] for o in out), "n_gpus": 1, "higher_is_better": True,
            "dtype": "f64", "data": "synthetic (seeded creatures, no dataset)",
            "config": {"workload": f"serving: {len(reqs)} requests per rate, V log-uniform [100, 1e4], horizon U[1e3, 5e3] "
                                   f"steps, 20% with self-collision, chunk {args.chunk_steps} steps per poll",
                       "kernel_build": args.precision},
            "rates": out}
    print(json.dumps(line))


def profile_case(args):
    """A short, self-terminating run for ncu: the workload's kernels, one launch each per step."""
    import gpuvoxels_gb300 as g
    cs, desc = make_workload(args.workload, 0, args.batch)
    ctx = g.Context(0, int(args.budget_gb * (1 << 30)))
    ctx.set_precision(g.FMA if args.precision == "fma" else g.EXACT)
    ids = [ctx.load_vxa(c.vxa, name=f"c{i}") for i, c in enumerate(cs)]
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
    ap.add_argument("--serve-requests", type=int, default=64)
    ap.add_argument("--serve-rates", default="5,10,20,40", help="offered request rates (req/s) for --workload serve")
    ap.add_argument("--chunk-steps", type=int, default=64)
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--budget-gb", type=float, default=64.0)
    ap.add_argument("--graph-steps", type=int, default=64)
    ap.add_argument("--tuning", default="", help="block_links,block_voxels,items_links,items_voxels (0 = keep)")
    ap.add_argument("--autotune", action="store_true")
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
