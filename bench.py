#!/usr/bin/env python3
"""Throughput benchmark of the Dornic-split lattice integrator on GB300.

Workload (one "step" = one time step of every instance): the batched ragged
finite-size sweep of the DP Langevin model
    d rho = (a rho - b rho^2 + D Lap rho) dt + sigma sqrt(rho) dW,
    b = 2, D = 1, sigma = 1, dx = 1, dt = 0.1, Euler-exact remainder + Dornic draw,
L in {64, 128, 256, 512, 1024} x 32 replicates x 16 a-values log-spaced within
2 % of the critical point a_c = 0.530 (2560 instances, 715,128,832 sites), FP32
state with FP64 reductions, rho0 = 1 + U(-0.01, 0.01) (seed 0): every site is
live, so every site runs the full Poisson -> Gamma draw (the costly regime).
a_c is where the decay exponent of rho(t) crosses the 2-D DP value at
L = 512-1024 (measured by trophic_maelstorm_gb300.surrogate).  Synthetic inputs:
the reference ships no data for this path.

The second half of the metric, the full runs needed to locate a_c to +-1e-3,
is the `critical_point_search` extra: the surrogate-guided search against a
uniform sweep of [0.50, 0.56] (a reduced corpus, L <= 256, to keep the run short).

Metric: site-updates/s (one lattice site of one instance advanced one step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Profiling cases (not the metric): --workload l1024x64 (64 x 1024^2, fully active) and
l1024x64_dilute (half the sites empty).

--impl reference times the CPU restatement of the reference's step (the
oracle, OpenMP over instances, all host threads) on a bounded sample of the
same workload: the reference's sources are not on the benchmark machine.
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

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

LS = (64, 128, 256, 512, 1024)
REPS = 32
NA = 16
A_CENTER = 0.530          # measured critical point of b=2, D=1, sigma=1, dt=0.1
MODEL = dict(b=2.0, D=1.0, sigma=1.0, dt=0.1, dx=1.0)
BYTES_PER_SITE_FP32 = 8  # read rho, write rho (neighbours from registers/shuffles)
METRIC = "site-updates/s at L=1024 (batched FP32 vs plain FP64); runs to locate a_c \u00b11e-3"


def a_values():
    return list(np.geomspace(A_CENTER * 0.98, A_CENTER * 1.02, NA))


def workload(kind="sweep"):
    Ls, seeds, avs = [], [], []
    if kind in ("l1024x64", "l1024x64_dilute"):  # profiling cases: 64 instances of the L=1024 subset (268 MB per buffer)
        for r in range(64):
            Ls.append(1024); seeds.append(1_000_003 * r + 17); avs.append(float(a_values()[r % NA]))
        return Ls, seeds, avs
    from trophic_maelstorm_gb300.study import sweep_workload
    return sweep_workload(LS, REPS, NA, A_CENTER)


def init_field(L, rng):
    return (1.0 + rng.uniform(-0.01, 0.01, (L, L))).astype(np.float32)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0])); mx.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ dist helpers
def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if n_gpus > 1 else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, world):
    """Slowest rank's time (the job's time): all-reduce MAX over the process group
    (NCCL on GPU ranks, gloo on CPU)."""
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, seconds_per_rank, world):
    """Whole-job throughput of independent replicas: every rank's units over the
    slowest rank's time (weak scaling)."""
    return units_per_rank * world / max_over_ranks(seconds_per_rank, world)


# ------------------------------------------------------------------ CPU baseline
def cpu_sample(dtype=np.float32):
    """The bounded CPU sample of the sweep: one instance per (L, a) -- every lattice
    side and a-value of the workload in its proportions, 1/32 of its replicates
    (80 instances, 22.3 M sites per step) -- with the workload's keys and start."""
    Ls, seeds, avs = workload("sweep")
    pick = list(range(0, len(Ls), REPS))
    rng = np.random.default_rng(0)
    return ([Ls[i] for i in pick], [seeds[i] for i in pick], [avs[i] for i in pick],
            [init_field(Ls[i], rng).astype(dtype) for i in pick])


def cpu_run(steps, threads, dtype=np.float32):
    """The oracle (CPU restatement of the reference step) over the sample, OpenMP
    over instances; returns (site-updates/s, seconds)."""
    from oracle import oracle as o
    o.build()
    Ls, seeds, avs, fields = cpu_sample(dtype)
    params = [o.dp_params(a=a, **MODEL) for a in avs]
    t0 = time.perf_counter()
    o.dp_batch_run(params, Ls, seeds, fields, steps, threads)
    el = time.perf_counter() - t0
    return sum(L * L for L in Ls) * steps / el, el


def cpu_baseline(threads, budget_s=15.0):
    # calibrate on one step, then size the run to about budget_s seconds
    rate, el = cpu_run(1, threads)
    steps = max(1, int(budget_s / max(el, 1e-6)))
    rate, el = cpu_run(steps, threads)
    return {"value": rate, "unit": "site-updates/s", "cores": threads, "kind": "port",
            "sample": f"one instance per (L, a) of the sweep (80 instances, every L in {{64..1024}}, "
                      f"22.3 M sites) x {steps} steps from the fully active start, FP32 port, {el:.1f} s, "
                      f"OpenMP over instances"}


def workload_config(kind):
    """The config block both arms print for a workload."""
    return {"workload": "ragged DP Dornic sweep: L in {64..1024} x 32 replicates x 16 a (2560 instances)"
            if kind == "sweep" else f"profiling case {kind}",
            "sites_per_step": int(sum(L * L for L in workload(kind)[0])), "b": 2.0, "D": 1.0, "sigma": 1.0,
            "dt": 0.1, "a_values": f"16 log-spaced in [{a_values()[0]:.4f}, {a_values()[-1]:.4f}]",
            "init": "half the sites U(0, 0.5), the others 0" if kind == "l1024x64_dilute"
            else "1+U(-0.01,0.01), all sites live", "state": "FP32, FP64 reductions",
            "l2": f"inputs larger than L2 ({4 * sum(L * L for L in workload(kind)[0]) / 1e9:.2f} GB state per buffer)"}


def run_reference(args):
    rank, world, _ = dist_setup(args.gpus)
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    from oracle import oracle as o
    o.build()
    Ls, seeds, avs, fields = cpu_sample(np.float32)
    params = [o.dp_params(a=a, **MODEL) for a in avs]
    sites = sum(L * L for L in Ls)
    o.dp_batch_run(params, Ls, seeds, fields, args.warmup, threads)
    t0 = time.perf_counter()
    o.dp_batch_run(params, Ls, seeds, fields, args.steps, threads)
    el = time.perf_counter() - t0
    val = sites * args.steps / el
    # the reference computes in FP64: the FP64 port on the same sample, fewer steps
    Ls64, seeds64, avs64, f64 = cpu_sample(np.float64)
    n64 = max(2, args.steps // 4)
    t0 = time.perf_counter()
    o.dp_batch_run([o.dp_params(a=a, **MODEL) for a in avs64], Ls64, seeds64, f64, n64, threads)
    val64 = sites * n64 / (time.perf_counter() - t0)
    line = {
        "impl": "reference", "metric": METRIC, "value": val,
        "unit": "site-updates/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": dict(workload_config(args.workload), parallelism=f"host threads x{threads}"),
        "cpu_baseline": {"value": val, "unit": "site-updates/s", "cores": threads, "kind": "port",
                         "sample": "each step: one instance per (L, a) of the sweep -- 80 instances, every L in "
                                   "{64..1024} and every a in the sweep's proportions, 22.3 M sites -- from the "
                                   "fully active start, FP32 port, OpenMP over instances",
                         "fp64_port_value": val64,
                         "fp64_port_sample": f"the same sample in FP64 (the reference's arithmetic), {n64} steps",
                         "calibration": "on x86 the FP32 port runs at 1.00x (one core) and 1.17x (eight cores, one "
                                        "a per thread) the reference's own percolationDornic_2D at its production "
                                        "flags (profiles/cpu_reference_vs_port.md)"},
        "e2e": {"value": val, "unit": "site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ GPU arm
def load_traffic():
    p = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def plain_fp64(ctx, tmg, torch, args, steps=6):
    """The plain path the batched sweep is compared with: one FP64 instance at a time,
    each L of the sweep, timed per step; sweep throughput weights each L by its
    share of the sweep's instances (all equal)."""
    stream = torch.cuda.ExternalStream(ctx.stream)
    rng = np.random.default_rng(1)
    per_L = {}
    tot_sites = 0.0
    tot_time = 0.0
    for L in LS:
        inst = tmg.instances([L], [7], A_CENTER)
        b = tmg.Batch(ctx, tmg.dp_model(**MODEL), inst, tmg.TM_FP64)
        f0 = (1.0 + rng.uniform(-0.01, 0.01, (L, L)))
        b.upload([f0])
        b.enqueue_steps(2)
        ctx.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(steps):
                b.enqueue_steps(1)
            e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        per_L[str(L)] = {"ms_per_step": ms, "site_updates_per_s": L * L / (ms * 1e-3)}
        tot_sites += L * L
        tot_time += ms * 1e-3
        b.close()
    return {"sweep_site_updates_per_s": tot_sites / tot_time, "per_L": per_L,
            "note": "one FP64 instance per batch, same fully-active start; sweep figure = sum(L^2)/sum(step time)"}


def late_regime(ctx, tmg, torch, args, burn=600, steps=10):
    """Throughput later in the run: the 64 x 1024^2 subset after `burn` steps from the
    fully-active start (near-critical decay leaves most sites absorbing)."""
    stream = torch.cuda.ExternalStream(ctx.stream)
    Ls, seeds, avs = workload("l1024x64")
    inst = tmg.instances(Ls, seeds, avs)
    b = tmg.Batch(ctx, tmg.dp_model(**MODEL), inst, tmg.TM_FP32)
    rng = np.random.default_rng(2)
    b.upload([init_field(1024, rng) for _ in Ls])
    b.enqueue_steps(burn)
    obs, _ = b.advance(0, [b.step])
    active = float(obs[0, :, 1].sum()) / (len(Ls) * 1024 * 1024)

    def timed(n):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(n):
                b.enqueue_steps(1)
            e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / n

    ms = timed(steps)
    sites = len(Ls) * 1024 * 1024
    b.close()
    return {"burn_steps": burn, "t": burn * MODEL["dt"], "active_site_fraction": active, "ms_per_step": ms,
            "site_updates_per_s": sites / (ms * 1e-3),
            "hbm_frac": BYTES_PER_SITE_FP32 * sites / (ms * 1e-3) / 1e9 / peaks()[0]}


def rietkerk_4096(ctx, tmg, torch, args, steps=10, L=4096, precision=None):
    """The single large Rietkerk instance: 4096^2 three-field lattice, R = 0.9,
    sigma = 0.5, RK4 dt = 1e-3 (Dornic draw on P + fused RK4 of the remainder).
    Algorithmic traffic 24 B/site FP32 (read and write P, W, O once)."""
    stream = torch.cuda.ExternalStream(ctx.stream)
    precision = tmg.TM_FP32 if precision is None else precision
    inst = tmg.instances([L], [2024], 0.9)
    b = tmg.Batch(ctx, tmg.rietkerk_model(), inst, precision)
    rng = np.random.default_rng(3)
    dtype = np.float32 if precision == tmg.TM_FP32 else np.float64
    f0 = np.stack([rng.uniform(0, 1, (L, L)), np.full((L, L), 0.5), np.full((L, L), 1.0)]).astype(dtype)
    b.upload([f0])
    b.enqueue_steps(3)
    ctx.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        for _ in range(steps):
            b.enqueue_steps(1)
        e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    b.close()
    sites = L * L
    bps = (24 if precision == tmg.TM_FP32 else 48) * sites / (ms * 1e-3) / 1e9
    return {"L": L, "precision": "f32" if precision == tmg.TM_FP32 else "f64", "ms_per_step": ms,
            "site_updates_per_s": sites / (ms * 1e-3), "achieved_gbs_alg": bps, "hbm_frac": bps / peaks()[0],
            "kernels_per_step": 2}


def config0_plain_fp64(ctx, tmg, torch, steps=200):
    """Config 0: one 128^2 FP64 DP lattice, a ramped linearly 0.72 -> 0.70 over 1e4 steps, Euler-exact
    remainder, exact sampler; timed over `steps` steps of the ramp."""
    stream = torch.cuda.ExternalStream(ctx.stream)
    L, n_total = 128, 10000
    inst = tmg.instances([L], [0], 0.72, (0.70 - 0.72) / n_total)
    b = tmg.Batch(ctx, tmg.dp_model(**MODEL), inst, tmg.TM_FP64)
    b.upload([init_field(L, np.random.default_rng(0)).astype(np.float64)])
    b.enqueue_steps(32)
    ctx.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        b.enqueue_steps(steps)
        e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    b.close()
    return {"L": L, "precision": "f64", "ms_per_step": ms, "site_updates_per_s": L * L / (ms * 1e-3),
            "run_1e4_steps_s": ms * n_total * 1e-3}


def config1_rietkerk_batch(ctx, tmg, torch, steps=64):
    """Config 1: Rietkerk 256^2, R = linspace(0.6, 1.2, 8) x 16 replicates (128 instances), RK4 dt = 1e-3,
    P ~ U(0,1), W = 0.5, O = 1; per-step time in FP32 and FP64."""
    stream = torch.cuda.ExternalStream(ctx.stream)
    L = 256
    Rs = np.linspace(0.6, 1.2, 8)
    inst = tmg.instances([L] * 128, list(range(100, 228)), np.repeat(Rs, 16))
    rng = np.random.default_rng(4)
    f0 = [np.stack([rng.uniform(0, 1, (L, L)), np.full((L, L), 0.5), np.full((L, L), 1.0)]) for _ in range(128)]
    out = {}
    for name, prec in (("f32", tmg.TM_FP32), ("f64", tmg.TM_FP64)):
        b = tmg.Batch(ctx, tmg.rietkerk_model(), inst, prec)
        b.upload([f.astype(np.float32 if prec == tmg.TM_FP32 else np.float64) for f in f0])
        b.enqueue_steps(32)
        ctx.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            b.enqueue_steps(steps)
            e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        b.close()
        sites = 128 * L * L
        out[name] = {"ms_per_step": ms, "site_updates_per_s": sites / (ms * 1e-3),
                     "run_1e5_steps_s": ms * 1e5 * 1e-3}
    return out


def fke_advdiff_timing(ctx, L=1024, reps=5):
    """The consumer-movement operator (advdiff_FKE_MultiSp) on one L x L FP64 field:
    the GPU gather (tm_fke_advdiff_device, scratch allocation and synchronisation
    included) against the oracle's CPU scatter in the reference's loop order
    (one thread; this leg is a CPU baseline)."""
    import torch
    import trophic_maelstorm_gb300 as tmg
    from oracle import oracle as o
    rng = np.random.default_rng(5)
    rho = rng.uniform(0, 2, (L, L))
    rho[rng.random((L, L)) < 0.3] = 0.0
    gam = rng.uniform(0, 1, (L, L))
    vx = rng.uniform(-1, 1, (L, L))
    vy = rng.uniform(-1, 1, (L, L))
    p = tmg.fke_parameters(1.0, 1.0, 1.0, 1.5)
    dev = torch.device("cuda", ctx.device)
    ts = [torch.as_tensor(a, dtype=torch.float64, device=dev) for a in (rho, gam, vx, vy)]
    tmg.fke_advdiff(*ts, p)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(reps):
        out = tmg.fke_advdiff(*ts, p)
    torch.cuda.synchronize(dev)
    gpu_ms = (time.perf_counter() - t0) * 1e3 / reps
    o.build()
    t0 = time.perf_counter()
    ref = o.fke_advdiff(rho, gam, vx, vy, p.pref, p.gD, p.gV)
    cpu_ms = (time.perf_counter() - t0) * 1e3
    err = float(np.abs(out.cpu().numpy().reshape(-1) - ref).max() / np.abs(ref).max())
    return {"L": L, "RD": p.RD, "RV": p.RV, "gpu_ms": gpu_ms, "cpu_baseline_ms": cpu_ms, "cpu_threads": 1,
            "cpu_kind": "port (reference loop order)", "max_rel_diff": err}


def critical_point_search(ctx):
    """Full runs needed to locate a_c to +-1e-3: surrogate-guided (tensor-core MLP
    trained on a corpus of integrator runs) against a uniform sweep, judged by
    8 replicates at L = 256 to t = 1000."""
    from trophic_maelstorm_gb300 import surrogate as sg
    t0 = time.perf_counter()
    r = sg.critical_point_study(ctx, Ls=(64, 128, 256), n_a=40, n_rep=15, judge_L=256, judge_rep=8,
                                t_max=1000.0, t1=100.0, seed=1)
    return {"runs_guided": r["guided"]["runs"], "runs_uniform": r["uniform"]["runs"],
            "ratio": r["runs_ratio_uniform_over_guided"], "bracket_guided": r["guided"]["bracket"],
            "bracket_uniform": r["uniform"]["bracket"], "a_hat": r["surrogate_a_hat"],
            "corpus_runs": r["corpus"]["runs"], "corpus_site_updates_per_s":
                r["corpus"]["site_updates"] / r["corpus"]["seconds"],
            "fit_seconds": r["fit"]["seconds"], "fit_loss_last": r["fit"]["loss_last"],
            "judge": r["judge"], "wall_s": time.perf_counter() - t0}


def run_ours(args):
    import torch
    import trophic_maelstorm_gb300 as tmg

    rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    ctx = tmg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)

    Ls, seeds, avs = workload(args.workload)
    # every rank runs the full workload on its own GPU (independent replicas, weak scaling)
    seeds = [s + 7919 * rank for s in seeds]
    inst = tmg.instances(Ls, seeds, avs)
    sites = int(sum(L * L for L in Ls))
    model = tmg.dp_model(**MODEL)
    b = tmg.Batch(ctx, model, inst, tmg.TM_FP32)
    total = b.total

    # initial state in pinned host memory (used for the device upload and the e2e leg)
    rng = np.random.default_rng(0)
    host = torch.empty(total, dtype=torch.float32, pin_memory=True)
    hv = host.numpy()
    hv[:] = 0
    _, off, fs = tmg.layout(inst, 1)
    for k, L in enumerate(Ls):
        if args.workload == "l1024x64_dilute":   # a dilute lattice: half the sites empty, the rest U(0, 0.5)
            v = rng.uniform(0.0, 0.5, L * L).astype(np.float32)
            v[rng.random(L * L) < 0.5] = 0.0
            hv[off[k]: off[k] + L * L] = v
        else:
            hv[off[k]: off[k] + L * L] = rng.uniform(-0.01, 0.01, L * L).astype(np.float32) + np.float32(1.0)
    b.upload(hv)

    if args.autotune:
        b.autotune(2)
    rows, ctas = b.get_launch()

    # warm-up, then restore the initial state so the timed steps start fully active
    b.enqueue_steps(args.warmup)
    ctx.sync()
    b.upload(hv)

    # ---- value: K steps, each the fused step kernel and the deferred-site kernel, events per step
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    clk = ClockSampler(local)
    clk.start()
    barrier(world)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        ev[0].record(stream)
        for i in range(args.steps):
            b.enqueue_steps(1)
            ev[i + 1].record(stream)
    stream.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    clocks = clk.stop()
    per = [ev[i].elapsed_time(ev[i + 1]) for i in range(args.steps)]
    t_ms = ev[0].elapsed_time(ev[-1])
    t_ms = max_over_ranks(t_ms, world)
    value = sites * args.steps * world / (t_ms * 1e-3)

    # ---- e2e: public API with host buffers: H2D of the initial state from pinned memory,
    # K steps, observables (mean rho, active sites) read back at step 0 and step K
    e_steps = args.steps
    meas = [b.step, b.step + e_steps]
    obs_bytes = len(meas) * len(Ls) * 2 * 8
    if not args.no_e2e:
        # warm-up of the e2e leg: advance() replays 32-step CUDA graphs, built on first use
        b.enqueue_steps(32)
    torch.cuda.synchronize()
    barrier(world)
    st = np.zeros(0, np.uint32)
    e2e = None
    e2e_reps = []
    if not args.no_e2e:
        # one untimed pass through the same calls, then five timed ones (median reported, each
        # repetition's upload and advance times kept in the line: the host-to-device copy of the
        # 2.86 GB state shares the host link with the machine's other jobs and varies by 10x)
        b.upload(hv, step=0)
        b.advance(e_steps, [0, e_steps])
        for _ in range(5):
            torch.cuda.synchronize()
            barrier(world)
            t0 = time.perf_counter()
            b.upload(hv, step=0)
            t1 = time.perf_counter()
            obs, st = b.advance(e_steps, [0, e_steps])
            t2 = time.perf_counter()
            e2e_reps.append({"total_s": t2 - t0, "upload_s": t1 - t0, "advance_s": t2 - t1,
                             "upload_gbs": total * 4 / (t1 - t0) / 1e9})
        e2e_s = statistics.median(r["total_s"] for r in e2e_reps)
        e2e_s = max_over_ranks(e2e_s, world)
        e2e = sites * e_steps * world / e2e_s

    extras = {}
    if not args.no_extras:
        extras["plain_fp64_single_instance"] = plain_fp64(ctx, tmg, torch, args)
        extras["late_regime"] = late_regime(ctx, tmg, torch, args)
        extras["rietkerk_4096"] = rietkerk_4096(ctx, tmg, torch, args)
        extras["critical_point_search"] = critical_point_search(ctx)
        extras["fke_advdiff"] = fke_advdiff_timing(ctx)
        extras["config0_dp_128_fp64_ramp"] = config0_plain_fp64(ctx, tmg, torch)
        extras["config1_rietkerk_256x128"] = config1_rietkerk_batch(ctx, tmg, torch)

    hbm, peak_kind = peaks()
    avg_launch_s = statistics.mean(per) * 1e-3
    alg_bytes = BYTES_PER_SITE_FP32 * sites
    achieved = alg_bytes / avg_launch_s / 1e9
    tr = load_traffic().get("dornic_step_fp32_per_site_bytes")
    traffic = tr * sites if tr else None

    line = None
    if rank == 0:
        cpu = cpu_baseline(os.cpu_count() or 1, budget_s=args.cpu_budget) if not args.no_cpu else None
        line = {
            "metric": METRIC,
            "value": value, "unit": "site-updates/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": dict(workload_config(args.workload), launch={"rows_per_task": rows, "ctas_per_sm": ctas},
                           parallelism=f"replicas x{world}"),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": "Dornic step: dornic_step_kernel + dornic_deferred_kernel <float, euler, exact "
                                   "sampler> (timed together per step)", "alg_bytes_per_site": BYTES_PER_SITE_FP32,
                         "avg_launch_ms": avg_launch_s * 1e3},
            "cpu_baseline": cpu,
            "e2e": None if e2e is None else {"value": e2e, "unit": "site-updates/s",
                                             "h2d_bytes_per_step": total * 4 / e_steps,
                                             "d2h_bytes_per_step": obs_bytes / e_steps, "steps": e_steps,
                                             "timing": "median of 5 after one untimed pass",
                                             "repetitions": e2e_reps},
            "gpu_launches": 2 * args.steps,   # per step: the step kernel and the deferred-site kernel
            "clocks": clocks,
            "status_bits": int(np.bitwise_or.reduce(st)) if len(st) else 0,
            "extras": extras,
        }
        print(json.dumps(line), flush=True)
    b.close()
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="skip the launch-shape autotuner (it runs before the timed region)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--workload", default="sweep", choices=["sweep", "l1024x64", "l1024x64_dilute"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
