#!/usr/bin/env python3
"""Throughput of the single-rank `--fc tree` Barnes-Hut step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Metric: body-steps/s (bodies x steps / second) of the full step of
src/main.cpp:191-282 -- kick, drift, bounding box, Morton keys, radix sort,
permutation, octree build with the single-rank merge, forces, kick -- on the
plain FP64 theta = 1.05 workload of 300,149 bodies (Sun, 8 planets, 300,140
asteroids of which 10 % in the outer belt), dt = 1 h.  Inputs are synthetic
and seeded (the reference's 300k CSV is not part of its repository).

* value: device time (CUDA events on the engine's stream), state resident in
  HBM, L2 flushed (256 MiB write) before every timed step.
* e2e: the same steps through the C ABI with the state on the host: each
  step is one bh_step_host call, which uploads pos, vel, mass, ids and acc
  from pinned memory, runs the step and downloads them again (host clock
  around the calls).
* roofline: the force kernel (the dominant phase) against the FP64 FMA peak
  measured in the same process; algorithmic work = 20 flops per accepted
  interaction (the conventional monopole count), interactions counted on the
  device.
* cpu_baseline: the oracle (C restatement of the reference's path, OpenMP,
  every host core) on the same workload, a bounded number of steps.
* hbm_phases: achieved GB/s of the data-movement phases (algorithmic bytes
  per body / phase time) against the measured HBM copy bandwidth.
* forms_4m: 4M bodies (85/10/5 with trojans), plain FP64 theta = 1.05
  against the FP32 far field over a theta sweep (1.05-2.0) and FP32 + learned
  criterion at several per-body error budgets (network trained first on 20
  seeded 1M-body systems, ~10M pairs, by the engine's GPU kernels); the
  line's top-level benchmark spec object summarises it (learned against plain
  FP64 at equal or lower error, and against the fastest theta-only run at
  the learned run's error) with the FP32 walk's roofline.
* learned_eval: the learned criterion on 5 unseen 1M-body systems at the
  same budgets against the same theta sweep, with its fallback rate.
* learned_high_accuracy: the learned criterion with theta = 0.5 as its
  fallback and a network trained for it, at budgets 3e-9-3e-7, against
  finer theta sweeps (0.35-0.8) on an unseen 1M-body system.
* precision_run: the FP32 far-field form on 1M bodies at theta {0.5, 0.8,
  1.05}, then 1,000 steps with error, energy and angular-momentum drift every
  100 steps.
* long_runs: the configurations' own run lengths -- 240 steps of the 19,054-
  body system in the bit-exact form (final state compared with the compiled
  reference's run), 2,000 steps of the 300k FP64 list workload and 500 steps
  of the 4M FP32 + learned form -- each timed as one span, with the final
  error and the energy/angular-momentum drift.
* let_exchange: the locally essential tree export and import at 4M bodies
  split over 8 ranks, against the oracle on the host cores.
* csv_ingest: readCSV of a 1M-body file on the GPU against the host reader.
  --no-extras skips these seven blocks; --blocks a,b runs only those.

Multi-GPU: the path does not shard on one GPU per rank; ranks run replicas
(weak scaling) and value is the sum of their body-steps over the slowest
rank's time.  `--impl reference` times the reference's CPU path (the oracle
port on hosts without the reference checkout) on rank 0 only.
"""
from __future__ import annotations

import argparse
import gc
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

G = 1.48812e-34
THETA = 1.05
DT = 1.0 / 24.0
N_BODIES = 300_149
SEED = 2
FLOPS_PER_INTERACTION = 20
L2_FLUSH_BYTES = 256 << 20
EXTRA_BLOCKS = ("forms_4m", "learned_eval", "learned_high_accuracy", "precision_run", "long_runs", "let_exchange",
                "csv_ingest")
WORKLOAD = "plain FP64 theta=1.05, dt=1h, 300,149 bodies (Sun, 8 planets, 300,140 asteroids, 10% outer belt)"
MODES = {"plain": 0, "fp64_list": 1, "fp32": 2, "learned": 3, "fp32_group": 4}
KERNEL = {0: "traverse_exact_kernel", 1: "traverse_masked_kernel<fp64>", 2: "traverse_masked_kernel<fp32>",
          3: "traverse_learned_kernel", 4: "traverse_masked_kernel<fp32, group>"}


def workload_name(args) -> str:
    if args.bodies == N_BODIES and args.mode == "fp64_list" and args.theta == THETA and args.outer == 0.1 \
            and args.trojan == 0.0:
        return WORKLOAD
    return (f"{args.mode} theta={args.theta}, dt=1h, {args.bodies:,} bodies (Sun, 8 planets, "
            f"{args.bodies - 9:,} asteroids, {args.outer:.0%} outer belt, {args.trojan:.0%} trojans)")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--bodies", type=int, default=N_BODIES)
    ap.add_argument("--mode", default="fp64_list", choices=list(MODES))
    ap.add_argument("--outer", type=float, default=0.10, help="outer-belt fraction of the asteroids")
    ap.add_argument("--trojan", type=float, default=0.0, help="Jupiter-trojan fraction of the asteroids")
    ap.add_argument("--theta", type=float, default=THETA)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="budget of the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--blocks", default=None,
                    help="comma-separated subset of the extra blocks: " + ",".join(EXTRA_BLOCKS))
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the 4M-body comparison, the learned evaluation and the 1M precision run")
    ap.add_argument("--ns-bodies", type=int, default=4_000_000)
    ap.add_argument("--ns-steps", type=int, default=3)
    ap.add_argument("--train-pairs", type=int, default=10_000_000, help="learned criterion: training pairs")
    ap.add_argument("--pr-bodies", type=int, default=1_000_000, help="precision run: bodies")
    ap.add_argument("--pr-steps", type=int, default=1000, help="precision run: steps at theta=1.05")
    ap.add_argument("--theta-max", type=float, default=3.0, help="learned criterion: candidate range")
    ap.add_argument("--budget", type=float, default=3e-6, help="learned criterion: per-body error budget")
    return ap.parse_args()


def dist_init():
    """Rank, world size and local rank from the launcher's environment; one
    process per GPU over NCCL (gloo where no GPU is present, for the host-side
    replica logic)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist.init_process_group("gloo")
    return rank, ws, local


class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, window=None):
        """Median SM clock and the throttle reasons seen over every sample
        (the pre-roll and the timed steps); samples_timed counts those that
        arrived within `window` (perf_counter start, end)."""
        sm, mx, reasons, inside = [], None, set(), 0
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ts, ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            if window and window[0] <= ts <= window[1]:
                inside += 1
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        out = {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
               "samples": len(sm)}
        if window:
            out["samples_timed"] = inside
            out["window"] = "200 ms samples over a 1 s untimed pre-roll of the same step and the timed steps"
        return out


def cpu_baseline(pos, vel, mass, ids, budget_s: float, theta: float = THETA, nsteps_max: int = 20):
    """Times the oracle's step loop on all host cores for a bounded sample."""
    from oracle.oracle import Oracle
    o = Oracle("port")
    kind = "port"
    try:
        ref = Oracle("reference")
        o, kind = ref, "reference"
    except (FileNotFoundError, OSError):
        pass
    n = len(mass)
    t0 = time.perf_counter()
    p, v, m, i, a, t, _ = o.simulate(pos, vel, mass, ids, DT, theta, G, 1)
    first = time.perf_counter() - t0
    extra = max(0, min(nsteps_max - 1, int(budget_s / max(first, 1e-3)) - 1))
    t1 = time.perf_counter()
    if extra:
        o.simulate(p, v, m, i, DT, theta, G, extra, t=t, acc=a)
    rest = time.perf_counter() - t1
    steps = 1 + extra
    secs = first + rest
    cores = Oracle("port").threads()
    return {"value": n * steps / secs, "unit": "body-steps/s", "cores": cores, "kind": kind,
            "sample": f"{steps} full steps of the {n:,}-body workload ({secs:.1f} s, OpenMP {cores} threads)"}


DATA = "synthetic (seeded solar system: the engine's generator; the reference arm uses its bit-exact restatement)"


def bench_config(args, n: int, ws: int) -> dict:
    """The workload description both arms print (same keys and values)."""
    return {"workload": workload_name(args), "bodies": n, "theta": args.theta, "dt_days": DT, "mode": args.mode,
            "seed": SEED, "outer": args.outer, "trojan": args.trojan,
            "l2": "flushed before every timed step (256 MiB write)", "parallelism": f"replicas x{ws}"}


def run_reference(args, rank):
    """The reference arm: the reference's CPU path (its compiled sources
    where they were built on this host, else the oracle port) on every host
    core, rank 0 only.  The inputs come from the oracle's restatement of the
    seeded generator, so this arm loads nothing of the engine."""
    if rank != 0:
        return
    from oracle.oracle import Oracle
    port = Oracle("port")
    pos, vel, mass, ids = port.generate_system(SEED, args.bodies, args.outer, args.trojan)
    o, kind = port, "port"
    try:
        o, kind = Oracle("reference"), "reference"
    except (FileNotFoundError, OSError):
        pass
    n = len(mass)
    theta = args.theta
    # Warm-up steps, then timed steps; both capped so the run ends in minutes.
    t0 = time.perf_counter()
    p, v, m, i, a, t, _ = o.simulate(pos, vel, mass, ids, DT, theta, G, 1)
    one = time.perf_counter() - t0
    warm = 1 + max(0, min(args.warmup - 1, int(30.0 / max(one, 1e-3))))
    if warm > 1:
        p, v, m, i, a, t, _ = o.simulate(p, v, m, i, DT, theta, G, warm - 1, t=t, acc=a)
    k = max(1, min(args.steps, int(120.0 / max(one, 1e-3))))
    t0 = time.perf_counter()
    o.simulate(p, v, m, i, DT, theta, G, k, t=t, acc=a)
    secs = time.perf_counter() - t0
    val = n * k / secs
    cores = port.threads()
    what = "the reference's own sources compiled on this host" if kind == "reference" else \
        "the oracle port (C restatement of the reference's path; the reference checkout is not on this host)"
    line = {"metric": "body-steps/s", "value": val, "unit": "body-steps/s", "n_gpus": args.gpus, "steps": k,
            "warmup": warm, "ms_per_step": 1e3 * secs / k, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": DATA, "impl": "reference",
            "config": bench_config(args, n, args.gpus),
            "reference_impl": f"CPU, {what}, OpenMP {cores} threads",
            "cpu_baseline": {"value": val, "unit": "body-steps/s", "cores": cores, "kind": kind,
                             "sample": f"{k} timed full steps after {warm} warm-up steps, OpenMP {cores} threads"},
            "e2e": {"value": val, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def time_steps(ctx, ext, flush, mode, theta, steps, warmup, t=0.0):
    """Device ms per step (CUDA events on the engine's stream, L2 flushed
    before each step) and accepted interactions per body of the last step."""
    import torch
    for _ in range(warmup):
        t = ctx.step(DT, theta, G, 1, mode, t=t)
    ms = []
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        t = ctx.step(DT, theta, G, 1, mode, t=t)
        e1.record(ext)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    return sum(ms) / len(ms), ctx.interaction_count() / ctx.n


def train_model(args):
    """The learned criterion's network, trained by the engine's own GPU
    kernels on pairs labelled by the plain walk at theta = 0.5: 20 seeded
    1M-body systems (10 with the 90/10 inner/outer belt mix, 10 with the
    85/10/5 mix that adds trojans), about 10M pairs."""
    learned = importlib.import_module("barnes-hut_gb300.learned")
    t0 = time.perf_counter()
    nb = min(args.ns_bodies, 1_000_000)
    half = args.train_pairs // 2
    F1, L1 = learned.collect_pairs(range(9001, 9011), nb, 0.10, 0.0, theta_max=args.theta_max, max_pairs=half)
    F2, L2 = learned.collect_pairs(range(9011, 9021), nb, 0.10, 0.05, theta_max=args.theta_max, max_pairs=half)
    F = np.concatenate([F1, F2]); L = np.concatenate([L1, L2])
    bh = importlib.import_module("barnes-hut_gb300")
    params, scale, losses = bh.mlp_train(F, L, epochs=6, batch=4096, lr=2e-3, seed=0)
    info = {"pairs": int(len(L)), "systems": 20, "system_bodies": nb, "epochs": 6,
            "final_loss": float(losses[-1]), "seconds": time.perf_counter() - t0, "label_theta": 0.5,
            "theta_max": args.theta_max, "seeds": "9001-9020"}
    return params, scale, info


def _sample_error(ctx, n, G_):
    rng = np.random.default_rng(0)
    sample = np.sort(rng.choice(n, min(n, 4096), replace=False))
    ref = ctx.direct_sum(sample, G_)

    def err(a):
        e = np.linalg.norm(a[sample] - ref, axis=1) / np.linalg.norm(ref, axis=1)
        return float(np.median(e)), float(np.quantile(e, 0.99))
    return err


def _fresh(ctx, pos, vel, mass, ids):
    ctx.set_bodies(pos, vel, mass, ids)
    ctx.compute_bbox(); ctx.compute_keys(); ctx.sort_bodies(); ctx.build_tree()


def long_run(dev, n, frac_outer, frac_trojan, seed, mode_name, steps, params=None, scale=None, budget=None,
             theta_max=3.0):
    """A run of the configuration's own length: `steps` steps through the
    step loop (graph replay after the first) timed as one span of CUDA events
    on the engine's stream, then the error against the FP64 direct sum on a
    4,096-body sample and the drift of energy and angular momentum."""
    import torch
    bh = importlib.import_module("barnes-hut_gb300")
    mode = MODES[mode_name]
    pos, vel, mass, ids = bh.generate_system(seed, n, frac_outer, frac_trojan)
    with bh.Context(n, dev) as ctx:
        ext = torch.cuda.ExternalStream(ctx.stream(), device=dev)
        if budget is not None:
            ctx.learned_set_model(params, scale, budget=budget, theta_max=theta_max)
        ctx.set_bodies(pos, vel, mass, ids)
        inv0 = ctx.invariants(G, THETA)
        ctx.set_bodies(pos, vel, mass, ids)
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        t = ctx.step(DT, THETA, G, steps, mode, t=0.0)
        e1.record(ext)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        inv = ctx.invariants(G, THETA)
        rng = np.random.default_rng(7)
        sample = np.sort(rng.choice(n, min(n, 4096), replace=False))
        ref = ctx.direct_sum(sample, G)
        a = ctx.compute_accelerations(THETA, G, 0.0, mode)
        e = np.linalg.norm(a[sample] - ref, axis=1) / np.linalg.norm(ref, axis=1)
    return {"bodies": n, "mode": mode_name, "budget": budget, "steps": steps, "simulated_days": t,
            "ms_total": ms, "body_steps_per_s": n * steps / (ms * 1e-3),
            "final_median_rel_err": float(np.median(e)), "final_p99_rel_err": float(np.quantile(e, 0.99)),
            "rel_energy_drift": float((inv["E"] - inv0["E"]) / abs(inv0["E"])),
            "rel_angular_momentum_drift": float(np.linalg.norm(inv["L"] - inv0["L"]) / np.linalg.norm(inv0["L"]))}


def config1_run(dev):
    """The CPU-runnable configuration's whole run: 240 steps of 1 h at theta
    1.05 on the 19,054-body system in the bit-exact form, from the inputs
    stored with the test fixtures, timed as one span; the final state's
    SHA-256 is compared with the compiled reference's own 240-step run
    (tests/golden/config1_240_steps.json)."""
    import hashlib
    import torch
    bh = importlib.import_module("barnes-hut_gb300")
    g = np.load(ROOT / "tests" / "golden" / "synthetic_19054.npz")
    want = json.loads((ROOT / "tests" / "golden" / "config1_240_steps.json").read_text())
    n = len(g["mass"])
    with bh.Context(n, dev) as ctx:
        ext = torch.cuda.ExternalStream(ctx.stream(), device=dev)
        ctx.set_bodies(g["pos"], g["vel"], g["mass"], g["ids"])
        ctx.step(DT, THETA, G, 3, MODES["plain"], t=0.0)  # warm-up, then the run from the start
        ctx.set_bodies(g["pos"], g["vel"], g["mass"], g["ids"])
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        t = ctx.step(DT, THETA, G, 240, MODES["plain"], t=0.0)
        e1.record(ext)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        state = ctx.get_bodies()
    h = hashlib.sha256()
    for a in state:
        h.update(np.ascontiguousarray(a).tobytes())
    return {"bodies": n, "mode": "plain (bit-exact)", "steps": 240, "simulated_days": t, "ms_total": ms,
            "body_steps_per_s": n * 240 / (ms * 1e-3),
            "final_state_bits_equal_reference": h.hexdigest() == want["digest"] and t == want["t"]}


def precision_run(args, dev):
    """The precision form on 1M bodies (90/10 inner/outer belt): FP32 far field
    with FP64 displacements, direct terms and state.  Error against the FP64
    direct sum at theta in {0.5, 0.8, 1.05}; then a run of --pr-steps steps at
    theta = 1.05 with the error on the 4,096-body sample and the energy and
    angular momentum every 100 steps."""
    import torch
    bh = importlib.import_module("barnes-hut_gb300")
    n = args.pr_bodies
    pos, vel, mass, ids = bh.generate_system(SEED + 2, n, 0.10, 0.0)
    out = {"workload": f"{n:,} bodies (Sun, 8 planets, 90% inner belt, 10% outer belt), fp32 far field, dt=1h"}
    with bh.Context(n, dev) as ctx:
        ext = torch.cuda.ExternalStream(ctx.stream(), device=dev)
        flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{dev}")
        _fresh(ctx, pos, vel, mass, ids)
        err = _sample_error(ctx, n, G)
        thetas = {}
        for th in (0.5, 0.8, 1.05):
            _fresh(ctx, pos, vel, mass, ids)
            med, p99 = err(ctx.compute_accelerations(th, G, 0.0, bh.MODE_FP32_FAR))
            ctx.set_bodies(pos, vel, mass, ids)
            ms, ipb = time_steps(ctx, ext, flush, bh.MODE_FP32_FAR, th, 3, 2)
            thetas[f"{th:g}"] = {"median_rel_err": med, "p99_rel_err": p99, "ms_per_step": ms,
                                 "body_steps_per_s": n / (ms * 1e-3), "interactions_per_body": ipb}
        out["theta"] = thetas
        ctx.set_bodies(pos, vel, mass, ids)
        inv0 = ctx.invariants(G, THETA)
        series = []
        t, done = 0.0, 0
        t0 = time.perf_counter()
        while done < args.pr_steps:
            k = min(100, args.pr_steps - done)
            t = ctx.step(DT, THETA, G, k, bh.MODE_FP32_FAR, t=t)
            done += k
            inv = ctx.invariants(G, THETA)
            rng = np.random.default_rng(done)
            sample = np.sort(rng.choice(n, 4096, replace=False))
            ref = ctx.direct_sum(sample, G)
            a = ctx.compute_accelerations(THETA, G, 0.0, bh.MODE_FP32_FAR)
            e = np.linalg.norm(a[sample] - ref, axis=1) / np.linalg.norm(ref, axis=1)
            series.append({"step": done, "median_rel_err": float(np.median(e)),
                           "p99_rel_err": float(np.quantile(e, 0.99)),
                           "rel_energy_drift": float((inv["E"] - inv0["E"]) / abs(inv0["E"])),
                           "rel_angular_momentum_drift": float(np.linalg.norm(inv["L"] - inv0["L"]) /
                                                               np.linalg.norm(inv0["L"]))})
        out["run"] = {"steps": done, "seconds": time.perf_counter() - t0, "every_100_steps": series,
                      "energy": "K exact; U: pairs with the Sun or a planet exact in FP64, the rest through the tree"}
    return out


LEARNED_BUDGETS = (1e-6, 3e-6, 1e-5, 3e-5)  # per-body error budgets of the learned criterion
THETA_SWEEP = (1.05, 1.3, 1.6, 2.0)          # the FP32 form with the theta test alone


def learned_eval(args, dev, params, scale):
    """The learned criterion on 5 unseen 1M-body systems (90/10 mix) at
    per-body error budgets, theta = 1.05 the fallback, against the FP32
    walk with the theta test alone over a theta sweep (1.05-2.0), each on
    the same state."""
    import torch
    bh = importlib.import_module("barnes-hut_gb300")
    n = min(args.ns_bodies, 1_000_000)
    rows = []
    cases = [(f"theta_{th:g}", bh.MODE_FP32_FAR, None, th) for th in THETA_SWEEP]
    cases += [(f"group_theta_{th:g}", bh.MODE_FP32_GROUP, None, th) for th in THETA_SWEEP]
    cases += [(f"budget_{b:g}", bh.MODE_LEARNED, b, THETA) for b in LEARNED_BUDGETS]
    with bh.Context(n, dev) as ctx:
        ext = torch.cuda.ExternalStream(ctx.stream(), device=dev)
        flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{dev}")
        for seed in range(9101, 9106):
            pos, vel, mass, ids = bh.generate_system(seed, n, 0.10, 0.0)
            _fresh(ctx, pos, vel, mass, ids)
            err = _sample_error(ctx, n, G)
            row = {"seed": seed}
            for name, mode, budget, theta in cases:
                if budget is not None:
                    ctx.learned_set_model(params, scale, budget=budget, theta_max=args.theta_max)
                _fresh(ctx, pos, vel, mass, ids)
                med, p99 = err(ctx.compute_accelerations(theta, G, 0.0, mode))
                r = {"median_rel_err": med, "p99_rel_err": p99}
                if budget is not None:
                    st = ctx.learned_stats()
                    r["fallback_rate"] = st["fallback"] / max(1, st["candidates"])
                    r["network_decided"] = st["accepted"] / max(1, st["candidates"])
                ctx.set_bodies(pos, vel, mass, ids)
                ms, ipb = time_steps(ctx, ext, flush, mode, theta, 2, 1)
                r.update({"ms_per_step": ms, "interactions_per_body": ipb})
                row[name] = r
            rows.append(row)
    summary = {name: {k: float(np.mean([r[name][k] for r in rows])) for k in rows[0][name]}
               for name, *_ in cases}
    return {"workload": f"{n:,} bodies (90/10), 5 unseen seeds 9101-9105, theta=1.05 fallback",
            "mean_over_seeds": summary, "comparison": _against_theta(summary), "per_seed": rows}


def learned_high_accuracy(args, dev):
    """The learned criterion where the theta test must be fine: theta = 0.5
    as its fallback, a network trained on pairs collected at theta = 0.5 and
    labelled by the walk at theta = 0.3 (six seeded 1M-body systems, 90/10),
    per-body budgets 3e-9 to 3e-7, against the FP32 per-body and group theta
    sweeps, on an unseen 1M-body system: interactions per body, median error
    against the FP64 direct sum, and force time (one walk, L2 flushed)."""
    import torch
    bh = importlib.import_module("barnes-hut_gb300")
    learned = importlib.import_module("barnes-hut_gb300.learned")
    n = min(args.ns_bodies, 1_000_000)
    t0 = time.perf_counter()
    F, L = learned.collect_pairs(range(9201, 9207), n, 0.10, 0.0, theta=0.5, theta_label=0.3, theta_max=3.0,
                                 max_pairs=6_000_000)
    params, scale, losses = bh.mlp_train(F, L, epochs=6, batch=4096, lr=2e-3, seed=0)
    info = {"pairs": int(len(L)), "systems": 6, "seeds": "9201-9206", "collect_theta": 0.5, "label_theta": 0.3,
            "final_loss": float(losses[-1]), "seconds": time.perf_counter() - t0}
    pos, vel, mass, ids = bh.generate_system(9301, n, 0.10, 0.0)
    rows = {}
    with bh.Context(n, dev) as ctx:
        ext = torch.cuda.ExternalStream(ctx.stream(), device=dev)
        flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{dev}")
        _fresh(ctx, pos, vel, mass, ids)
        err = _sample_error(ctx, n, G)
        cases = [(f"theta_{th:g}", bh.MODE_FP32_FAR, th, None) for th in (0.35, 0.4, 0.45, 0.5, 0.6, 0.7, 0.8)]
        cases += [(f"group_theta_{th:g}", bh.MODE_FP32_GROUP, th, None) for th in (0.4, 0.5, 0.6, 0.7, 0.8)]
        cases += [(f"budget_{b:g}", bh.MODE_LEARNED, 0.5, b) for b in (3e-9, 1e-8, 3e-8, 1e-7, 3e-7)]
        for name, mode, th, b in cases:
            if b is not None:
                ctx.learned_set_model(params, scale, budget=b, theta_max=3.0)
            med, p99 = err(ctx.compute_accelerations(th, G, 0.0, mode))
            ipb = ctx.interaction_count() / n
            ms = []
            for _ in range(4):
                flush.fill_(1.0)
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(ext)
                ctx.compute_accelerations(th, G, 0.0, mode, download=False)
                e1.record(ext)
                e1.synchronize()
                ms.append(e0.elapsed_time(e1))
            rows[name] = {"theta": th, "budget": b, "median_rel_err": med, "p99_rel_err": p99,
                          "interactions_per_body": ipb, "force_ms": sorted(ms)[1]}
    cmp = {}
    thetas = {k: r for k, r in rows.items() if not k.startswith("budget_")}
    for k, r in rows.items():
        if not k.startswith("budget_"):
            continue
        ok = [t for t in thetas.values() if t["median_rel_err"] <= r["median_rel_err"]]
        if ok:
            fewest = min(ok, key=lambda t: t["interactions_per_body"])
            fastest = min(ok, key=lambda t: t["force_ms"])
            cmp[k] = {"theta_interactions_at_equal_or_lower_error": fewest["interactions_per_body"],
                      "learned_interactions": r["interactions_per_body"],
                      "theta_force_ms_at_equal_or_lower_error": fastest["force_ms"],
                      "learned_force_ms": r["force_ms"]}
    return {"workload": f"{n:,} bodies (90/10), unseen seed 9301, theta = 0.5 fallback", "training": info,
            "rows": rows, "comparison": cmp}


def _against_theta(rows):
    """Each learned row against the theta-only rows: the fastest theta run
    at equal or lower median error, and the time ratio (above 1: the learned
    form is faster)."""
    out = {}
    thetas = {k: r for k, r in rows.items() if k.startswith(("theta_", "group_theta_"))}
    for k, r in rows.items():
        if not k.startswith("budget_"):
            continue
        ok = [(t["ms_per_step"], name) for name, t in thetas.items() if t["median_rel_err"] <= r["median_rel_err"]]
        if ok:
            ms, name = min(ok)
            out[k] = {"fastest_theta_at_equal_or_lower_error": name, "theta_ms_per_step": ms,
                      "learned_ms_per_step": r["ms_per_step"], "theta_ms_over_learned_ms": ms / r["ms_per_step"]}
        else:
            out[k] = {"fastest_theta_at_equal_or_lower_error": None, "learned_ms_per_step": r["ms_per_step"],
                      "note": "no theta run of the sweep reaches this error"}
    return out


def forms_4m(args, dev, params, scale, info):
    """The 4M-body combined-scale system (85 % inner belt, 10 % outer belt, 5 %
    trojans): plain FP64 theta=1.05 (fp64_list: the reference's interaction
    set in FP64) against the FP32 far field over a theta sweep and the FP32 +
    learned criterion at several per-body budgets, each with its median
    relative error against the FP64 direct sum on a 4,096-body sample
    (evaluated on the same initial state).  Returns the rows and the
    spec summary: the fastest learned run at an error no higher than
    the plain form's against the plain form, and against the fastest
    theta-only run at an error no higher than its own."""
    import torch
    bh = importlib.import_module("barnes-hut_gb300")
    n = args.ns_bodies
    pos, vel, mass, ids = bh.generate_system(SEED + 1, n, 0.10, 0.05)
    out = {"workload": f"{n:,} bodies (Sun, 8 planets, 85% inner belt, 10% outer belt, 5% trojans), dt=1h",
           "training": info}
    with bh.Context(n, dev) as ctx:
        ext = torch.cuda.ExternalStream(ctx.stream(), device=dev)
        flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{dev}")
        _fresh(ctx, pos, vel, mass, ids)
        err = _sample_error(ctx, n, G)
        peak32 = ctx.measure_fma_peak(False)
        rows = {}
        cases = [("plain_fp64", bh.MODE_FP64_LIST, None, THETA)]
        cases += [(f"theta_{th:g}", bh.MODE_FP32_FAR, None, th) for th in THETA_SWEEP]
        cases += [(f"group_theta_{th:g}", bh.MODE_FP32_GROUP, None, th) for th in THETA_SWEEP]
        cases += [(f"budget_{b:g}", bh.MODE_LEARNED, b, THETA) for b in LEARNED_BUDGETS]
        for name, mode, budget, theta in cases:
            if budget is not None:
                ctx.learned_set_model(params, scale, budget=budget, theta_max=args.theta_max)
            _fresh(ctx, pos, vel, mass, ids)
            a = ctx.compute_accelerations(theta, G, 0.0, mode)
            med, p99 = err(a)
            row = {"theta": theta, "median_rel_err": med, "p99_rel_err": p99}
            if budget is not None:
                st = ctx.learned_stats()
                row["budget"] = budget
                row["fallback_rate"] = st["fallback"] / max(1, st["candidates"])
                row["network_decided"] = st["accepted"] / max(1, st["candidates"])
                row["analytic_accepted"] = st["analytic"] / max(1, st["candidates"])
            ctx.set_bodies(pos, vel, mass, ids)
            ms, ipb = time_steps(ctx, ext, flush, mode, theta, args.ns_steps, 2)
            # phase split from a separate profiled pass (kernels one by one)
            ctx.set_profiling(True)
            for _ in range(2):
                flush.fill_(1.0)
                ctx.step(DT, theta, G, 1, mode, t=1.0)
            torch.cuda.synchronize()
            phases, _ = ctx.phase_times()
            ctx.set_profiling(False)
            ph = {k: v / 2 for k, v in phases.items()}
            row.update({"ms_per_step": ms, "body_steps_per_s": n / (ms * 1e-3), "interactions_per_body": ipb,
                        "phases_ms_per_step": ph})
            if mode in (bh.MODE_FP32_FAR, bh.MODE_FP32_GROUP) and theta == THETA:
                achieved = ipb * n * FLOPS_PER_INTERACTION / (ph["forces"] * 1e-3) / 1e12
                key = "fp32" if mode == bh.MODE_FP32_FAR else "fp32_group"
                row["roofline"] = {"kernel": KERNEL[mode], "bound": "fp32", "achieved": achieved, "peak": peak32,
                                   "unit": "TFLOP/s", "frac": achieved / peak32,
                                   "peak_source": "measured in-process: FP32 FMA chains (bh_measure_fma_peak)",
                                   "work": f"{FLOPS_PER_INTERACTION} flops x {ipb * n:.4g} interactions per launch",
                                   "traffic": TRAFFIC_BYTES.get((key, n)), "traffic_unit": "bytes per launch (ncu)"}
            rows[name] = row
        out["hbm_phases"] = hbm_phases(rows[f"theta_{THETA:g}"]["phases_ms_per_step"], n)
    out["forms"] = rows
    out["comparison"] = _against_theta(rows)
    base = rows["plain_fp64"]
    eligible = [k for k, r in rows.items() if k.startswith("budget_") and r["median_rel_err"] <= base["median_rel_err"]]
    best = max(eligible, key=lambda k: rows[k]["body_steps_per_s"]) if eligible else None
    ns = {"workload": out["workload"], "target": "FP32 + learned criterion >= 3x plain FP64 theta=1.05 at equal or "
                                                 "lower median error vs the FP64 direct sum (<= 1e-5)",
          "plain_fp64": {k: base[k] for k in ("ms_per_step", "body_steps_per_s", "median_rel_err")},
          "fp32_theta_1.05": {k: rows[f"theta_{THETA:g}"][k] for k in ("ms_per_step", "body_steps_per_s",
                                                                        "median_rel_err")},
          "fp32_group_theta_1.05": {k: rows[f"group_theta_{THETA:g}"][k]
                                    for k in ("ms_per_step", "body_steps_per_s", "median_rel_err")},
          "fp32_learned": None, "learned_vs_plain_fp64": None, "best_theta_fp32": None,
          "learned_vs_best_theta": None,
          "roofline_fp32_walk": rows[f"theta_{THETA:g}"].get("roofline"),
          "roofline_fp32_group_walk": rows[f"group_theta_{THETA:g}"].get("roofline")}
    # The fastest network-free FP32 run at an error no higher than the plain
    # FP64 form's, and its ratio to it.
    free = [k for k in rows if k.startswith(("theta_", "group_theta_"))
            and rows[k]["median_rel_err"] <= base["median_rel_err"]]
    if free:
        f = max(free, key=lambda k: rows[k]["body_steps_per_s"])
        ns["fastest_fp32_without_network"] = {"form": f, "ms_per_step": rows[f]["ms_per_step"],
                                              "median_rel_err": rows[f]["median_rel_err"],
                                              "vs_plain_fp64": rows[f]["body_steps_per_s"] / base["body_steps_per_s"]}
    if best:
        r = rows[best]
        ns["fp32_learned"] = {"budget": r["budget"], "ms_per_step": r["ms_per_step"],
                              "body_steps_per_s": r["body_steps_per_s"], "median_rel_err": r["median_rel_err"]}
        ns["learned_vs_plain_fp64"] = r["body_steps_per_s"] / base["body_steps_per_s"]
        cmp = out["comparison"][best]
        if cmp.get("fastest_theta_at_equal_or_lower_error"):
            t = rows[cmp["fastest_theta_at_equal_or_lower_error"]]
            ns["best_theta_fp32"] = {"theta": t["theta"], "ms_per_step": t["ms_per_step"],
                                     "median_rel_err": t["median_rel_err"]}
            ns["learned_vs_best_theta"] = t["ms_per_step"] / r["ms_per_step"]
    out["north_star"] = ns
    return out


# DRAM traffic per launch of the force kernel (dram__bytes_read.sum +
# dram__bytes_write.sum) from one ncu --set full capture of that kernel on
# that workload, keyed by (mode, bodies).
TRAFFIC_BYTES = {("fp64_list", 300_149): 52.34e6 + 1.16e6, ("fp32", 4_000_000): 482.41e6 + 183.02e6,
                 ("fp32_group", 4_000_000): 483.43e6 + 183.40e6}

# Algorithmic bytes per body of the HBM-bound phases: the minimum traffic of
# each phase's work (reads + writes of its inputs and outputs once).
PHASE_BYTES = {"kick_drift_bbox": 120, "keys": 32, "sort": 200, "permute": 128, "build": 136}


def bucket_domains(keys, bucket_bits, nranks):
    """update_rank_domains' split (src/load_balancing.cpp:12-65): the owner
    rank of each body and each rank's non-empty bucket prefixes."""
    bidx = (keys >> np.uint64(63 - bucket_bits)).astype(np.int64)
    hist = np.bincount(bidx, minlength=1 << bucket_bits)
    ideal = (len(keys) + nranks - 1) // nranks
    split, run = [], 0
    for i, h in enumerate(hist.tolist()):
        run += h
        if len(split) < nranks - 1 and run >= (len(split) + 1) * ideal:
            split.append(i)
    owner = np.searchsorted(np.array(split, np.int64), np.arange(1 << bucket_bits), side="right")
    doms = [(np.nonzero((hist > 0) & (owner == r))[0].astype(np.uint64)) << np.uint64(63 - bucket_bits)
            for r in range(nranks)]
    return owner[bidx], doms


def let_exchange(args, dev):
    """The LET data path at the 4M-body size split over 8 ranks (18-bit
    buckets, theta = 1.05): rank 0's device tree exports to the 7 other
    domains (createInteractionListForRank), and the records rank 0 receives
    from them are built into a map (buildTreeFromPseudoLeaves).  Host clock
    around the C-ABI calls (records copied back to the host included); the
    oracle does the same export and import on the host cores."""
    bh = importlib.import_module("barnes-hut_gb300")
    from oracle.oracle import Oracle
    n = args.ns_bodies
    pos, vel, mass, ids = bh.generate_system(SEED + 3, n, 0.10, 0.05)
    with bh.Context(n, dev) as full:
        full.set_bodies(pos, vel, mass, ids)
        bb = full.compute_bbox()
        keys = full.compute_keys()
    owner, doms = bucket_domains(keys, 18, 8)
    boxes = [bh.let_bucket_boxes(doms[r], 18, bb) for r in range(8)]
    theta2 = THETA * THETA

    def local(r):
        sel = np.nonzero(owner == r)[0]
        c = bh.Context(len(sel), dev)
        c.set_bodies(pos[sel], vel[sel], mass[sel], ids[sel])
        c.set_bbox(bb)
        c.compute_keys()
        c.sort_bodies()
        c.build_tree(merge=False)
        return c, sel

    ctx0, sel0 = local(0)
    ctx0.let_export(boxes[1], bb, theta2)
    t0 = time.perf_counter()
    sent = [ctx0.let_export(boxes[r], bb, theta2) for r in range(1, 8)]
    t_exp = time.perf_counter() - t0
    recv = []
    for r in range(1, 8):
        c, _ = local(r)
        recv.append(c.let_export(boxes[0], bb, theta2))
        c.close()
    p, d, m, com = (np.concatenate([x[k] for x in recv]) for k in range(4))
    ctx0.pseudo_leaf_tree(p, d, m, com)
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        cells = ctx0.pseudo_leaf_tree(p, d, m, com)
    t_imp = (time.perf_counter() - t0) / reps
    ctx0.let_accelerations(p, d, m, com, THETA, G)
    t0 = time.perf_counter()
    for _ in range(reps):
        acc_let = ctx0.let_accelerations(p, d, m, com, THETA, G)
    t_acc = (time.perf_counter() - t0) / reps
    ctx0.close()

    o, kind = Oracle("port"), "port"
    try:
        o, kind = Oracle("reference"), "reference"
    except (FileNotFoundError, OSError):
        pass
    sk, sp, sm, *_ = o.sort(keys[sel0], pos[sel0], mass[sel0], vel[sel0], ids[sel0])
    tree = o.tree(sk, sp, sm, merge=False)
    t0 = time.perf_counter()
    cpu_sent = o.let_export(tree, boxes[1], bb, theta2)
    c_exp = time.perf_counter() - t0
    tree.close()
    t0 = time.perf_counter()
    pt = o.pseudo_tree(p, d, m, com)
    c_imp = time.perf_counter() - t0
    same_cells = len(pt) == len(cells[0])
    pt.close()
    tree = o.tree(sk, sp, sm, merge=False)
    t0 = time.perf_counter()
    cpu_acc = o.let_accelerations(tree, (p, d, m, com), sk, sp, THETA, G, bb)
    c_acc = time.perf_counter() - t0
    tree.close()
    acc_equal = bool(np.array_equal(cpu_acc.view(np.uint64), acc_let.view(np.uint64)))
    return {"bodies": n, "ranks": 8, "bucket_bits": 18, "theta": THETA, "rank0_bodies": int(len(sel0)),
            "export": {"destinations": 7, "boxes": [int(len(b)) for b in boxes[1:]],
                       "records": [int(len(x[0])) for x in sent], "ms_per_export": 1e3 * t_exp / 7,
                       "cpu_ms_rank1": 1e3 * c_exp, "cpu_records_rank1": int(len(cpu_sent[0])),
                       "records_equal_rank1": int(len(sent[0][0])) == int(len(cpu_sent[0]))},
            "import": {"records": int(len(p)), "cells": int(len(cells[0])), "ms": 1e3 * t_imp,
                       "cpu_ms": 1e3 * c_imp, "cpu_cells_equal": bool(same_cells)},
            "let_forces": {"bodies": int(len(sel0)), "ms": 1e3 * t_acc, "cpu_ms": 1e3 * c_acc,
                           "bits_equal_oracle": acc_equal,
                           "form": "computeAccelerationsWithLET: pseudo-leaf map merged into the local map, "
                                   "exact FP64 walk per body"},
            "cpu_kind": kind, "timing": "host clock around the C-ABI call, results copied to the host"}


def csv_ingest(args, dev, n=1_000_000):
    """readCSV at 1M bodies: the state-vector CSV written once, then parsed
    on the GPU straight into a context (bh_load_csv) and by the host reader
    (std::getline + std::stod, one pass); the values are compared bit for
    bit.  Host clock; the file is in the page cache for both."""
    import tempfile
    bh = importlib.import_module("barnes-hut_gb300")
    pos, vel, mass, ids = bh.generate_system(SEED + 4, n, 0.10, 0.05)
    with tempfile.TemporaryDirectory() as d:
        f = Path(d) / "bodies.csv"
        bh.write_csv(f, ids, mass, pos, vel)
        size = f.stat().st_size
        with bh.Context(n, dev) as ctx:
            ctx.load_csv(f, 10)
            t0 = time.perf_counter()
            ctx.load_csv(f)
            t_gpu = time.perf_counter() - t0
            gp, gv, gm, gi, _ = ctx.get_bodies()
        lib = bh.library()
        import ctypes as C
        hi = np.empty(n, np.uint64); hm = np.empty(n); hp = np.empty((n, 3)); hv = np.empty((n, 3))
        k = C.c_int64(0)
        t0 = time.perf_counter()
        lib.bh_read_csv(str(f).encode(), -1, C.byref(k), hi.ctypes.data_as(C.c_void_p), hm.ctypes.data_as(C.c_void_p),
                        hp.ctypes.data_as(C.c_void_p), hv.ctypes.data_as(C.c_void_p))
        t_host = time.perf_counter() - t0
    same = all(np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))
               for a, b in ((gp, hp), (gv, hv), (gm, hm), (gi, hi)))
    return {"bodies": n, "file_mb": size / 1e6, "gpu_load_csv_s": t_gpu, "host_read_csv_s": t_host,
            "bits_equal": bool(same), "timing": "host clock, file in the page cache"}


def hbm_peak_gbs():
    try:
        return float(json.loads((Path(__file__).resolve().parent / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


def hbm_view(traffic, ms):
    """The force kernel against the HBM roofline: its measured DRAM traffic
    per launch over the launch's duration, as a fraction of the measured
    copy bandwidth (small: the kernel is not memory-bound)."""
    if not traffic or not ms:
        return None
    gbs = traffic / (ms * 1e-3) / 1e9
    peak = hbm_peak_gbs()
    return {"achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)"}


def hbm_phases(phases_ms, n):
    peak = hbm_peak_gbs()
    out = {}
    for k, b in PHASE_BYTES.items():
        if k in phases_ms and phases_ms[k] > 0:
            gbs = b * n / (phases_ms[k] * 1e-3) / 1e9
            out[k] = {"bytes_per_body": b, "ms": phases_ms[k], "achieved_gbs": gbs, "frac_of_measured_hbm": gbs / peak}
    return out


def run_ours(args, rank, ws, local):
    import torch
    bh = importlib.import_module("barnes-hut_gb300")
    dev = local
    torch.cuda.set_device(dev)
    pos, vel, mass, ids = bh.generate_system(SEED, args.bodies, args.outer, args.trojan)
    n = len(mass)
    mode = MODES[args.mode]
    theta = args.theta
    ctx = bh.Context(n, dev)
    ext = torch.cuda.ExternalStream(ctx.stream(), device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{dev}")
    if mode == bh.MODE_LEARNED:
        params, scale, _ = train_model(args)
        ctx.learned_set_model(params, scale, budget=args.budget, theta_max=args.theta_max)
    ctx.set_bodies(pos, vel, mass, ids)
    t = 0.0
    for _ in range(args.warmup):
        t = ctx.step(DT, theta, G, 1, mode, t=t)
    peak = ctx.measure_fma_peak(mode <= 1)

    times, inter = [], 0
    with ClockSampler(dev) as clk:
        # Untimed pre-roll of the same step, so that the sampler (which
        # starts slowly) records the clocks under this load around the
        # timed steps, which can be shorter than one sampling period.  It
        # runs for a time, not a step count, so the state is put back after
        # it: the timed steps and the accuracy sample then see the same
        # state however fast the pre-roll went.
        snap, t_snap = ctx.get_bodies(), t
        t_pre = time.perf_counter() + 1.0
        while time.perf_counter() < t_pre:
            flush.fill_(1.0)
            t = ctx.step(DT, theta, G, 1, mode, t=t)
            torch.cuda.synchronize(dev)
        ctx.set_bodies(*snap[:4])
        ctx.set_accelerations(snap[4])
        t = t_snap
        barrier(ws)
        l0 = ctx.launches()
        # No collector pause inside the event-timed steps: a host stall
        # between the first event and the step's launch would be counted as
        # device time.
        gc.collect()
        gc.disable()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize(dev)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            t = ctx.step(DT, theta, G, 1, mode, t=t)
            e1.record(ext)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            inter += ctx.interaction_count()
        torch.cuda.synchronize(dev)
        barrier(ws)
        w1 = time.perf_counter()
        gc.enable()
        time.sleep(0.25)  # the sample that covers the last timed step
    torch.cuda.synchronize(dev)
    launches = ctx.launches() - l0
    total_ms = sum(times)
    total_ms = reduce_max(total_ms, ws)
    # Per-phase device times: the same number of steps again with CUDA events
    # around each phase (kernels launched one by one), outside the timed run.
    ctx.set_profiling(True)
    for _ in range(args.steps):
        flush.fill_(1.0)
        t = ctx.step(DT, theta, G, 1, mode, t=t)
    torch.cuda.synchronize(dev)
    phases, _ = ctx.phase_times()
    ctx.set_profiling(False)

    # End to end through the C ABI with host-resident state (pinned memory).
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()  # noqa: E731
    hp, hv, hm = pin((n, 3), torch.float64), pin((n, 3), torch.float64), pin((n,), torch.float64)
    hi = pin((n,), torch.int64).view(np.uint64)
    ha = pin((n, 3), torch.float64)
    hp[:], hv[:], hm[:], hi[:], ha[:] = ctx.get_bodies()
    e2e_steps = max(1, args.e2e_steps)
    barrier(ws)
    gc.collect()
    gc.disable()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        # one C-ABI call per step: the state's upload, the step and the
        # download of the new state and accelerations (bh_step_host)
        t = ctx.step_host(hp, hv, hm, hi, ha, DT, theta, G, 1, mode, t=t)
    e2e_s = reduce_max(time.perf_counter() - t0, ws)
    gc.enable()
    h2d = hp.nbytes + hv.nbytes + hm.nbytes + hi.nbytes + ha.nbytes
    d2h = h2d

    # Accuracy of this mode against the FP64 direct-sum sampler (4,096 bodies).
    rng = np.random.default_rng(0)
    sample = np.sort(rng.choice(n, min(n, 4096), replace=False))
    ref = ctx.direct_sum(sample, G)
    acc = ctx.compute_accelerations(theta, G, 0.0, mode)
    err = np.linalg.norm(acc[sample] - ref, axis=1) / np.linalg.norm(ref, axis=1)
    accuracy = {"median_rel_err": float(np.median(err)), "p99_rel_err": float(np.quantile(err, 0.99)),
                "sample": int(len(sample)), "against": "FP64 direct sum"}

    ns = pr = le = lh = runs = let = ingest = None
    blocks = set(EXTRA_BLOCKS) if args.blocks is None else set(args.blocks.split(","))
    if rank == 0 and ws == 1 and not args.no_extras:
        needs_model = blocks & {"forms_4m", "learned_eval", "long_runs"}
        params, scale, info = train_model(args) if needs_model else (None, None, None)
        ns = forms_4m(args, dev, params, scale, info) if "forms_4m" in blocks else None
        le = learned_eval(args, dev, params, scale) if "learned_eval" in blocks else None
        lh = learned_high_accuracy(args, dev) if "learned_high_accuracy" in blocks else None
        pr = precision_run(args, dev) if "precision_run" in blocks else None
        let = let_exchange(args, dev) if "let_exchange" in blocks else None
        ingest = csv_ingest(args, dev) if "csv_ingest" in blocks else None
        if "long_runs" in blocks:
            runs = {"config1_19k_plain_240_steps": config1_run(dev),
                    "config2_300k_fp64_list_2000_steps": long_run(dev, N_BODIES, 0.10, 0.0, SEED, "fp64_list",
                                                                  2000),
                    "config5_4m_fp32_learned_500_steps": long_run(dev, args.ns_bodies, 0.10, 0.05, SEED + 1,
                                                                  "learned", 500, params, scale, args.budget,
                                                                  args.theta_max)}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(pos, vel, mass, ids, args.cpu_seconds, theta)
    ctx.close()
    if rank != 0:
        return
    k = args.steps
    force_ms = phases["forces"] / k
    inter_per_step = inter / k
    achieved = inter_per_step * FLOPS_PER_INTERACTION / (force_ms * 1e-3) / 1e12
    fp = "fp64" if mode <= 1 else "fp32"
    value = replica_value(ws, n, k, total_ms)
    line = {
        "metric": "body-steps/s", "value": value, "unit": "body-steps/s", "n_gpus": ws, "steps": k,
        "warmup": args.warmup, "ms_per_step": total_ms / k, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if mode <= 1 else "f32 far field + f64 state/direct terms",
        "data": DATA,
        "config": bench_config(args, n, ws),
        "roofline": {"kernel": KERNEL[mode], "bound": fp, "achieved": achieved,
                     "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                     "peak_source": f"measured in-process: {fp.upper()} FMA chains (bh_measure_fma_peak)",
                     "work": f"{FLOPS_PER_INTERACTION} flops x {inter_per_step:.4g} interactions per launch",
                     "traffic": TRAFFIC_BYTES.get((args.mode, n)),
                     "traffic_unit": "bytes per launch (ncu)",
                     "hbm_view": hbm_view(TRAFFIC_BYTES.get((args.mode, n)), force_ms)},
        "phases_ms_per_step": {kk: v / k for kk, v in phases.items()},
        "hbm_phases": hbm_phases({kk: v / k for kk, v in phases.items()}, n),
        "interactions_per_body": inter_per_step / n,
        "interactions_per_s": inter_per_step / (force_ms * 1e-3),
        "accuracy": accuracy,
        "e2e": {"value": ws * n * e2e_steps / e2e_s, "unit": "body-steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clk.summary((w0, w1)),
        "cpu_baseline": cpu,
        "north_star": ns.get("north_star") if ns else None,
        "forms_4m": ns,
        "learned_eval": le,
        "learned_high_accuracy": lh,
        "precision_run": pr,
        "long_runs": runs,
        "let_exchange": let,
        "csv_ingest": ingest,
    }
    print(json.dumps(line), flush=True)


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce_max(x: float, ws: int) -> float:
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ws: int, n: int, k: int, slowest_ms: float) -> float:
    """Whole-job body-steps/s of ws replicas that each ran k steps of n
    bodies, over the slowest rank's time (weak scaling)."""
    return ws * n * k / (slowest_ms * 1e-3)


def main():
    args = parse()
    rank, ws, local = (0, 1, 0)
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        run_reference(args, rank)
        return
    rank, ws, local = dist_init()
    run_ours(args, rank, ws, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
