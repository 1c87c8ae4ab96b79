"""Benchmark of the gravity/SPH substep: body-substeps/s, FP32-mixed vs FP64.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl cuda|reference]

Workload (default): the 100,000-body quasar merger — two exponential disks,
mass ratio 1:1.2, 50 deg tilt, 10% SPH gas, theta 0.5, softening 0.01,
dt 1e-3 — seeded synthetic initial conditions of that shape (no dataset).
A step is one kick-drift-kick substep: tree build, gravity walk, SPH density
and forces, kicks, cooling. The headline `value` is the FP32-mixed walk; the
FP64 plain walk is measured on the same workload beside it, over the same K
substeps.

Timing: W untimed warm-up substeps, then K substeps each bracketed by CUDA
events on the library's stream (torch's current stream), with a 512 MB write
between substeps to flush L2 (the 100k working set fits in L2). `e2e` is the
same metric through the reference-facing C call integrator_step() with the
Body array and pool in pinned host memory, host<->device copies included
(K calls). Under torchrun (N > 1) every rank runs an independent replica (the
path does not shard: replicas only); value = all ranks' body-substeps / max
time.

At N = 1 the line also carries `targets_1m`: the 1,000,000-body bulge + disk
at theta 0.3 and 0.5 (softening 0.005), FP32-mixed and FP64 plain over K
substeps each, their force errors against an FP64 direct sum on a seeded
4096-body sample, and the reference's CPU algorithm on the host cores at the
same theta (bounded sample) — the FP32/FP64 and FP64/CPU ratios the targets
are stated on.

--impl reference times the reference's CPU algorithm (the oracle port in
oracle/, OpenMP on all host cores) on the same workload; it draws its bodies
with the oracle's generator and never loads the product library.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "body-substeps/s (FP32-mixed walk; FP64 plain beside it)"
UNIT = "body-substeps/s"

CONFIGS = {
    "merger100k": dict(kind=1, n=100_000, theta=0.5, eps=0.01, dt=1e-3, sph=True,
                       desc="quasar merger: 2 exp. disks 1:1.2, 50deg tilt, 10% SPH gas"),
    "disk20k": dict(kind=0, n=20_000, theta=0.5, eps=0.01, dt=1e-3, sph=False,
                    desc="single exponential-disk galaxy (reference default run)"),
    "bulge1m": dict(kind=2, n=1_000_000, theta=0.5, eps=0.005, dt=1e-3, sph=False,
                    desc="Plummer bulge 300k + exponential disk 700k"),
}
# batched ensemble: 64 exponential-disk galaxies, N log-uniform in [2000, 50000]
# (size seed 12: 1,102,884 bodies), each with its own seed, scale length in
# [0.5, 2] and SMBH fraction in [0.001, 0.02]; FP32-mixed walk, FP64 drift
ENSEMBLE = dict(n_gal=64, n_min=2000, n_max=50000, size_seed=12, theta=0.5, eps=0.01, dt=1e-3,
                desc="64 independent exp.-disk galaxies, N log-uniform [2000, 50000], one handle")
FLOP_PER_INTERACTION = 20  # monopole body-cell interaction: 3 sub, 3 fma d2, rsqrt, 3 mul, 3 fma acc
# DRAM bytes per body of one k_walk32 launch, from the ncu capture of the
# 100k merger (profiles/k_walk32_merger100k_fp32.md: 10.07 MB read, 0 written
# for 100,000 bodies): the first touch of the tree and the bodies; the tree
# stays in L2 during the walk. Other workloads scale it by the body count.
WALK32_DRAM_BYTES_PER_BODY = 10.07e6 / 100_000
# issue slots busy in the same capture (k_walk32, 100k merger): 55.2%
WALK32_ISSUE_BUSY = 0.552
WALK32_NOTE = ("20 flop per reference interaction / the walk's time inside the substep (CUDA "
               "events around it, SPH running beside it); peak = FP32 FMA throughput "
               "measured live by csg_measure_fp_peaks (the walk is CUDA-core bound: no dense "
               "contraction, tree resident in L2). What bounds it is instruction issue in the "
               "traversal. traffic and issue_slots_busy_ncu are per-launch DRAM bytes and issue "
               "activity from the committed ncu capture of k_walk32 on the 100k merger "
               "(profiles/), traffic scaled by the body count")
# The FP32 walk of a system with few 32-body tasks for the GPU (at most 12 per
# SM) runs eight warps per task, one per child subtree of the root
# (k_walk32_units, then k_walk_sum adds the eight partials): the same bits.
WALK32_SPLIT_TASKS_PER_SM = 12
# the same two figures for k_walk32_units from its capture on the 20k disk
# (profiles/walk_units_disk20k.md: 2.05 MB read, 0 written; issue 48.6% busy)
WALK32U_DRAM_BYTES_PER_BODY = 2.04672e6 / 20_000
WALK32U_ISSUE_BUSY = 0.486


def walk32_kernel(torch, n_bodies, n_systems=1):
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    if n_bodies // 32 + n_systems + 1 <= WALK32_SPLIT_TASKS_PER_SM * sms:
        return "k_walk32_units + k_walk_sum (gravity walk, a warp per root child)", True
    return "k_walk32 (gravity walk)", False


SEED = 0x5EED0000


def max_over_ranks(torch, values, device):
    """Each value's maximum over the ranks: a job's time is its slowest rank's."""
    t = torch.tensor(values, dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return t.tolist()


def job_rate(units_per_rank, world, secs_max):
    """Whole-job throughput: every rank's units over the slowest rank's time
    (replicas: each rank runs its own independent system)."""
    return units_per_rank * world / secs_max


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class ClockSampler:
    """nvidia-smi samples (every 200 ms) of SM clock and throttle reasons over
    the whole run of the GPU legs. Timed regions are marked with window();
    the reported median is over the samples that fall inside them (all
    samples of the run when fewer than 3 do), the reasons over every sample."""

    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.windows = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def window(self, t0, t1):
        self.windows.append((t0, t1))

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows, reasons = [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((t, float(parts[1]), float(parts[2])))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        # a sample read at t covers roughly [t - 0.2 s, t]
        inside = [r for r in rows if any(a - 0.05 <= r[0] <= b + 0.25 for a, b in self.windows)]
        use = inside if len(inside) >= 3 else rows
        return {"sm_mhz": float(np.median([r[1] for r in use])) if use else None,
                "sm_max_mhz": max(r[2] for r in rows) if rows else None,
                "samples": len(rows), "samples_in_timed_regions": len(inside),
                "median_over": "timed regions" if use is inside else "whole GPU run",
                "reasons": sorted(reasons)}


def flush_buffer(torch):
    return torch.empty(512 << 20, dtype=torch.uint8, device="cuda")


def time_substeps(torch, sim, k, flush, sampler=None):
    """Sum of per-substep device times (events on the launching stream)."""
    st = torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(k)]
    torch.cuda.synchronize()
    t0 = time.time()
    for a, b in evs:
        flush.zero_()
        a.record(st)
        sim.substeps_async(1)
        b.record(st)
    torch.cuda.synchronize()
    if sampler:
        sampler.window(t0, time.time())
    return sum(a.elapsed_time(b) for a, b in evs) / 1e3


def time_phase(torch, fn, k, flush):
    st = torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(k)]
    for a, b in evs:
        flush.zero_()
        a.record(st)
        fn()
        b.record(st)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in evs) / k / 1e3


def rel_err_stats(a, b):
    err = np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)
    return {"median": float(np.median(err)), "p99": float(np.quantile(err, 0.99)),
            "max": float(err.max()),
            "global": float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))}


def acc(b):
    return np.stack([b["ax"], b["ay"], b["az"]], axis=1)


def run_cuda(args, torch, lib, cfg, rank, world, sampler):
    """The headline workload: FP32-mixed and FP64 substeps timed on the
    device (K substeps each), their phases and walk counters, the force
    errors, and K end-to-end integrator_step calls on pinned host buffers."""
    stream = torch.cuda.current_stream()
    assert stream.cuda_stream != 0, "the library needs a non-default stream handle"
    flush = flush_buffer(torch)
    bodies = lib.generate_ics(cfg["kind"], cfg["n"], SEED + rank)
    n_alive = int((bodies["mass"] > 0).sum())
    common = dict(softening=cfg["eps"], theta=cfg["theta"], dt=cfg["dt"], sph=cfg["sph"])
    out = {}
    for prec, name in ((lib.PREC_FP32_MIXED, "fp32_mixed"), (lib.PREC_FP64, "fp64")):
        sim = lib.Sim.from_bodies(bodies, precision=prec, **common)
        sim.set_stream(stream.cuda_stream)
        for _ in range(args.warmup):
            flush.zero_()
            sim.substeps_async(1)
        torch.cuda.synchronize()
        k = args.steps
        l0 = sim.launch_count()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        secs = time_substeps(torch, sim, k, flush, sampler)
        sim.sync()  # raises if any substep reported an error
        launches = sim.launch_count() - l0
        # phases inside the real substep: the same kernels, direct launches
        # with CUDA events between the phases (cosmosim_phase_times)
        sim.enable_phase_timing(True)
        for _ in range(k):
            flush.zero_()
            sim.substeps_async(1)
        sim.sync()
        ph = sim.phase_times()
        sim.enable_phase_timing(False)
        phases = {key[:-3]: ph[key] / ph["substeps"] for key in ph if key.endswith("_ms")}
        walk_s = phases["gravity"] / 1e3
        build_s = phases["build"] / 1e3
        # the walk launched alone on the state reached (no SPH beside it)
        walk_alone_s = time_phase(torch, sim.gravity_async, 5, flush)
        sim.sync()
        sim.enable_stats(True)
        sim.gravity_async()
        inter, wsteps, wactive = sim.walk_stats()
        sim.enable_stats(False)
        out[name] = dict(secs=secs, steps=k, launches=launches, build_s=build_s, walk_s=walk_s,
                         walk_alone_s=walk_alone_s, phases=phases,
                         interactions=inter, warp_steps=wsteps, active_lane_steps=wactive,
                         state=sim.bodies() if name == "fp32_mixed" else None)
        sim.close()
    # precision and algorithmic error on the FP32 run's final state
    st = out["fp32_mixed"]["state"]
    g64 = lib.Sim.from_bodies(st, precision=lib.PREC_FP64, **common)
    g32 = lib.Sim.from_bodies(st, precision=lib.PREC_FP32_MIXED, **common)
    a64, a32 = acc(g64.bodies()), acc(g32.bodies())
    alive = st["mass"] > 0
    rng = np.random.default_rng(1)
    sample = rng.choice(np.nonzero(alive)[0], size=min(4096, int(alive.sum())), replace=False)
    direct = g64.direct_forces(sample)
    errors = {"fp32_vs_fp64_walk": rel_err_stats(a32[alive], a64[alive]),
              "fp64_walk_vs_direct": rel_err_stats(a64[sample], direct),
              "fp32_walk_vs_direct": rel_err_stats(a32[sample], direct),
              "direct_sample": int(len(sample))}
    g64.close()
    g32.close()
    # end to end through integrator_step with pinned host buffers
    pinned = torch.empty(cfg["n"] * 168, dtype=torch.uint8, pin_memory=True)
    hb = pinned.numpy().view(bodies.dtype)
    hb[:] = bodies
    from cosmosim_gb300.abi import NODE_DTYPE

    pool_t = torch.empty(8 * cfg["n"] * 104, dtype=torch.uint8, pin_memory=True)
    pool = pool_t.numpy().view(NODE_DTYPE)
    lib.set_precision(lib.PREC_FP32_MIXED)
    lib.integrator_init_accelerations(hb, 1.0, cfg["eps"], cfg["theta"], pool)
    for _ in range(args.warmup):
        lib.integrator_step(hb, cfg["dt"], 1.0, cfg["eps"], cfg["theta"], pool, int(cfg["sph"]))
    ke = args.steps
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0w, t0 = time.time(), time.perf_counter()
    for _ in range(ke):
        lib.integrator_step(hb, cfg["dt"], 1.0, cfg["eps"], cfg["theta"], pool, int(cfg["sph"]))
    e2e_s = time.perf_counter() - t0
    sampler.window(t0w, time.time())
    lib.set_precision(lib.PREC_FP64)
    _, nodes = lib.octree_build(hb, pool)
    return dict(n_alive=n_alive, runs=out, errors=errors, e2e_s=e2e_s, e2e_steps=ke,
                e2e_nodes=nodes)


def ensemble_sizes():
    r = np.random.default_rng(ENSEMBLE["size_seed"])
    lo, hi = np.log(ENSEMBLE["n_min"]), np.log(ENSEMBLE["n_max"])
    return np.exp(r.uniform(lo, hi, ENSEMBLE["n_gal"])).astype(np.int64)


def ensemble_bodies(gen, rank):
    """The 64 galaxies, drawn by gen (the library's or the oracle's
    generate_ics: byte-identical)."""
    from cosmosim_gb300.abi import BODY_DTYPE

    sizes = ensemble_sizes()
    parts = [gen(3, int(n), SEED + 1000 * rank + g) for g, n in enumerate(sizes)]
    return np.concatenate(parts).astype(BODY_DTYPE), parts


def time_calls(torch, fn, k, flush):
    """Total device time of k calls of fn, each bracketed by events (L2 flushed before)."""
    st = torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(k)]
    for a, b in evs:
        flush.zero_()
        a.record(st)
        fn()
        b.record(st)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in evs) / 1e3


def run_ensemble(args, torch, lib, rank, world):
    """64 galaxies in one handle (one walk launch per substep, one graph) vs the
    same galaxies as 64 handles stepped one after another."""
    e = ENSEMBLE
    dev = torch.cuda.current_device()
    stream = torch.cuda.current_stream()
    flush = flush_buffer(torch)
    t0 = time.perf_counter()
    allb, parts = ensemble_bodies(lib.generate_ics, rank)
    t_host_ics = time.perf_counter() - t0
    sizes = [len(p) for p in parts]
    n_total = len(allb)
    # the same 64 systems generated on the GPU straight into a handle
    t0 = time.perf_counter()
    dev_ens = lib.Sim.ensemble_ics(3, sizes, SEED + 1000 * rank, softening=e["eps"],
                                   theta=e["theta"], dt=e["dt"], precision=lib.PREC_FP32_MIXED)
    t_dev_ics = time.perf_counter() - t0
    dev_ens.close()
    common = dict(softening=e["eps"], theta=e["theta"], dt=e["dt"])
    res = {}
    # the batched handle, FP32-mixed: autotune the walk shape, then time substeps
    ens = lib.Sim.ensemble(allb, sizes, precision=lib.PREC_FP32_MIXED, **common)
    ens.set_stream(stream.cuda_stream)
    best, cands = ens.autotune_walk(reps=3)
    for _ in range(args.warmup):
        flush.zero_()
        ens.substeps_async(1)
    torch.cuda.synchronize()
    sampler = ClockSampler(dev)
    sampler.start()
    if world > 1:
        torch.distributed.barrier()
    l0 = ens.launch_count()
    secs = time_substeps(torch, ens, args.steps, flush, sampler)
    ens.sync()
    launches = ens.launch_count() - l0
    build_s = time_phase(torch, ens.build_tree_async, 5, flush)
    walk_s = time_phase(torch, ens.gravity_async, 5, flush)
    ens.enable_stats(True)
    ens.gravity_async()
    inter = ens.interactions()
    ens.enable_stats(False)
    state = ens.bodies()
    # end to end through the handle API: pinned host Body[] in, result out
    pin_in = torch.empty(n_total * 168, dtype=torch.uint8, pin_memory=True)
    pin_out = torch.empty(n_total * 168, dtype=torch.uint8, pin_memory=True)
    hin = pin_in.numpy().view(allb.dtype)
    hout = pin_out.numpy().view(allb.dtype)
    hin[:] = state
    ke = args.steps
    torch.cuda.synchronize()
    t0w, t0 = time.time(), time.perf_counter()
    for _ in range(ke):
        ens.set_bodies(hin)
        ens.substeps_async(1)
        lib.load().cosmosim_copy_bodies(ens.h, hout.ctypes.data, n_total)
    e2e_s = time.perf_counter() - t0
    sampler.window(t0w, time.time())
    ens.sync()
    ens.close()
    res["fp32"] = dict(secs=secs, steps=args.steps, launches=launches, build_s=build_s,
                       walk_s=walk_s, interactions=inter)
    # the batched handle, FP64 plain (default walk shape)
    k64 = args.steps
    ens64 = lib.Sim.ensemble(allb, sizes, precision=lib.PREC_FP64, **common)
    ens64.set_stream(stream.cuda_stream)
    for _ in range(args.warmup):
        ens64.substeps_async(1)
    res["fp64"] = dict(secs=time_substeps(torch, ens64, k64, flush, sampler), steps=k64)
    ens64.sync()
    ens64.close()
    # the same galaxies as 64 separate handles, stepped one after another
    kseq = args.steps
    for prec, name in ((lib.PREC_FP64, "seq_fp64"), (lib.PREC_FP32_MIXED, "seq_fp32")):
        sims = [lib.Sim.from_bodies(p, precision=prec, **common) for p in parts]
        for sm in sims:
            sm.set_stream(stream.cuda_stream)
            for _ in range(args.warmup):
                sm.substeps_async(1)

        def one_substep_all():
            for sm in sims:
                sm.substeps_async(1)

        torch.cuda.synchronize()
        res[name] = dict(secs=time_calls(torch, one_substep_all, kseq, flush), steps=kseq)
        for sm in sims:
            sm.sync()
            sm.close()
    clocks = sampler.stop()
    # per-galaxy error of the FP32-mixed walk vs the FP64 walk, and of both
    # against an FP64 direct sum on 64 bodies per galaxy (4096 in all)
    g64 = lib.Sim.ensemble(state, sizes, precision=lib.PREC_FP64, **common)
    g32 = lib.Sim.ensemble(state, sizes, precision=lib.PREC_FP32_MIXED, **common)
    a64, a32 = acc(g64.bodies()), acc(g32.bodies())
    rng = np.random.default_rng(1)
    offs = np.concatenate([[0], np.cumsum(sizes)])
    sample = np.concatenate([offs[g] + rng.choice(sizes[g], size=64, replace=False)
                             for g in range(len(sizes))])
    direct = g64.direct_forces(sample)
    g64.close()
    g32.close()
    per_gal = []
    for g in range(len(sizes)):
        sl = slice(offs[g], offs[g + 1])
        st = rel_err_stats(a32[sl], a64[sl])
        per_gal.append({"n": int(sizes[g]), "median": st["median"], "max": st["max"]})
    errors = {
        "fp32_vs_fp64_walk_per_galaxy": {
            "worst_median": max(p["median"] for p in per_gal),
            "worst_max": max(p["max"] for p in per_gal),
            "galaxies": [[p["n"], float(f"{p['median']:.3g}"), float(f"{p['max']:.3g}")]
                         for p in per_gal]},
        "fp32_walk_vs_direct": rel_err_stats(a32[sample], direct),
        "fp64_walk_vs_direct": rel_err_stats(a64[sample], direct),
        "direct_sample": int(len(sample))}
    return dict(n_total=n_total, sizes=sizes, runs=res, best=best, candidates=cands,
                errors=errors, clocks=clocks, e2e_s=e2e_s, e2e_steps=ke,
                ic_s={"host_generator_64_galaxies": t_host_ics,
                      "device_generated_handle_incl_first_forces": t_dev_ics})


def ensemble_line(args, torch, lib, rank, world, fp32_peak):
    r = run_ensemble(args, torch, lib, rank, world)
    runs = r["runs"]
    times = [runs["fp32"]["secs"], r["e2e_s"]]
    if world > 1:
        times = max_over_ranks(torch, times, "cuda")
    n = r["n_total"]

    def rate(run):
        return n * run["steps"] / run["secs"]

    value = job_rate(n * runs["fp32"]["steps"], world, times[0])
    f32 = runs["fp32"]
    achieved = FLOP_PER_INTERACTION * f32["interactions"] / f32["walk_s"] / 1e12
    e = ENSEMBLE
    return {
        "metric": "body-substeps/s (batched ensemble, FP32-mixed walk)", "value": value,
        "unit": UNIT, "n_gpus": world, "steps": f32["steps"], "warmup": args.warmup,
        "ms_per_step": 1e3 * f32["secs"] / f32["steps"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "precision": "FP32 pair forces (compensated sums); FP64 positions, tree moments, drift", "data": "synthetic",
        "config": {"workload": f"ensemble64: {e['desc']}", "n_bodies": n, "n_systems": e["n_gal"],
                   "sizes_min_max": [int(min(r["sizes"])), int(max(r["sizes"]))],
                   "theta": e["theta"], "softening": e["eps"], "dt": e["dt"], "sph": False,
                   "l2": "512 MB flush between timed substeps",
                   "parallelism": f"replicas x{world}"},
        "walk_shape": {"autotuned": r["best"], "candidates": r["candidates"]},
        "initial_conditions_s": r["ic_s"],
        "baselines": {
            "ensemble_fp64_plain": rate(runs["fp64"]),
            "sequential_64_handles_fp64_plain": rate(runs["seq_fp64"]),
            "sequential_64_handles_fp32_mixed": rate(runs["seq_fp32"]),
            "speedup_vs_sequential_fp64_plain": value / world / rate(runs["seq_fp64"]),
            "speedup_vs_sequential_fp32_mixed": value / world / rate(runs["seq_fp32"])},
        "phases_ms": {"build": 1e3 * f32["build_s"], "walk_fp32": 1e3 * f32["walk_s"]},
        "interactions_per_substep": f32["interactions"],
        "roofline": {"bound": "fp32-pipe", "kernel": "k_walk32 (gravity walk, all systems)",
                     "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": WALK32_DRAM_BYTES_PER_BODY * n},
        "errors": r["errors"],
        "e2e": {"value": job_rate(n * r["e2e_steps"], world, times[1]), "unit": UNIT,
                "api": "cosmosim_set_bodies + cosmosim_substeps_async(1) + cosmosim_copy_bodies "
                       "(pinned host Body[])",
                "steps": r["e2e_steps"], "h2d_bytes_per_step": 168 * n,
                "d2h_bytes_per_step": 168 * n},
        "gpu_launches": f32["launches"],
        "clocks": r["clocks"],
    }


def ensemble_reference(args, world):
    """The reference's CPU algorithm over the 64 galaxies (one system at a time,
    as the reference runs them), substep sweeps within --cpu-budget seconds."""
    from cosmosim_gb300.abi import NODE_DTYPE
    from oracle import orc

    orc.build()
    o = orc.Oracle()
    cores = o.set_threads(os.cpu_count() or 1)
    e = ENSEMBLE
    _, parts = ensemble_bodies(o.generate_ics, 0)
    pools = [np.zeros(8 * len(p), dtype=NODE_DTYPE) for p in parts]
    for p, pool in zip(parts, pools):
        o.integrator_init_accelerations(p, 1.0, e["eps"], e["theta"], pool)
    def sweep():
        for p, pool in zip(parts, pools):
            o.integrator_step(p, e["dt"], 1.0, e["eps"], e["theta"], pool, 0)

    # untimed warm-up sweeps (within 30 s), then the timed ones
    warm = 0
    t0 = time.perf_counter()
    while warm < args.warmup and (warm < 1 or time.perf_counter() - t0 < 30.0):
        sweep()
        warm += 1
    sweeps = 0
    t0 = time.perf_counter()
    while sweeps < max(1, args.steps) and (sweeps < 1 or time.perf_counter() - t0 < args.cpu_budget):
        sweep()
        sweeps += 1
    secs = time.perf_counter() - t0
    n = sum(len(p) for p in parts)
    v = n * sweeps / secs
    return {"metric": "body-substeps/s (batched ensemble, FP32-mixed walk)", "value": v,
            "unit": UNIT, "impl": "reference", "n_gpus": world, "steps": sweeps, "warmup": warm,
            "ms_per_step": 1e3 * secs / sweeps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"ensemble64: {e['desc']}", "n_bodies": n},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{sweeps} substep sweeps over the 64 galaxies after "
                                       f"{warm} untimed (oracle/orc.c, OpenMP, {cores} threads)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# differentiable merger: two disks as the 100k merger, 10,000 stars, no SPH,
# 200 substeps at dt 2e-3, checkpoints every 20, loss = mean squared distance
# of the final positions to a seeded target snapshot
ADJOINT = dict(n=10_000, substeps=200, dt=2e-3, checkpoint_every=20, eps=0.01, theta=0.5,
               desc="two-disk merger, 10k stars, 200 KDK substeps dt 2e-3, checkpoints every 20")


def adjoint_line(args):
    """Gradient of the loss w.r.t. all initial positions/velocities and three
    orbital parameters: the C-ABI adjoint (Barnes-Hut, frozen interaction
    lists) timed, checked against central differences (h = 1e-6, 32 random
    directions) and against the FP64 direct-sum adjoint."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from adjoint_harness import MergerProblem, floored_errors, rel_errors
    from cosmosim_gb300 import lib

    e = ADJOINT
    kw = dict(n=e["n"], substeps=e["substeps"], dt=e["dt"],
              checkpoint_every=e["checkpoint_every"], softening=e["eps"], theta=e["theta"])
    pr = MergerProblem(**kw)
    b0 = pr.ic.bodies(*[t.numpy() for t in pr.ic.state(__import__("torch").tensor(pr.p0))])
    # timing: checkpointed forward + backward (the production path)
    for _ in range(max(1, args.warmup // 3)):
        pr.adj.forward(b0, pr.target)
        pr.adj.backward()
    reps = 3
    t0 = time.perf_counter()
    l0 = pr.adj.stats()["launches"]
    for _ in range(reps):
        pr.adj.forward(b0, pr.target)
    t_fwd = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        pr.adj.backward()
    t_bwd = (time.perf_counter() - t0) / reps
    launches = (pr.adj.stats()["launches"] - l0) // reps
    mem_ckpt = pr.adj.stats()["device_bytes"]
    # gradients through the autograd Function (recorded lists for the checks)
    loss, gp, gx, gv = pr.gradients(record=True)
    st = pr.adj.stats()
    gnorm = float(np.sqrt((gx ** 2).sum() + (gv ** 2).sum()))
    fd6 = pr.fd_directions(gx, gv, k=32, h=1e-6)
    fd5 = pr.fd_directions(gx, gv, k=32, h=1e-5)
    fdp = pr.fd_params(gp, h=1e-6)
    r6, r5, rp = rel_errors(fd6), rel_errors(fd5), rel_errors(fdp)
    f6 = floored_errors(fd6, gnorm)
    pr.close()
    # FP64 direct-sum adjoint of the same run
    dr = MergerProblem(mode=lib.ADJ_DIRECT, **kw)
    t0 = time.perf_counter()
    _, dgp, dgx, dgv = dr.gradients(record=False)
    t_direct = time.perf_counter() - t0
    dfd = dr.fd_directions(dgx, dgv, k=4, h=1e-6, frozen=False)
    dr.close()
    a = np.concatenate([gx.ravel(), gv.ravel()])
    bb = np.concatenate([dgx.ravel(), dgv.ravel()])
    n, T = e["n"], e["substeps"]
    value = n * T / (t_fwd + t_bwd)
    return {
        "metric": "adjoint body-substeps/s (forward + backward, Barnes-Hut, FP64)",
        "value": value, "unit": UNIT, "n_gpus": 1, "steps": T, "warmup": args.warmup,
        "ms_per_step": 1e3 * (t_fwd + t_bwd) / T, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"adjoint10k: {e['desc']}", "n_bodies": n, "theta": e["theta"],
                   "softening": e["eps"], "dt": e["dt"], "substeps": T,
                   "checkpoint_every": e["checkpoint_every"], "sph": False,
                   "timing": "host wall clock of the blocking C-ABI calls"},
        "times_s": {"forward": t_fwd, "backward_with_recompute": t_bwd,
                    "direct_sum_forward_backward": t_direct},
        "memory_bytes": {"checkpointed": mem_ckpt, "all_lists_recorded": st["device_bytes"]},
        "interactions_per_run": st["interactions"],
        "loss": loss,
        "grad_orbital": {"pericentre": float(gp[0]), "inclination_deg": float(gp[1]),
                         "approach_speed": float(gp[2])},
        "checks": {
            "fd_h1e-6_32dirs": {"median_rel": float(np.median(r6)), "max_rel": float(max(r6)),
                                "n_within_1e-4": int(sum(x <= 1e-4 for x in r6)),
                                "max_rel_floored_1e-3_grad": float(max(f6))},
            "fd_h1e-5_32dirs": {"median_rel": float(np.median(r5)), "max_rel": float(max(r5))},
            "fd_orbital_params_h1e-6": [float(x) for x in rp],
            "direct_adjoint_vs_tree_adjoint": {
                "rel_l2": float(np.linalg.norm(a - bb) / np.linalg.norm(bb)),
                "cosine": float(a @ bb / (np.linalg.norm(a) * np.linalg.norm(bb))),
                "orbital_rel": [float(abs(x - y) / abs(y)) for x, y in zip(gp, dgp)]},
            "direct_adjoint_fd_h1e-6_4dirs_max_rel_floored": float(max(
                floored_errors(dfd, float(np.sqrt((dgx ** 2).sum() + (dgv ** 2).sum())))))},
        "gpu_launches": launches,
    }


def theta_sweep(args, torch, lib, cfg, thetas, flush, k, sampler=None):
    """Per opening angle: FP32-mixed and FP64 ms/substep over k timed
    substeps, walk times, and the force errors of the initial state (FP32 vs
    FP64 walk; both vs an FP64 direct sum on a seeded 4096-body sample)."""
    stream = torch.cuda.current_stream()
    bodies = lib.generate_ics(cfg["kind"], cfg["n"], SEED)
    alive = bodies["mass"] > 0
    n_alive = int(alive.sum())
    rng = np.random.default_rng(1)
    sample = rng.choice(np.nonzero(alive)[0], size=min(4096, n_alive), replace=False)
    out = {}
    for th in thetas:
        row = {}
        accs = {}
        for prec, name in ((lib.PREC_FP32_MIXED, "fp32_mixed"), (lib.PREC_FP64, "fp64")):
            sim = lib.Sim.from_bodies(bodies, softening=cfg["eps"], theta=th, dt=cfg["dt"],
                                      sph=cfg["sph"], precision=prec)
            sim.set_stream(stream.cuda_stream)
            accs[name] = acc(sim.bodies())
            for _ in range(args.warmup):
                sim.substeps_async(1)
            secs = time_substeps(torch, sim, k, flush, sampler)
            sim.sync()
            walk_s = time_phase(torch, sim.gravity_async, 3, flush)
            sim.enable_stats(True)
            sim.gravity_async()
            inter = sim.interactions()
            sim.close()
            row[name] = {"body_substeps_per_s": n_alive * k / secs, "ms_per_substep": 1e3 * secs / k,
                         "steps": k, "walk_ms": 1e3 * walk_s,
                         "interactions_per_body": inter / n_alive,
                         "walk_tflops": FLOP_PER_INTERACTION * inter / walk_s / 1e12}
        g = lib.Sim.from_bodies(bodies, softening=cfg["eps"], theta=th)
        direct = g.direct_forces(sample)
        g.close()
        row["fp32_mixed_speedup"] = (row["fp32_mixed"]["body_substeps_per_s"] /
                                     row["fp64"]["body_substeps_per_s"])
        row["errors"] = {"fp32_vs_fp64_walk": rel_err_stats(accs["fp32_mixed"][alive],
                                                           accs["fp64"][alive]),
                         "fp64_walk_vs_direct": rel_err_stats(accs["fp64"][sample], direct),
                         "fp32_walk_vs_direct": rel_err_stats(accs["fp32_mixed"][sample], direct)}
        out[str(th)] = row
    return out


def target_leg(args, torch, lib, flush, sampler):
    """The stated targets, on the 1M bulge + disk at theta 0.3 and 0.5:
    FP32-mixed >= 5x FP64 plain at force error <= 1e-3 against an FP64 direct
    sum (4096-body sample; median), and FP64 plain >= 50x the reference's CPU
    algorithm on the host cores (main() adds that CPU sample after every
    GPU leg has run)."""
    cfg = CONFIGS["bulge1m"]
    thetas = (0.3, 0.5)
    rows = theta_sweep(args, torch, lib, cfg, thetas, flush, args.steps, sampler)
    out = {"workload": f"bulge1m: {cfg['desc']}", "n_bodies": cfg["n"], "softening": cfg["eps"],
           "dt": cfg["dt"], "steps": args.steps, "thetas": {}}
    for th in thetas:
        row = rows[str(th)]
        err = row["errors"]["fp32_walk_vs_direct"]["median"]
        t = {"fp32_mixed": row["fp32_mixed"], "fp64_plain": row["fp64"],
             "fp32_over_fp64": row["fp32_mixed_speedup"], "errors": row["errors"],
             "fp32_err_vs_direct_median": err,
             "target_5x_at_err_1e-3": bool(row["fp32_mixed_speedup"] >= 5.0 and err <= 1e-3)}
        out["thetas"][str(th)] = t
    return out


def energy_drift(torch, lib, cfg, k, flush):
    """|E(k substeps) - E(0)| / |E(0)| (FP64 kinetic + softened potential, all
    pairs) of FP32-mixed and FP64 runs from the same initial conditions."""
    bodies = lib.generate_ics(cfg["kind"], cfg["n"], SEED)
    out = {"substeps": k, "dt": cfg["dt"]}
    e0 = None
    for prec, name in ((lib.PREC_FP32_MIXED, "fp32_mixed"), (lib.PREC_FP64, "fp64")):
        sim = lib.Sim.from_bodies(bodies, softening=cfg["eps"], theta=cfg["theta"], dt=cfg["dt"],
                                  sph=cfg["sph"], precision=prec)
        if e0 is None:
            ke, pe = sim.energy()
            e0 = ke + pe
            out["e0"] = e0
        t0 = time.perf_counter()
        sim.substeps_async(k)
        sim.sync()
        secs = time.perf_counter() - t0
        ke, pe = sim.energy()
        out[name] = {"rel_drift": abs(ke + pe - e0) / abs(e0), "run_s": secs}
        sim.close()
    return out


def cpu_reference(cfg, steps, seed=SEED, time_budget=None, warmup=0, warmup_budget=30.0):
    """The reference's CPU algorithm (oracle port, OpenMP on every host core):
    `warmup` untimed substeps (at most `warmup_budget` seconds of them), then
    `steps` timed ones (stopping early, after at least 2, once `time_budget`
    seconds have passed). The bodies come from the oracle's generator (equal
    byte for byte to the library's): this leg never loads the library."""
    from cosmosim_gb300.abi import NODE_DTYPE
    from oracle import orc

    orc.build()
    o = orc.Oracle()
    cores = o.set_threads(os.cpu_count() or 1)
    b = o.generate_ics(cfg["kind"], cfg["n"], seed)
    pool = np.zeros(8 * cfg["n"], dtype=NODE_DTYPE)
    o.integrator_init_accelerations(b, 1.0, cfg["eps"], cfg["theta"], pool)
    tw = time.perf_counter()
    for _ in range(warmup):
        o.integrator_step(b, cfg["dt"], 1.0, cfg["eps"], cfg["theta"], pool, int(cfg["sph"]))
        if time.perf_counter() - tw > warmup_budget:
            break
    done = 0
    t0 = time.perf_counter()
    while done < steps:
        o.integrator_step(b, cfg["dt"], 1.0, cfg["eps"], cfg["theta"], pool, int(cfg["sph"]))
        done += 1
        if time_budget and time.perf_counter() - t0 > time_budget and done >= 2:
            break
    secs = time.perf_counter() - t0
    n_alive = int((b["mass"] > 0).sum())
    return {"value": n_alive * done / secs, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{done} substeps of the {cfg['n']}-body workload (oracle/orc.c, "
                      f"OpenMP, {cores} threads)", "secs": secs, "steps": done}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="cuda", choices=["cuda", "reference"])
    ap.add_argument("--config", default="merger100k",
                    choices=sorted(CONFIGS) + ["ensemble64", "adjoint10k"])
    ap.add_argument("--no-targets", action="store_true",
                    help="skip the 1M-body target leg (theta 0.3 and 0.5) of the default line")
    ap.add_argument("--cpu-budget", type=float, default=20.0,
                    help="seconds of CPU work for the cpu_baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", default=None, choices=["fp32", "fp64", "both"],
                    help="only run warm-up + --steps substeps at this precision (for ncu)")
    ap.add_argument("--n", type=int, default=None,
                    help="--profile only: body count of a smaller case of the workload")
    ap.add_argument("--thetas", default=None,
                    help="comma-separated opening angles: add a per-theta speed/error study")
    ap.add_argument("--drift", type=int, default=0,
                    help="add the energy drift over this many substeps (FP32-mixed and FP64)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_env()
    if args.config == "adjoint10k":
        if rank == 0 and args.impl == "cuda":
            import torch

            torch.cuda.set_device(local)
            print(json.dumps(adjoint_line(args)))
        elif rank == 0:
            print(json.dumps({"impl": "reference", "unavailable":
                              "the reference has no adjoint (forward CPU runs: --config merger100k)"}))
        return
    if args.config == "ensemble64":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps(ensemble_reference(args, world)))
            return
        import torch

        torch.cuda.set_device(local)
        work_stream = torch.cuda.Stream()
        torch.cuda.set_stream(work_stream)
        if world > 1:
            torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
        from cosmosim_gb300 import lib

        lib.load()
        fp32_peak, _ = lib.measure_fp_peaks()
        line = ensemble_line(args, torch, lib, rank, world, fp32_peak)
        if rank == 0 and world == 1 and not args.no_cpu_baseline:
            cb = ensemble_reference(args, world)["cpu_baseline"]
            line["cpu_baseline"] = cb
            line["speedup_vs_cpu"] = {"fp32_mixed": line["value"] / cb["value"],
                                      "e2e": line["e2e"]["value"] / cb["value"]}
        if rank == 0:
            print(json.dumps(line))
        if world > 1:
            torch.distributed.barrier()
            torch.distributed.destroy_process_group()
        return
    cfg = CONFIGS[args.config]
    config = {"workload": f"{args.config}: {cfg['desc']}", "n_bodies": cfg["n"],
              "theta": cfg["theta"], "softening": cfg["eps"], "dt": cfg["dt"],
              "sph": cfg["sph"], "l2": "512 MB flush between timed substeps",
              "parallelism": f"replicas x{world}"}

    if args.impl == "reference":
        if rank != 0:
            return
        # warm-up substeps untimed, then the timed ones (at most ~2.5 minutes
        # of them: the line reports the substeps actually timed)
        ref = cpu_reference(cfg, args.steps, time_budget=150.0, warmup=args.warmup)
        line = {"metric": METRIC, "value": ref["value"], "unit": UNIT, "impl": "reference",
                "n_gpus": world, "steps": ref["steps"], "warmup": args.warmup,
                "ms_per_step": 1e3 * ref["secs"] / ref["steps"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config,
                "cpu_baseline": {k: ref[k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": ref["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch

    torch.cuda.set_device(local)
    # a dedicated stream: the library and the timing events share it
    work_stream = torch.cuda.Stream()
    torch.cuda.set_stream(work_stream)
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    from cosmosim_gb300 import lib

    lib.load()
    if args.profile:
        n = args.n or cfg["n"]
        b = lib.generate_ics(cfg["kind"], n, SEED)
        precs = {"fp32": [lib.PREC_FP32_MIXED], "fp64": [lib.PREC_FP64],
                 "both": [lib.PREC_FP32_MIXED, lib.PREC_FP64]}[args.profile]
        for prec in precs:
            sim = lib.Sim.from_bodies(b, softening=cfg["eps"], theta=cfg["theta"], dt=cfg["dt"],
                                      sph=cfg["sph"], precision=prec)
            sim.set_stream(work_stream.cuda_stream)
            sim.substeps_async(args.warmup + args.steps)
            sim.sync()
            print(json.dumps({"profile": prec, "config": args.config, "n": n,
                              "substeps": args.warmup + args.steps,
                              "launches": sim.launch_count()}))
            sim.close()
        return
    fp32_peak, fp64_peak = lib.measure_fp_peaks()
    sampler = ClockSampler(torch.cuda.current_device())
    sampler.start()
    r = run_cuda(args, torch, lib, cfg, rank, world, sampler)
    targets = None
    if rank == 0 and world == 1 and args.config == "merger100k" and not args.no_targets:
        targets = target_leg(args, torch, lib, flush_buffer(torch), sampler)
    clocks = sampler.stop()
    f32, f64 = r["runs"]["fp32_mixed"], r["runs"]["fp64"]
    # whole-job aggregation: max time over ranks
    t32, t64, te = f32["secs"], f64["secs"], r["e2e_s"]
    if world > 1:
        t32, t64, te = max_over_ranks(torch, [t32, t64, te], "cuda")
    value = job_rate(r["n_alive"] * f32["steps"], world, t32)
    v64 = job_rate(r["n_alive"] * f64["steps"], world, t64)
    e2e_value = job_rate(r["n_alive"] * r["e2e_steps"], world, te)
    achieved = FLOP_PER_INTERACTION * f32["interactions"] / f32["walk_s"] / 1e12
    achieved64 = FLOP_PER_INTERACTION * f64["interactions"] / f64["walk_s"] / 1e12
    walk_name, walk_split = walk32_kernel(torch, cfg["n"])
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": f32["steps"],
        "warmup": args.warmup, "ms_per_step": 1e3 * f32["secs"] / f32["steps"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "precision": "FP32 pair forces (compensated sums); FP64 positions, tree moments, drift", "data": "synthetic",
        "config": config,
        "fp64_plain": {"value": v64, "ms_per_step": 1e3 * f64["secs"] / f64["steps"],
                       "steps": f64["steps"], "fp32_mixed_speedup": value / v64,
                       "walk_ms": 1e3 * f64["walk_s"],
                       "walk_tflops": achieved64, "fp64_peak_tflops": fp64_peak,
                       "walk_frac_of_fp64_peak": achieved64 / fp64_peak},
        "phases_ms": {"fp32_mixed": f32["phases"], "fp64": f64["phases"],
                      "walk_alone_fp32": 1e3 * f32["walk_alone_s"],
                      "walk_alone_fp64": 1e3 * f64["walk_alone_s"],
                      "how": "per substep, CUDA events between the phases of the real substep "
                             "(cosmosim_phase_times, direct launches, L2 flushed between "
                             "substeps); walk_alone = the walk launched by itself"},
        "interactions_per_substep": f32["interactions"],
        "walk_traversal": {"warp_steps": f32["warp_steps"],
                           "lane_utilisation": f32["active_lane_steps"] / max(32 * f32["warp_steps"], 1),
                           "interactions_per_lane_step": f32["interactions"] / max(32 * f32["warp_steps"], 1)},
        "roofline": {"bound": "fp32-pipe", "kernel": walk_name,
                     "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak,
                     "traffic": (WALK32U_DRAM_BYTES_PER_BODY if walk_split
                                 else WALK32_DRAM_BYTES_PER_BODY) * cfg["n"],
                     "issue_slots_busy_ncu": WALK32U_ISSUE_BUSY if walk_split else WALK32_ISSUE_BUSY,
                     "note": WALK32_NOTE + ("; this workload takes the split walk: traffic and "
                                            "issue from the capture of k_walk32_units on the 20k "
                                            "disk (profiles/walk_units_disk20k.md)"
                                            if walk_split else "")},
        "errors": r["errors"],
        "e2e": {"value": e2e_value, "unit": UNIT, "api": "integrator_step (pinned host Body[])",
                "steps": r["e2e_steps"], "h2d_bytes_per_step": 168 * cfg["n"],
                "d2h_bytes_per_step": (104 if cfg["sph"] else 72) * cfg["n"] + 104 * r["e2e_nodes"]},
        "gpu_launches": f32["launches"],
        "clocks": clocks,
    }
    if rank == 0 and args.thetas:
        line["theta_sweep"] = theta_sweep(args, torch, lib, cfg,
                                          [float(t) for t in args.thetas.split(",")],
                                          flush_buffer(torch), args.steps)
    if rank == 0 and args.drift > 0:
        line["energy_drift"] = energy_drift(torch, lib, cfg, args.drift, flush_buffer(torch))
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_reference(cfg, 10**9, time_budget=args.cpu_budget)
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        line["speedup_vs_cpu"] = {"fp32_mixed": value / cb["value"], "fp64_plain": v64 / cb["value"],
                                  "e2e": e2e_value / cb["value"]}
        if targets is not None:
            for th, t in targets["thetas"].items():
                cbt = cpu_reference(dict(CONFIGS["bulge1m"], theta=float(th)), 10**9,
                                    time_budget=args.cpu_budget)
                t["cpu_baseline"] = {k: cbt[k] for k in ("value", "unit", "cores", "kind", "sample")}
                t["fp64_over_cpu"] = t["fp64_plain"]["body_substeps_per_s"] / cbt["value"]
                t["fp32_over_cpu"] = t["fp32_mixed"]["body_substeps_per_s"] / cbt["value"]
                t["target_50x_cpu"] = bool(t["fp64_over_cpu"] >= 50.0)
    if targets is not None:
        line["targets_1m"] = targets
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
