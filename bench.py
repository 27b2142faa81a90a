#!/usr/bin/env python3
"""Benchmark of the GB300 BioFVM reaction-diffusion step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

A step is one `solve(1)` of the large single-domain workload (320^3 voxels x 8
substrates, FP32 field, 1,000,000 agents, Dirichlet on the x faces and 10,000
interior voxels): three ADI sweeps, Dirichlet, cells.  The metric is
voxel-substrate-steps per second (VSS/s) = voxels * substrates * steps / time.

Arms
  gb300      (default) the hand-written sm_103a kernels through the C ABI.  Inputs
             are resident in HBM when the timed region starts; the field (1.05 GB)
             is larger than L2, so no flush is needed between steps.  `e2e` repeats
             the step through the same C ABI with host buffers: per step the agent
             positions/activity go host->device from pinned memory, the voxel
             ballot is rebuilt (the agents moved) and the whole field comes back
             device->host into pinned memory; two host buffers in turn, so the
             readback of step k overlaps step k+1.
  reference  the reference's CPU algorithm (the OpenMP restatement in oracle/,
             FP64, all host threads) on the same workload, a bounded number of
             steps.  Under torchrun only rank 0 runs it.
Multi-GPU: every rank steps its own replica (the path does not shard a single
domain); value = all ranks' VSS / max-over-ranks time; scaling "weak".
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "voxel-substrate-steps/s + % HBM roofline, batched vs plain; serve p50/p99"
UNIT = "voxel-substrate-steps/s"
WORKLOAD = dict(n=320, S=8, agents=1_000_000, interior=10_000, seed=1)
FALLBACK_HBM_GBS = 6800.0


def workload_config(w):
    n = w["n"]
    return {"workload": f"large_{n}: {n}^3 voxels of 20 um x {w['S']} substrates, FP32 field, "
                        f"{w['agents']:,} agents (internalized tracking on), Dirichlet x faces + "
                        f"{w['interior']:,} interior voxels, D log-uniform [10,1e5], decay log-uniform [1e-4,1]",
            "grid": [n, n, n], "substrates": w["S"], "agents": w["agents"], "seed": w["seed"],
            "l2": "inputs larger than L2 (field %.2f GB > 129 MB L2); no flush" % (n ** 3 * w["S"] * 4 / 1e9),
            "step": "solve(1): x/y/z Thomas sweeps, Dirichlet faces+interior, cell secretion/uptake"}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(x, world, device="cuda"):
    """The largest of every rank's x (the slowest replica sets the job's time)."""
    if world <= 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, seconds):
    """Whole-job throughput of `world` replicas that each processed units_per_rank
    units, timed by the slowest (weak scaling: the per-GPU work is fixed)."""
    return units_per_rank * world / seconds


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            return float(d["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (of measured)"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback 6.8 TB/s (of fallback)"


def ncu_traffic(kernel):
    """DRAM bytes per launch from the committed ncu summary, when one exists."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return None
    try:
        d = json.load(open(p))
        return d.get(kernel, {}).get("bytes_per_launch")
    except Exception:
        return None


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[3 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def build_problem(w):
    from physicore_gb300 import workloads as W
    return W.large(seed=w["seed"], n=w["n"], S=w["S"], agents=w["agents"], interior=w["interior"])


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def time_reference(p, steps, warmup, threads, budget_s=60.0):
    """The reference algorithm on the host: FP64, OpenMP over `threads` threads."""
    from oracle import oracle
    from physicore_gb300 import workloads as W
    o = W.apply(oracle.OracleSolver(threads=threads), p)
    o.solve(1)  # the first solve call rebuilds the ballots (openmp_solver.cpp:39)
    for _ in range(max(0, warmup - 1)):
        o.solve(1)
    done, t0 = 0, time.perf_counter()
    while done < steps:
        o.solve(1)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    n, S = p["bbmax"][0] // p["voxel"][0], len(p["D"])
    return n ** 3 * S * done / dt, done, dt


def run_reference(args, w):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    p = build_problem(w)
    threads = cpu_threads()
    value, done, secs = time_reference(p, args.steps, min(args.warmup, 1), threads,
                                       budget_s=float(os.environ.get("PCG_REF_BUDGET_S", "90")))
    sample = f"{done} timed steps (after 1 warm-up) of the {args.steps}-step request, {secs:.1f} s"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": done, "warmup": 1, "ms_per_step": 1e3 * secs / max(done, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded PCG64)",
            "config": workload_config(w),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gb300(args, w):
    import torch

    import physicore_gb300 as pcg
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    p = build_problem(w)
    from physicore_gb300 import workloads as W
    s = W.apply(pcg.Solver(pcg.FP32, device=local), p)
    n, S = w["n"], w["S"]
    vss_step = n ** 3 * S
    s.solve(1)  # first call: ballots rebuilt
    for _ in range(max(0, args.warmup - 1)):
        s.solve(1)
    s.synchronize()

    stream = torch.cuda.ExternalStream(s.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.set_kernel_timing(True)
    s.reset_kernel_stats()
    launches0 = s.launch_count()
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            s.solve(1)
        ev1.record(stream)
        ev1.synchronize()
    torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    launches = s.launch_count() - launches0
    stats = s.kernel_stats()
    s.set_kernel_timing(False)
    ms = max_over_ranks(ms, world)
    value = job_rate(vss_step * args.steps, world, ms / 1e3)

    # roofline of the dominant kernel (largest share of device time)
    peak, peak_src = measured_peaks()
    timed = {k: v for k, v in stats.items() if v["launches"] and v["ms"] > 0}
    dom = max(timed, key=lambda k: timed[k]["ms"])
    d = timed[dom]
    per_launch_bytes = d["bytes"] / d["launches"]
    achieved = per_launch_bytes / (d["ms"] / d["launches"] / 1e3) / 1e9
    step_bytes = sum(v["bytes"] for v in stats.values()) / args.steps
    kernels = {k: {"launches": v["launches"], "ms_total": round(v["ms"], 4),
                   "share": round(v["ms"] / sum(x["ms"] for x in timed.values()), 4),
                   "gbps": round(v["bytes"] / (v["ms"] / 1e3) / 1e9, 1) if v["ms"] > 0 else None}
               for k, v in timed.items()}

    # the per-step FP64 mass check on the same workload (off in the timed step above)
    mc_steps = max(3, min(args.steps, 100))
    s.set_mass_check(True)
    s.solve(1)
    s.synchronize()
    s.set_mass_check(True)  # record from here on
    s.set_kernel_timing(True)
    s.reset_kernel_stats()
    ev0.record(stream)
    for _ in range(mc_steps):
        s.solve(1)
    ev1.record(stream)
    ev1.synchronize()
    mc_ms = ev0.elapsed_time(ev1) / mc_steps
    mc_stats = s.kernel_stats().get("mass_check", {})
    s.set_kernel_timing(False)
    chk = s.get_mass_check()
    s.set_mass_check(False)
    mass_check = {"steps": chk["steps"], "ms_per_step": round(mc_ms, 4),
                  "overhead": round(mc_ms / (ms / args.steps) - 1.0, 4),
                  "worst_residual": float(chk["worst"].max()),
                  "residual": "max over substrates and steps of |after*f - before|/|before|, f the product of "
                              "the sweep matrices' column sums",
                  "kernel_gbps": round(mc_stats["bytes"] / (mc_stats["ms"] / 1e3) / 1e9, 1)
                  if mc_stats.get("ms") else None}

    # end to end through the C ABI with host buffers
    A = p["agents"]["volumes"].size
    pos_h = torch.empty((A, 3), dtype=torch.float64, pin_memory=True)
    act_h = torch.empty(A, dtype=torch.uint8, pin_memory=True)
    pos_h.numpy()[:] = p["agents"]["positions"]
    act_h.numpy()[:] = p["agents"]["is_active"]
    # two pinned field buffers: step k's field is read back while step k+1 runs
    fields = [torch.empty((S, n, n, n), dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
    pos_np, act_np, field_np = pos_h.numpy(), act_h.numpy(), fields[0]
    e2e_steps = max(3, min(args.steps, args.e2e_steps))
    pending = []

    def e2e_step(k):
        # agents moved: upload positions, rebuild the voxel ballot, step, read the field
        s.update_agents(pos_np, act_np)
        s.recompute_positional_data()
        s.solve(1)
        pending.append(s.get_field_async(fields[k % 2], layout=pcg.LAYOUT_PLANAR))
        if len(pending) > 1:  # the previous step's field is in host memory
            s.wait_field(pending.pop(0))

    e2e_step(0)
    s.wait_field(pending.pop(0))
    barrier()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        e2e_step(k)
    s.wait_field(pending.pop(0))  # every step's field is in host memory
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = {"value": job_rate(vss_step * e2e_steps, world, e2e_s), "unit": UNIT,
           "h2d_bytes_per_step": int(pos_np.nbytes + act_np.nbytes),
           "d2h_bytes_per_step": int(field_np.nbytes), "steps": e2e_steps,
           "path": "pcg_update_agents(pinned) -> pcg_recompute_positional_data -> pcg_solve(1) -> "
                   "pcg_get_field_async(pinned, planar f32), waited one step later (every step's field "
                   "reaches host memory inside the timed region)"}
    s.close()

    if rank != 0:
        return
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        threads = cpu_threads()
        v, done, secs = time_reference(p, args.cpu_steps, 1, threads, budget_s=30.0)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{done} steps of large_{n} on the oracle (FP64 OpenMP restatement), {secs:.1f} s"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded PCG64)",
            "config": dict(workload_config(w), parallelism=f"replicas x{world}"),
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": ncu_traffic(dom),
                         "algorithmic_bytes_per_launch": per_launch_bytes, "peak_source": peak_src},
            "step_roofline": {"achieved": round(step_bytes / (ms / args.steps / 1e3) / 1e9, 1), "peak": peak,
                              "frac": round(step_bytes / (ms / args.steps / 1e3) / 1e9 / peak, 4),
                              "algorithmic_bytes_per_step": step_bytes},
            "kernels": kernels, "clocks": clk.summary(), "gpu_launches": int(launches), "e2e": e2e,
            "cpu_baseline": cpu, "mass_check": mass_check}
    if args.batch_domains > 0:
        line["batched"] = run_batched(args, local, ClockSampler)
    if args.serve_duration > 0:
        line["serve"] = run_serve(args, local)
    if args.dense_steps > 0:
        line["dense"] = run_dense(args, local)
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_batched(args, local, clock_sampler=None):
    """The batched workload (256 uneven domains, FP32): the same contexts stepped one
    after another on one stream (the plain path: pcg_solve per domain) and then
    together through a batch (one launch per phase, CUDA-graph replay, autotuned)."""
    import torch

    import physicore_gb300 as pcg
    from physicore_gb300 import workloads as W
    t0 = time.perf_counter()
    solvers = [W.apply(pcg.Solver(pcg.FP32, device=local), p)
               for p in W.batched_uneven(count=args.batch_domains)]
    setup_s = time.perf_counter() - t0
    vss_step = sum(s.voxels * s.S for s in solvers)
    steps, warm = args.batch_steps, max(3, args.warmup)

    # one stream owned here (it must outlive every context that uses it)
    cs = torch.cuda.Stream()
    for s in solvers:
        s.set_stream(cs.cuda_stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(warm):
        for s in solvers:
            s.solve(1)
    solvers[0].synchronize()
    l0 = sum(s.launch_count() for s in solvers)
    ev0.record(cs)
    for _ in range(steps):
        for s in solvers:
            s.solve(1)
    ev1.record(cs)
    ev1.synchronize()
    plain_ms = ev0.elapsed_time(ev1)
    plain_launches = sum(s.launch_count() for s in solvers) - l0

    b = pcg.Batch(solvers)
    t0 = time.perf_counter()
    if not args.no_batch_autotune:
        b.autotune()
    b.synchronize()
    tune_s = time.perf_counter() - t0
    bs = torch.cuda.ExternalStream(b.stream())
    for _ in range(warm):
        b.solve(1)
    b.synchronize()
    b.reset_kernel_stats()
    sampler = clock_sampler(local) if clock_sampler else None
    if sampler:
        sampler.__enter__()
    ev0.record(bs)
    b.solve(steps)
    ev1.record(bs)
    ev1.synchronize()
    if sampler:
        sampler.__exit__(None, None, None)
    batched_ms = ev0.elapsed_time(ev1)
    batched_launches = b.launch_count()
    step_bytes = sum(v["bytes"] for v in b.kernel_stats().values()) / steps
    # per-kernel times from a short run of direct (event-timed) launches
    b.set_kernel_timing(True)
    b.reset_kernel_stats()
    kt = min(steps, 20)
    b.solve(kt)
    b.synchronize()
    stats = b.kernel_stats()
    b.set_kernel_timing(False)
    peak, peak_src = measured_peaks()
    timed = {k: v for k, v in stats.items() if v["launches"] and v["ms"] > 0}
    total_ms = sum(v["ms"] for v in timed.values())
    kernels = {k: {"launches": v["launches"], "share": round(v["ms"] / total_ms, 4),
                   "us_per_launch": round(1e3 * v["ms"] / v["launches"], 1),
                   "gbps": round(v["bytes"] / (v["ms"] / 1e3) / 1e9, 1)} for k, v in timed.items()}
    dom = max(timed, key=lambda k: timed[k]["ms"])
    dgb = timed[dom]["bytes"] / (timed[dom]["ms"] / 1e3) / 1e9
    tuned = b.describe()
    b.close()
    for s in solvers:
        s.set_stream(None)
        s.close()
    plain_v = vss_step * steps / (plain_ms / 1e3)
    batched_v = vss_step * steps / (batched_ms / 1e3)
    out = {"workload": f"batched_{args.batch_domains}: {args.batch_domains} domains, sides log-uniform [32,160] "
                       "per axis, 1-6 substrates, 100-50,000 agents, FP32, x-face Dirichlet + interior nodes",
           "vss_per_step": vss_step, "steps": steps, "warmup": warm, "setup_s": round(setup_s, 1),
           "plain": {"value": plain_v, "ms_per_step": plain_ms / steps, "gpu_launches": int(plain_launches),
                     "path": "pcg_solve(1) per domain, one domain after another on one stream"},
           "batched": {"value": batched_v, "ms_per_step": batched_ms / steps, "gpu_launches": int(batched_launches),
                       "path": "pcg_batch_solve: one launch per phase over all domains, CUDA-graph replay",
                       "autotune_s": round(tune_s, 2)},
           "speedup": batched_v / plain_v, "unit": UNIT,
           "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(dgb, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(dgb / peak, 4), "peak_source": peak_src},
           "step_roofline": {"achieved": round(step_bytes / (batched_ms / steps / 1e3) / 1e9, 1), "peak": peak,
                             "frac": round(step_bytes / (batched_ms / steps / 1e3) / 1e9 / peak, 4),
                             "algorithmic_bytes_per_step": step_bytes},
           "kernels": kernels, "autotune": tuned["buckets"]}
    if sampler:
        out["clocks"] = sampler.summary()
    return out


class PinnedArena:
    """First-fit extents of one pinned float32 buffer, shared by a producer that
    takes slices and a consumer that gives them back."""

    def __init__(self, torch, elems):
        self.buf = torch.empty(elems, dtype=torch.float32, pin_memory=True).numpy()
        self.free = [(0, elems)]  # sorted (offset, length)
        self.cv = threading.Condition()

    def take(self, n):
        """Offset of n free elements, or None when no free extent is that long."""
        with self.cv:
            for k, (o, l) in enumerate(self.free):
                if l >= n:
                    self.free[k:k + 1] = [(o + n, l - n)] if l > n else []
                    return o
            return None

    def give(self, off, n):
        with self.cv:
            self.free.append((off, n))
            self.free.sort()
            merged = []
            for o, l in self.free:
                if merged and merged[-1][0] + merged[-1][1] == o:
                    merged[-1] = (merged[-1][0], merged[-1][1] + l)
                else:
                    merged.append((o, l))
            self.free = merged
            self.cv.notify_all()


def run_serve(args, local):
    """The served request stream (Poisson arrivals of independent simulations of
    random sizes and step counts; workloads.ServedStream) through the simulation
    server: a feeder thread submits each request at its arrival time with a slice
    of a pinned host arena for its field, which the server fills (FP32, planar)
    before returning the request; the main thread collects finished ones, frees
    their slices and destroys them.  Reports time-to-result percentiles (submit ->
    field in host memory, on the server's clock and on the collector's) and
    aggregate VSS/s."""
    import torch

    import physicore_gb300 as pcg
    from physicore_gb300 import workloads as W
    stream = W.ServedStream(duration=args.serve_duration)
    n = len(stream)
    srv = pcg.Server(pcg.FP32, device=local, steps_per_tick=args.serve_tick, reserve_bytes=1 << 30)
    elems = [int(np.prod(stream.sides[i]) * stream.S[i]) for i in range(n)]
    # pinned slices for the fields of requests in flight; beyond 16 GB of them (a
    # backlog under overload) a request gets a pageable buffer instead
    arena = PinnedArena(torch, min(sum(elems), 4 << 30))
    host = arena.buf
    submit_wall = np.zeros(n)
    lag = np.zeros(n)
    slices = {}
    pageable = [0]
    err = []

    def feed():
        t0 = time.perf_counter()
        try:
            for i in range(n):
                delay = stream.arrivals[i] - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                s = stream.request(pcg.Solver(pcg.FP32, device=local), i)
                lag[i] = max(0.0, time.perf_counter() - t0 - stream.arrivals[i])
                nx, ny, nz = (int(v) for v in stream.sides[i])
                off = arena.take(elems[i])
                slices[i] = off
                pageable[0] += off is None
                out = (host[off: off + elems[i]] if off is not None else np.empty(elems[i], np.float32))
                submit_wall[i] = time.perf_counter()
                srv.submit(s, int(stream.steps[i]), i, out=out.reshape(int(stream.S[i]), nz, ny, nx),
                           layout=pcg.LAYOUT_PLANAR)
        except Exception as e:  # surfaced by the main thread
            err.append(e)

    th = threading.Thread(target=feed, daemon=True)
    t_start = time.perf_counter()
    th.start()
    lat_dev, lat_host, statuses, vss_done, agent_steps = [], [], {}, 0, 0
    t_first = t_last = None
    got = 0
    profile, next_sample = [], 0.5  # [t, active, queued, cumulative vss] every half second
    while got < n and not err:
        if time.perf_counter() - t_start >= next_sample:
            sp = srv.stats()
            profile.append([round(time.perf_counter() - t_start, 2), sp["active"], sp["queued"], sp["vss"]])
            next_sample += 0.5
        for r in srv.poll(64, wait_ms=20):
            got += 1
            statuses[r["status"]] = statuses.get(r["status"], 0) + 1
            s = r["solver"]
            i = r["tag"]
            off = slices.pop(i)
            if off is not None:
                arena.give(off, elems[i])
            if r["status"] == "done":
                lat_host.append(time.perf_counter() - submit_wall[i])
                lat_dev.append(r["t_done"] - r["t_submit"])
                vss_done += stream.vss(i)
                agent_steps += int(stream.A[i]) * int(stream.steps[i])
                t_first = r["t_submit"] if t_first is None else min(t_first, r["t_submit"])
                t_last = r["t_done"] if t_last is None else max(t_last, r["t_done"])
            s.close()
        if time.perf_counter() - t_start > args.serve_duration * 20 + 120:
            break
    wall = time.perf_counter() - t_start
    st = srv.stats()
    srv.close()
    if err:
        raise err[0]
    # plain: a sample of the same requests, one after another through pcg_solve
    # (create, solve all steps, read the field, destroy), on the same device
    sample = list(range(0, n, max(1, n // args.serve_plain_sample)))[: args.serve_plain_sample]
    cs = torch.cuda.Stream()
    t0 = time.perf_counter()
    vss_plain = 0
    for i in sample:
        s = stream.request(pcg.Solver(pcg.FP32, device=local), i)
        s.set_stream(cs.cuda_stream)
        s.initialize()
        s.solve(int(stream.steps[i]))
        nx, ny, nz = (int(v) for v in stream.sides[i])
        S = int(stream.S[i])
        s.get_field(layout=pcg.LAYOUT_PLANAR, dtype=np.float32, out=host[: S * nx * ny * nz].reshape(S, nz, ny, nx))
        s.set_stream(None)
        s.close()
        vss_plain += stream.vss(i)
    plain_s = time.perf_counter() - t0
    offered = sum(stream.vss(i) for i in range(n)) / args.serve_duration
    q = lambda a, p: float(np.percentile(a, p)) if len(a) else None
    return {"workload": f"served: Poisson arrivals at 200/s for {args.serve_duration:g} s ({n} requests), sides "
                        "log-uniform [32,256] per axis, 1-8 substrates, 0-200,000 agents, steps log-uniform "
                        "[10,1000], FP32",
            "requests": n, "statuses": statuses, "offered_vss_per_s": offered,
            "value": vss_done / (t_last - t_first) if t_last else None, "unit": UNIT,
            "agent_steps_per_s": agent_steps / (t_last - t_first) if t_last else None,
            "plain": {"value": vss_plain / plain_s, "requests": len(sample),
                      "path": "the same requests (an even sample) one after another: pcg_create, pcg_solve(steps), "
                              "pcg_get_field, pcg_destroy"},
            "speedup_vs_plain": (vss_done / (t_last - t_first)) / (vss_plain / plain_s) if t_last else None,
            "time_to_result_s": {"p50": q(lat_dev, 50), "p99": q(lat_dev, 99), "mean": float(np.mean(lat_dev))
                                 if lat_dev else None,
                                 "measured": "submit -> field (FP32, planar) in pinned host memory, server clock"},
            "time_to_host_s": {"p50": q(lat_host, 50), "p99": q(lat_host, 99),
                               "measured": "submit -> result collected by the caller (includes its polling)"},
            "feeder_lag_s": {"p50": q(lag, 50), "max": float(lag.max()) if n else None},
            "result_buffers": {"pinned": int(n - pageable[0]), "pageable": int(pageable[0])},
            "server": {k: (round(st[k], 3) if isinstance(st[k], float) else st[k])
                       for k in ("ticks", "rebuilds", "prebuilds", "steps", "admitted", "refused", "failed",
                                 "rebuild_s", "prebuild_s", "step_s", "admit_s")},
            "steps_per_tick": args.serve_tick, "wall_s": round(wall, 2),
            "profile": {"columns": ["t_s", "active", "queued", "vss_per_s_over_the_half_second"],
                        "rows": [[t, a, q, (v - profile[k - 1][3]) / (t - profile[k - 1][0]) if k else v / t]
                                 for k, (t, a, q, v) in enumerate(profile)]}}


def run_dense(args, local):
    """The dense-agent stress workload (200^3 x 4 FP32, 4,000,000 agents in a
    Gaussian cluster of sigma 200 um, up to ~100 agents per voxel): device time per
    step with the agents fixed, and with the ballot rebuilt every step (as when the
    agents move each step), with the cell kernels' times."""
    import torch

    import physicore_gb300 as pcg
    from physicore_gb300 import workloads as W
    p = W.dense()
    s = W.apply(pcg.Solver(pcg.FP32, device=local), p)
    cs = torch.cuda.Stream()
    s.set_stream(cs.cuda_stream)
    steps = args.dense_steps
    for _ in range(max(3, args.warmup)):
        s.solve(1)
    s.synchronize()
    counts = s.get_counts()

    def timed(k, rebuild):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(cs)
        for _ in range(k):
            if rebuild:
                s.recompute_positional_data()
            s.solve(1)
        ev1.record(cs)
        ev1.synchronize()
        return ev0.elapsed_time(ev1) / k

    def kernels(k, rebuild):
        s.set_kernel_timing(True)
        s.reset_kernel_stats()
        for _ in range(k):
            if rebuild:
                s.recompute_positional_data()
            s.solve(1)
        s.synchronize()
        st = s.kernel_stats()
        s.set_kernel_timing(False)
        return {kk: round(v["ms"] / v["launches"] * 1e3, 1) for kk, v in st.items() if v["launches"]}

    vss = s.voxels * s.S
    A = int(p["agents"]["volumes"].size)
    ms_fixed = timed(steps, False)
    ms_moving = timed(max(10, steps // 5), True)
    out = {"workload": "dense_200: 200^3 voxels x 4 substrates FP32, 4,000,000 agents N(centre, 200 um) "
                       "(internalized tracking on)", "vss_per_step": vss, "agents": A,
           "max_agents_per_voxel": int(counts.max()), "occupied_voxels": int((counts > 0).sum()),
           "steps": steps,
           "agents_fixed": {"ms_per_step": ms_fixed, "value": vss / (ms_fixed / 1e3), "unit": UNIT,
                            "agent_steps_per_s": A / (ms_fixed / 1e3), "kernels_us": kernels(10, False)},
           "ballot_rebuilt_every_step": {"ms_per_step": ms_moving, "value": vss / (ms_moving / 1e3), "unit": UNIT,
                                         "agent_steps_per_s": A / (ms_moving / 1e3),
                                         "kernels_us": kernels(10, True)}}
    s.set_stream(None)
    s.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--n", type=int, default=WORKLOAD["n"], help="grid side (default: the 320^3 workload)")
    ap.add_argument("--batch-domains", type=int, default=256, help="domains of the batched workload (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=200)
    ap.add_argument("--no-batch-autotune", action="store_true", help="keep the default line mappings")
    ap.add_argument("--only-batched", action="store_true", help="run only the batched workload")
    ap.add_argument("--serve-duration", type=float, default=10.0, help="seconds of request arrivals (0: skip)")
    ap.add_argument("--serve-tick", type=int, default=8, help="steps between admission points")
    ap.add_argument("--only-serve", action="store_true", help="run only the served request stream")
    ap.add_argument("--serve-plain-sample", type=int, default=100, help="requests timed one after another")
    ap.add_argument("--dense-steps", type=int, default=100, help="steps of the dense-agent workload (0: skip)")
    ap.add_argument("--only-dense", action="store_true", help="run only the dense-agent workload")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    w = dict(WORKLOAD, n=args.n)
    if args.impl == "reference":
        run_reference(args, w)
    elif args.only_serve:
        import torch
        torch.cuda.set_device(dist_env()[2])
        print(json.dumps(run_serve(args, dist_env()[2])), flush=True)
    elif args.only_dense:
        import torch
        torch.cuda.set_device(dist_env()[2])
        print(json.dumps(run_dense(args, dist_env()[2])), flush=True)
    elif args.only_batched:
        import torch
        torch.cuda.set_device(dist_env()[2])
        print(json.dumps(run_batched(args, dist_env()[2], ClockSampler)), flush=True)
    else:
        run_gb300(args, w)


if __name__ == "__main__":
    main()
