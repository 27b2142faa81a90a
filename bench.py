#!/usr/bin/env python3
"""Benchmark of the GB300 BioFVM reaction-diffusion step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--detail-out FILE]

A step is one `solve(1)` of the large single-domain workload (320^3 voxels x 8
substrates, FP32 field, 1,000,000 agents, Dirichlet on the x faces and 10,000
interior voxels): three ADI sweeps, Dirichlet, cells, and the per-step FP64
mass check of the sweeps.  The metric is voxel-substrate-steps per second
(VSS/s) = voxels * substrates * steps / time.

Output: stdout carries exactly one line, the compact JSON headline (strict JSON,
a few KB), printed last.  Every sub-measurement's full record (per-kernel tables,
the served stream's queue profile, autotuner buckets, ...) is written to stderr
as one JSON line per leg, and to --detail-out as one JSON document when given.

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
import ctypes
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

METRIC = "voxel-substrate-steps/s + % HBM roofline, batched vs plain; serve p50/p99"
UNIT = "voxel-substrate-steps/s"
WORKLOAD = dict(n=320, S=8, agents=1_000_000, interior=10_000, seed=1)
FALLBACK_HBM_GBS = 6800.0
FP32_RTOL = 1e-5
FP64_RTOL = 1e-12


def workload_config(w, mass_check=True):
    n = w["n"]
    return {"workload": f"large_{n}: {n}^3 voxels of 20 um x {w['S']} substrates, FP32 field, "
                        f"{w['agents']:,} agents, Dirichlet x faces + {w['interior']:,} interior voxels",
            "grid": [n, n, n], "substrates": w["S"], "agents": w["agents"], "seed": w["seed"],
            "l2": "inputs larger than L2 (field %.2f GB > 129 MB L2); no flush" % (n ** 3 * w["S"] * 4 / 1e9),
            "step": "solve(1): x/y/z Thomas sweeps, Dirichlet faces+interior, cell secretion/uptake"
                    + (", FP64 mass check" if mass_check else "")}


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


def _finite(x):
    """JSON-safe: NaN/inf become None (the headline is strict JSON)."""
    if isinstance(x, float) and not math.isfinite(x):
        return None
    if isinstance(x, dict):
        return {k: _finite(v) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [_finite(v) for v in x]
    if isinstance(x, (np.floating,)):
        return _finite(float(x))
    if isinstance(x, (np.integer,)):
        return int(x)
    return x


def r4(x):
    return None if x is None else float("%.4g" % x)


class Details:
    """Full records of every leg: one JSON line each on stderr, and the whole set
    in one file at the end when a path is given."""

    def __init__(self, path):
        self.path = path
        self.items = {}

    def add(self, name, obj):
        obj = _finite(obj)
        self.items[name] = obj
        print(json.dumps({"detail": name, **obj} if isinstance(obj, dict) else {"detail": name, "value": obj},
                         allow_nan=False), file=sys.stderr, flush=True)

    def write(self):
        if not self.path:
            return
        d = os.path.dirname(os.path.abspath(self.path))
        os.makedirs(d, exist_ok=True)
        with open(self.path, "w") as f:
            json.dump(self.items, f, indent=1, allow_nan=False)


class ClockSampler:
    """Samples SM clocks, power and throttle reasons during a timed region: through
    NVML (every 5 ms, so short regions get samples) when libnvidia-ml loads, else
    with nvidia-smi every 200 ms.  Only reads the GPU's state."""

    NAMES = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []  # (sm_mhz, max_mhz, reasons set)
        self.proc = None
        self.stop = threading.Event()
        self.thread = None
        self.nvml = None
        self.handle = None

    def _nvml_open(self):
        try:
            L = ctypes.CDLL("libnvidia-ml.so.1")
            if L.nvmlInit_v2() != 0:
                return False
            h = ctypes.c_void_p()
            ok = False
            try:
                import torch
                uuid = str(torch.cuda.get_device_properties(self.device).uuid)
                ok = L.nvmlDeviceGetHandleByUUID(("GPU-" + uuid).encode(), ctypes.byref(h)) == 0
            except Exception:
                ok = False
            if not ok:
                vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
                idx = int(vis.split(",")[self.device]) if vis and vis.split(",")[0].isdigit() else self.device
                ok = L.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(idx), ctypes.byref(h)) == 0
            if not ok:
                return False
            self.nvml, self.handle = L, h
            return True
        except Exception:
            return False

    def _nvml_loop(self):
        L, h = self.nvml, self.handle
        clk, mx, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        get_reasons = getattr(L, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            L.nvmlDeviceGetCurrentClocksThrottleReasons
        while not self.stop.is_set():
            if L.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk)) == 0 and \
                    L.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:
                reasons = set()
                if get_reasons(h, ctypes.byref(rs)) == 0:
                    reasons = {n for bit, n in self.NAMES.items() if rs.value & bit}
                self.rows.append((float(clk.value), float(mx.value), reasons))
            self.stop.wait(0.005)

    def _smi_loop(self):
        for line in self.proc.stdout:
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 7 and p[0].replace(".", "").isdigit():
                names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
                self.rows.append((float(p[0]), float(p[1]) if p[1].replace(".", "").isdigit() else 0.0,
                                  {names[k] for k in range(4) if p[3 + k].lower().startswith("active")}))

    def __enter__(self):
        if self._nvml_open():
            self.thread = threading.Thread(target=self._nvml_loop, daemon=True)
            self.thread.start()
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._smi_loop, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.nvml is not None:
            self.stop.set()
            self.thread.join(timeout=2)
        elif self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [r[0] for r in self.rows]
        mx = [r[1] for r in self.rows if r[1] > 0]
        reasons = sorted(set().union(*[r[2] for r in self.rows]))
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows), "via": "nvml" if self.nvml is not None else "nvidia-smi"}


def bind_near_gpu(device):
    """Restricts this process to the CPUs that NVML reports as local to `device`
    (pinned host buffers are then placed on the GPU's own host memory node);
    returns the previous CPU set, or None when nothing was changed.  Reads the
    GPU's topology only."""
    try:
        prev = os.sched_getaffinity(0)
        L = ctypes.CDLL("libnvidia-ml.so.1")
        if L.nvmlInit_v2() != 0:
            return None
        h = ctypes.c_void_p()
        ok = False
        try:
            import torch
            uuid = str(torch.cuda.get_device_properties(device).uuid)
            ok = L.nvmlDeviceGetHandleByUUID(("GPU-" + uuid).encode(), ctypes.byref(h)) == 0
        except Exception:
            ok = False
        if not ok:
            return None
        words = (ctypes.c_ulong * 16)()
        if L.nvmlDeviceGetCpuAffinity(h, ctypes.c_uint(16), words) != 0:
            return None
        local = {64 * k + b for k in range(16) for b in range(64) if (words[k] >> b) & 1}
        cpus = local & prev
        if not cpus or cpus == prev:
            return None
        os.sched_setaffinity(0, cpus)
        return prev
    except Exception:
        return None


def build_problem(w):
    from physicore_gb300 import workloads as W
    return W.large(seed=w["seed"], n=w["n"], S=w["S"], agents=w["agents"], interior=w["interior"])


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def time_reference(p, steps, warmup, threads, budget_s=60.0):
    """The reference algorithm on the host: FP64, OpenMP over `threads` threads.
    Returns (VSS/s, timed steps, seconds, the oracle, solve(1) calls made)."""
    from oracle import oracle
    from physicore_gb300 import workloads as W
    o = W.apply(oracle.OracleSolver(threads=threads), p)
    o.solve(1)  # the first solve call rebuilds the ballots (openmp_solver.cpp:39)
    calls = 1
    for _ in range(max(0, warmup - 1)):
        o.solve(1)
        calls += 1
    done, t0 = 0, time.perf_counter()
    while done < steps:
        o.solve(1)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    g = o.grid if hasattr(o, "grid") else None
    S = len(p["D"])
    vox = int(np.prod(g)) if g else (p["bbmax"][0] // p["voxel"][0]) ** 3
    return vox * S * done / dt, done, dt, o, calls + done


def field_error(got, ref):
    """Max-relative (per substrate, normalised by max |ref| of that substrate) and
    L2-relative (||got - ref||_2 / ||ref||_2 per substrate) error, worst substrate.
    Both arrays are [..., S] (interleaved) float arrays."""
    S = ref.shape[-1]
    g = got.reshape(-1, S).astype(np.float64)
    r = ref.reshape(-1, S).astype(np.float64)
    diff = np.abs(g - r)
    norm = np.maximum(np.abs(r).max(axis=0), 1e-300)
    l2 = np.sqrt((diff ** 2).sum(axis=0)) / np.maximum(np.sqrt((r ** 2).sum(axis=0)), 1e-300)
    return float((diff.max(axis=0) / norm).max()), float(l2.max())


def run_reference(args, w):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    p = build_problem(w)
    threads = cpu_threads()
    value, done, secs, _, _ = time_reference(p, args.steps, args.warmup, threads,
                                             budget_s=float(os.environ.get("PCG_REF_BUDGET_S", "90")))
    sample = (f"{done} timed steps (after {args.warmup} warm-up) of the {args.steps}-step request, "
              f"{secs:.1f} s, OpenMP over {threads} threads")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": done, "warmup": args.warmup, "ms_per_step": 1e3 * secs / max(done, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded PCG64)",
            "config": workload_config(w, mass_check=False),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(_finite(line), allow_nan=False), flush=True)


def kernel_table(stats, steps=None):
    """Per-kernel launches, time, share and achieved GB/s from kernel stats."""
    timed = {k: v for k, v in stats.items() if v["launches"] and v["ms"] > 0}
    total = sum(v["ms"] for v in timed.values()) or 1.0
    return {k: {"launches": v["launches"], "us_per_launch": round(1e3 * v["ms"] / v["launches"], 2),
                "share": round(v["ms"] / total, 4),
                "gbps": round(v["bytes"] / (v["ms"] / 1e3) / 1e9, 1)} for k, v in timed.items()}


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

    det = Details(args.detail_out if rank == 0 else None)
    prev_cpus = bind_near_gpu(local)
    mass_on = args.mass_check == "on"
    p = build_problem(w)
    from physicore_gb300 import workloads as W
    s = W.apply(pcg.Solver(pcg.FP32, device=local), p)
    n, S = w["n"], w["S"]
    vss_step = n ** 3 * S
    s.set_mass_check(mass_on)
    s.solve(1)  # first call: ballots rebuilt
    for _ in range(max(0, args.warmup - 1)):
        s.solve(1)
    s.synchronize()
    if mass_on:
        s.set_mass_check(True)  # the residual record restarts with the timed steps

    stream = torch.cuda.ExternalStream(s.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
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
    ms = max_over_ranks(ms, world)
    value = job_rate(vss_step * args.steps, world, ms / 1e3)
    chk = s.get_mass_check() if mass_on else None

    # per-kernel device times: the same steps again with an event pair around every
    # launch (kept out of the timed region above)
    s.set_kernel_timing(True)
    s.reset_kernel_stats()
    kt_steps = max(3, min(args.steps, 50))
    for _ in range(kt_steps):
        s.solve(1)
    s.synchronize()
    stats = s.kernel_stats()
    s.set_kernel_timing(False)
    peak, peak_src = measured_peaks()
    timed = {k: v for k, v in stats.items() if v["launches"] and v["ms"] > 0}
    dom = max(timed, key=lambda k: timed[k]["ms"])
    d = timed[dom]
    per_launch_bytes = d["bytes"] / d["launches"]
    achieved = per_launch_bytes / (d["ms"] / d["launches"] / 1e3) / 1e9
    step_bytes = sum(v["bytes"] for v in stats.values()) / kt_steps
    step_gbs = step_bytes / (ms / args.steps / 1e3) / 1e9
    kernels = kernel_table(stats)
    det.add("kernels_large", {"steps": kt_steps, "kernels": kernels, "algorithmic_bytes_per_step": step_bytes})

    # the step with the mass check off, for its overhead
    s.set_mass_check(False)
    s.solve(1)
    s.synchronize()
    ev0.record(stream)
    for _ in range(kt_steps):
        s.solve(1)
    ev1.record(stream)
    ev1.synchronize()
    ms_off = ev0.elapsed_time(ev1) / kt_steps
    mass_check = {"on_in_headline": mass_on, "ms_per_step_off": round(ms_off, 4),
                  "overhead": round((ms / args.steps) / ms_off - 1.0, 4) if mass_on else None,
                  "worst_residual": float(chk["worst"].max()) if chk else None,
                  "steps_checked": chk["steps"] if chk else 0,
                  "residual": "max over substrates and steps of |after*f - before|/|before|, f the product of "
                              "the sweep matrices' column sums"}
    det.add("mass_check", mass_check)

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
    s.set_mass_check(mass_on)

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
           "ms_per_step": round(1e3 * e2e_s / e2e_steps, 3)}
    det.add("e2e", dict(e2e, path="pcg_update_agents(pinned) -> pcg_recompute_positional_data -> pcg_solve(1) -> "
                                  "pcg_get_field_async(pinned, planar f32), waited one step later (every step's "
                                  "field reaches host memory inside the timed region)"))
    s.close()
    del fields, pos_h, act_h

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    e2e["host_cpus"] = len(os.sched_getaffinity(0))
    head = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded PCG64)",
            "config": dict(workload_config(w, mass_on), parallelism=f"replicas x{world}"),
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": ncu_traffic(dom),
                         "algorithmic_bytes_per_launch": per_launch_bytes, "peak_source": peak_src},
            "step_roofline": {"achieved": round(step_gbs, 1), "frac": round(step_gbs / peak, 4),
                              "algorithmic_bytes_per_step": round(step_bytes)},
            "gpu_launches": int(launches), "clocks": clk.summary(), "e2e": e2e,
            "mass_check": {k: mass_check[k] for k in ("on_in_headline", "overhead", "worst_residual")}}

    # CPU baseline (the oracle on the host's cores, a bounded sample) and the FP32
    # field's error against that FP64 run after the same solve calls
    if prev_cpus:
        os.sched_setaffinity(0, prev_cpus)
    if world == 1 and not args.no_cpu_baseline:
        threads = cpu_threads()
        v, done, secs, o, calls = time_reference(p, args.cpu_steps, 1, threads, budget_s=30.0)
        head["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{done} steps of large_{n} (after 1 warm-up) on the oracle (FP64 "
                                          f"OpenMP restatement), {secs:.1f} s"}
        g = W.apply(pcg.Solver(pcg.FP32, device=local), p)
        for _ in range(calls):
            g.solve(1)
        mr, l2 = field_error(g.get_field(), o.get_field())
        counts_ok = bool(np.array_equal(g.get_counts().reshape(-1), o.get_counts().reshape(-1)))
        g.close()
        del o
        head["error_vs_fp64"] = {"max_rel": mr, "l2_rel": l2, "steps": calls, "counts_bit_exact": counts_ok,
                                 "tolerance": FP32_RTOL,
                                 "normaliser": "per substrate: max |oracle| (max_rel), ||oracle||_2 (l2_rel)"}
        det.add("error_vs_fp64", head["error_vs_fp64"])
    else:
        head["cpu_baseline"] = None

    if args.error_steps > 0:
        head["error_vs_fp64_long"] = run_error_long(args, w, p, local, det)
    del p
    if args.fp64:
        head["fp64"] = run_fp64(args, w, local, det)
        head["plain_100_fp64"] = run_plain_100(args, local, det)
        head["s1_sweeps"] = run_s1(args, local, det)
    if args.batch_domains > 0:
        b = run_batched(args, local, ClockSampler)
        det.add("batched", b)
        head["batched"] = {"speedup": r4(b["speedup"]), "value": b["batched"]["value"],
                           "plain_value": b["plain"]["value"], "frac": b["roofline"]["frac"],
                           "max_rel_vs_plain": b["parity"]["max_rel_vs_plain"]}
    if args.serve_duration > 0:
        sv = run_serve(args, local)
        det.add("serve", sv)
        head["serve"] = {"value": sv["value"], "speedup_vs_plain": r4(sv["speedup_vs_plain"]),
                         "p50_s": r4(sv["time_to_result_s"]["p50"]), "p99_s": r4(sv["time_to_result_s"]["p99"]),
                         "offered": sv["offered_vss_per_s"], "arrivals_s": args.serve_duration,
                         "requests": sv["requests"]}
    if args.dense_steps > 0:
        dn = run_dense(args, local)
        det.add("dense", dn)
        head["dense"] = {"ms_per_step_agents_fixed": r4(dn["agents_fixed"]["ms_per_step"]),
                         "ms_per_step_ballot_rebuilt": r4(dn["ballot_rebuilt_every_step"]["ms_per_step"]),
                         "counts_bit_exact": dn.get("counts_bit_exact")}
    head["kernels_us"] = {k: v["us_per_launch"] for k, v in kernels.items()}
    head["detail"] = "stderr (one JSON line per leg)" + (f" and {args.detail_out}" if args.detail_out else "")
    det.write()
    line = json.dumps(_finite(head), allow_nan=False, separators=(",", ":"))
    print(line, flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_error_long(args, w, p, local, det):
    """The FP32 field after `--error-steps` solve calls against the oracle's FP64
    run of the same calls (the full-length error of the headline workload)."""
    import physicore_gb300 as pcg
    from oracle import oracle
    from physicore_gb300 import workloads as W
    steps = args.error_steps
    g = W.apply(pcg.Solver(pcg.FP32), p)
    o = W.apply(oracle.OracleSolver(threads=cpu_threads()), p)
    t0 = time.perf_counter()
    checkpoints = sorted({c for c in (1, 10, 100, 300, steps) if c <= steps})
    rows, done = [], 0
    for c in checkpoints:
        g.solve(c - done)
        o.solve(c - done)
        done = c
        fg, fo = g.get_field(), o.get_field()
        mr, l2 = field_error(fg, fo)
        Sx = fo.shape[-1]
        dd = np.abs(fg.reshape(-1, Sx) - fo.reshape(-1, Sx))
        per_s = (dd.max(axis=0) / np.abs(fo.reshape(-1, Sx)).max(axis=0)).tolist()
        mass_rel = (np.abs(fg.reshape(-1, Sx).sum(axis=0) - fo.reshape(-1, Sx).sum(axis=0))
                    / np.abs(fo.reshape(-1, Sx).sum(axis=0))).tolist()
        rows.append({"steps": c, "max_rel": mr, "l2_rel": l2, "max_rel_by_substrate": [r4(v) for v in per_s],
                     "mass_rel_by_substrate": [r4(v) for v in mass_rel]})
    out = {"steps": steps, "max_rel": rows[-1]["max_rel"], "l2_rel": rows[-1]["l2_rel"],
           "counts_bit_exact": bool(np.array_equal(g.get_counts().reshape(-1), o.get_counts().reshape(-1))),
           "by_steps": rows, "oracle_s": round(time.perf_counter() - t0, 1), "tolerance": FP32_RTOL}
    g.close()
    det.add("error_vs_fp64_long", out)
    return {k: out[k] for k in ("steps", "max_rel", "l2_rel", "counts_bit_exact")}


def run_fp64(args, w, local, det):
    """The headline workload with an FP64 field (the reference's arithmetic type)."""
    import torch

    import physicore_gb300 as pcg
    from physicore_gb300 import workloads as W
    p = W.large(seed=w["seed"], n=w["n"], S=w["S"], agents=w["agents"], interior=w["interior"],
                field_dtype=np.float64)
    s = W.apply(pcg.Solver(pcg.FP64, device=local), p)
    del p
    vss = s.voxels * s.S
    for _ in range(3):
        s.solve(1)
    s.synchronize()
    st = torch.cuda.ExternalStream(s.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k = max(3, min(args.steps, 30))
    ev0.record(st)
    for _ in range(k):
        s.solve(1)
    ev1.record(st)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1) / k
    s.set_kernel_timing(True)
    s.reset_kernel_stats()
    for _ in range(5):
        s.solve(1)
    s.synchronize()
    stats = s.kernel_stats()
    s.close()
    peak, _ = measured_peaks()
    step_bytes = sum(v["bytes"] for v in stats.values()) / 5
    gbs = step_bytes / (ms / 1e3) / 1e9
    out = {"value": vss / (ms / 1e3), "ms_per_step": round(ms, 4), "step_gbps": round(gbs, 1),
           "frac": round(gbs / peak, 4), "steps": k}
    det.add("fp64_large", dict(out, kernels=kernel_table(stats)))
    return out


def run_s1(args, local, det):
    """One substrate at 320^3 in FP32 (x sweep on its row-per-thread path, y/z tiles
    of 32 voxels): per-kernel device times and achieved bandwidth."""
    import physicore_gb300 as pcg
    from physicore_gb300 import workloads as W
    p = W.large(seed=5, n=args.n, S=1, agents=0, interior=0)
    p["agents"] = None
    s = W.apply(pcg.Solver(pcg.FP32, device=local), p)
    del p
    for _ in range(3):
        s.solve(1)
    s.synchronize()
    s.set_kernel_timing(True)
    s.reset_kernel_stats()
    steps = max(3, min(args.steps, 30))
    for _ in range(steps):
        s.solve(1)
    s.synchronize()
    kt = kernel_table(s.kernel_stats())
    s.close()
    peak, _ = measured_peaks()
    out = {k: {"us": v["us_per_launch"], "gbps": v["gbps"], "frac": round(v["gbps"] / peak, 4)}
           for k, v in kt.items() if k.startswith("sweep")}
    det.add("s1_320", {"workload": f"{args.n}^3 x 1 substrate FP32, x faces Dirichlet, no agents", "kernels": kt})
    return out


def run_plain_100(args, local, det):
    """The plain single-domain workload (100^3 x 1 substrate, FP64, 1,000 agents,
    all six faces Dirichlet, 100 steps) on the GPU, against the oracle's field."""
    import torch

    import physicore_gb300 as pcg
    from oracle import oracle
    from physicore_gb300 import workloads as W
    p = W.plain_100()
    s = W.apply(pcg.Solver(pcg.FP64, device=local), p)
    st = torch.cuda.ExternalStream(s.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = 100
    ev0.record(st)
    s.solve(steps)
    ev1.record(st)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1)
    o = W.apply(oracle.OracleSolver(threads=cpu_threads()), p)
    t0 = time.perf_counter()
    o.solve(steps)
    cpu_s = time.perf_counter() - t0
    mr, l2 = field_error(s.get_field(), o.get_field())
    counts_ok = bool(np.array_equal(s.get_counts().reshape(-1), o.get_counts().reshape(-1)))
    s.set_kernel_timing(True)
    s.reset_kernel_stats()
    s.solve(10)
    s.synchronize()
    kt = kernel_table(s.kernel_stats())
    vss = s.voxels * s.S * steps
    s.close()
    out = {"value": vss / (ms / 1e3), "ms_per_step": round(ms / steps, 4), "steps": steps, "max_rel": mr,
           "l2_rel": l2, "counts_bit_exact": counts_ok, "tolerance": FP64_RTOL,
           "cpu_value": vss / cpu_s, "cpu_cores": cpu_threads()}
    det.add("plain_100_fp64", dict(out, kernels=kt,
                                   note="field 8 MB: L2-resident, so this step is latency-bound, not HBM-bound"))
    return out


def run_batched(args, local, clock_sampler=None):
    """The batched workload (256 uneven domains, FP32).  Two identical sets of
    contexts: one stepped one domain after another on one stream (the plain path:
    pcg_solve per domain), the other together through a batch (one launch per
    phase, CUDA-graph replay, autotuned).  After the same number of steps every
    domain's batched field is compared with its plain field."""
    import torch

    import physicore_gb300 as pcg
    from physicore_gb300 import workloads as W
    t0 = time.perf_counter()
    plain, batched = [], []
    for p in W.batched_uneven(count=args.batch_domains):
        plain.append(W.apply(pcg.Solver(pcg.FP32, device=local), p))
        batched.append(W.apply(pcg.Solver(pcg.FP32, device=local), p))
    setup_s = time.perf_counter() - t0
    vss_step = sum(s.voxels * s.S for s in plain)
    steps, warm = args.batch_steps, max(3, args.warmup)

    # one stream owned here (it must outlive every context that uses it)
    cs = torch.cuda.Stream()
    for s in plain:
        s.set_stream(cs.cuda_stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(warm):
        for s in plain:
            s.solve(1)
    plain[0].synchronize()
    l0 = sum(s.launch_count() for s in plain)
    ev0.record(cs)
    for _ in range(steps):
        for s in plain:
            s.solve(1)
    ev1.record(cs)
    ev1.synchronize()
    plain_ms = ev0.elapsed_time(ev1)
    plain_launches = sum(s.launch_count() for s in plain) - l0

    b = pcg.Batch(batched)
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

    # parity: both sets have taken warm + steps steps
    worst, worst_dom, counts_ok, worst_fields = 0.0, -1, True, None
    for k, (sp, sb) in enumerate(zip(plain, batched)):
        fp = sp.get_field(dtype=np.float32)
        fb = sb.get_field(dtype=np.float32)
        e, _ = field_error(fb, fp)
        if e > worst:
            worst, worst_dom, worst_fields = e, k, (fp, fb)
        counts_ok &= bool(np.array_equal(sp.get_counts(), sb.get_counts()))
    # the most different domain, both paths against the FP64 oracle after the same steps
    vs_oracle = None
    if worst_dom >= 0:
        from oracle import oracle
        import itertools
        p_w = next(itertools.islice(W.batched_uneven(count=worst_dom + 1), worst_dom, None))
        o = W.apply(oracle.OracleSolver(threads=cpu_threads()), p_w)
        for _ in range(warm + steps):
            o.solve(1)
        fo = o.get_field()
        vs_oracle = {"plain": field_error(worst_fields[0], fo), "batched": field_error(worst_fields[1], fo)}
        vs_oracle = {k: {"max_rel": v[0], "l2_rel": v[1]} for k, v in vs_oracle.items()}

    # per-kernel times from a short run of direct (event-timed) launches
    b.set_kernel_timing(True)
    b.reset_kernel_stats()
    kt = min(steps, 20)
    b.solve(kt)
    b.synchronize()
    stats = b.kernel_stats()
    b.set_kernel_timing(False)
    # algorithmic bytes per step from the timed launches (these count the agents of
    # shared voxels, known only on the device)
    step_bytes = sum(v["bytes"] for v in stats.values()) / kt
    peak, peak_src = measured_peaks()
    timed = {k: v for k, v in stats.items() if v["launches"] and v["ms"] > 0}
    kernels = kernel_table(stats)
    dom = max(timed, key=lambda k: timed[k]["ms"])
    dgb = timed[dom]["bytes"] / (timed[dom]["ms"] / 1e3) / 1e9
    tuned = b.describe()
    b.close()
    for s in plain + batched:
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
           "parity": {"max_rel_vs_plain": worst, "worst_domain": worst_dom, "counts_equal": counts_ok,
                      "worst_domain_vs_fp64_oracle": vs_oracle,
                      "steps": warm + steps, "tolerance": FP32_RTOL,
                      "normaliser": "per domain and substrate: max |plain field|"},
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
    aggregate VSS/s, with the offered and served rates and the queue every half
    second."""
    import torch

    import physicore_gb300 as pcg
    from physicore_gb300 import workloads as W
    stream = W.ServedStream(duration=args.serve_duration)
    n = len(stream)
    # a bounded queue sheds load under sustained overload (refused requests come
    # back at once); 0 keeps the server's default (2^20)
    srv = pcg.Server(pcg.FP32, device=local, steps_per_tick=args.serve_tick, reserve_bytes=1 << 30,
                     max_queue=args.serve_max_queue)
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
    lat_by_req = {}
    vss_admitted = [0]
    t_first = t_last = None
    got = 0
    profile, next_sample = [], 0.5  # [t, active, queued, cumulative vss, submitted] every half second
    while got < n and not err:
        if time.perf_counter() - t_start >= next_sample:
            sp = srv.stats()
            profile.append([round(time.perf_counter() - t_start, 2), sp["active"], sp["queued"], sp["vss"],
                            sp["submitted"]])
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
                vss_admitted[0] += stream.vss(i)
                lat_host.append(time.perf_counter() - submit_wall[i])
                lat_dev.append(r["t_done"] - r["t_submit"])
                lat_by_req[i] = r["t_done"] - r["t_submit"]
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
    # latency percentiles by arrival window: is the tail bounded over the run?
    win = max(1.0, min(60.0, args.serve_duration / 10))
    windows = []
    for k in range(int(math.ceil(args.serve_duration / win))):
        lat = [v for i, v in lat_by_req.items() if k * win <= stream.arrivals[i] < (k + 1) * win]
        if lat:
            windows.append([round(k * win, 1), len(lat), r4(q(lat, 50)), r4(q(lat, 99))])
    served = vss_done / (t_last - t_first) if t_last else None
    return {"workload": f"served: Poisson arrivals at 200/s for {args.serve_duration:g} s ({n} requests), sides "
                        "log-uniform [32,256] per axis, 1-8 substrates, 0-200,000 agents, steps log-uniform "
                        "[10,1000], FP32",
            "requests": n, "statuses": statuses, "offered_vss_per_s": offered,
            "max_queue": args.serve_max_queue or None,
            "completed_vss_per_arrival_s": vss_admitted[0] / args.serve_duration,
            "value": served, "unit": UNIT,
            "agent_steps_per_s": agent_steps / (t_last - t_first) if t_last else None,
            "plain": {"value": vss_plain / plain_s, "requests": len(sample),
                      "path": "the same requests (an even sample) one after another: pcg_create, pcg_solve(steps), "
                              "pcg_get_field, pcg_destroy"},
            "speedup_vs_plain": served / (vss_plain / plain_s) if t_last else None,
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
            "latency_by_arrival_window": {"columns": ["window_start_s", "requests", "p50_s", "p99_s"],
                                          "rows": windows},
            "profile": {"columns": ["t_s", "active", "queued", "vss_per_s_over_the_half_second", "submitted"],
                        "rows": [[t, a, qd, (v - profile[k - 1][3]) / (t - profile[k - 1][0]) if k else v / t, sb]
                                 for k, (t, a, qd, v, sb) in enumerate(profile)]}}


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
    # the per-voxel agent counts against numpy's FP64 voxel positions (the oracle's rule)
    pos = p["agents"]["positions"]
    idx = np.floor((pos - 0.0) / 20.0).astype(np.int64)  # positions are >= 0: trunc == floor
    n = s.grid[0]
    ref = np.bincount(idx[:, 0] + n * (idx[:, 1] + n * idx[:, 2]), minlength=n ** 3)
    counts_ok = bool(np.array_equal(counts.reshape(-1), ref))

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
        return kernel_table(st)

    vss = s.voxels * s.S
    A = int(p["agents"]["volumes"].size)
    ms_fixed = timed(steps, False)
    ms_moving = timed(max(10, steps // 5), True)
    out = {"workload": "dense_200: 200^3 voxels x 4 substrates FP32, 4,000,000 agents N(centre, 200 um) "
                       "(internalized tracking on)", "vss_per_step": vss, "agents": A,
           "max_agents_per_voxel": int(counts.max()), "occupied_voxels": int((counts > 0).sum()),
           "counts_bit_exact": counts_ok, "steps": steps,
           "agents_fixed": {"ms_per_step": ms_fixed, "value": vss / (ms_fixed / 1e3), "unit": UNIT,
                            "agent_steps_per_s": A / (ms_fixed / 1e3), "kernels": kernels(10, False)},
           "ballot_rebuilt_every_step": {"ms_per_step": ms_moving, "value": vss / (ms_moving / 1e3), "unit": UNIT,
                                         "agent_steps_per_s": A / (ms_moving / 1e3),
                                         "kernels": kernels(10, True)}}
    s.set_stream(None)
    s.close()
    return out


def run_served_batch(args, local):
    """A steady batch of the served mix: the first N requests of the served stream
    (workloads.ServedStream), initialised and stepped together with every request
    taking part in every step.  About the server's active set at its 1,024-request
    cap for N = 990; it explains the served rate apart from admissions, ticks and
    readbacks.  With --served-batch-direct the steps are launched directly instead
    of replayed from a graph (so that a profiler sees each kernel)."""
    import torch

    import physicore_gb300 as pcg
    from physicore_gb300 import workloads as W
    N = args.only_served_batch
    stream = W.ServedStream(duration=600)
    t0 = time.perf_counter()
    sol = []
    for i in range(N):
        s = stream.request(pcg.Solver(pcg.FP32, device=local), i)
        s.initialize()
        sol.append(s)
    setup_s = time.perf_counter() - t0
    vss = sum(int(np.prod(stream.sides[i])) * int(stream.S[i]) for i in range(N))
    b = pcg.Batch(sol)
    b.set_graph(not args.served_batch_direct)
    b.solve(max(3, args.warmup))
    b.synchronize()
    bs = torch.cuda.ExternalStream(b.stream())
    steps = args.served_batch_steps
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(bs)
    b.solve(steps)
    ev1.record(bs)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    b.set_kernel_timing(True)
    b.reset_kernel_stats()
    b.solve(min(steps, 8))
    b.synchronize()
    kt = kernel_table(b.kernel_stats())
    b.set_kernel_timing(False)
    b.close()
    for s in sol:
        s.close()
    return {"workload": f"the first {N} requests of the served stream (sides log-uniform [32,256] per axis, "
                        "1-8 substrates, 0-200,000 agents, FP32), every one stepping",
            "requests": N, "vss_per_step": vss, "agents": int(sum(int(a) for a in stream.A[:N])),
            "steps": steps, "ms_per_step": ms, "value": vss / (ms / 1e3), "unit": UNIT,
            "graph": not args.served_batch_direct, "setup_s": round(setup_s, 1), "kernels": kt}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--detail-out", default=None, help="write every leg's full record to this JSON file")
    ap.add_argument("--mass-check", choices=["on", "off"], default="on",
                    help="per-step FP64 mass check in the headline step")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--error-steps", type=int, default=0,
                    help="also compare the FP32 field with the oracle after this many steps (e.g. 1000)")
    ap.add_argument("--no-fp64", dest="fp64", action="store_false", help="skip the FP64 sub-figures")
    ap.add_argument("--n", type=int, default=WORKLOAD["n"], help="grid side (default: the 320^3 workload)")
    ap.add_argument("--batch-domains", type=int, default=256, help="domains of the batched workload (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=200)
    ap.add_argument("--no-batch-autotune", action="store_true", help="keep the default line mappings")
    ap.add_argument("--only-batched", action="store_true", help="run only the batched workload")
    ap.add_argument("--serve-duration", type=float, default=10.0, help="seconds of request arrivals (0: skip)")
    ap.add_argument("--serve-tick", type=int, default=8, help="steps between admission points")
    ap.add_argument("--only-serve", action="store_true", help="run only the served request stream")
    ap.add_argument("--serve-plain-sample", type=int, default=100, help="requests timed one after another")
    ap.add_argument("--serve-max-queue", type=int, default=0,
                    help="queued requests beyond which submissions are refused (0: no practical limit)")
    ap.add_argument("--dense-steps", type=int, default=100, help="steps of the dense-agent workload (0: skip)")
    ap.add_argument("--only-dense", action="store_true", help="run only the dense-agent workload")
    ap.add_argument("--only-served-batch", type=int, default=0,
                    help="run only a steady batch of the first N requests of the served stream")
    ap.add_argument("--served-batch-steps", type=int, default=16)
    ap.add_argument("--served-batch-direct", action="store_true", help="direct launches instead of a graph")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    w = dict(WORKLOAD, n=args.n)
    if args.impl == "reference":
        run_reference(args, w)
        return
    only = [(args.only_serve, "serve", run_serve), (args.only_dense, "dense", run_dense),
            (args.only_batched, "batched", lambda a, l: run_batched(a, l, ClockSampler)),
            (args.only_served_batch > 0, "served_batch", run_served_batch)]
    for flag, name, fn in only:
        if flag:
            import torch
            torch.cuda.set_device(dist_env()[2])
            det = Details(args.detail_out)
            det.add(name, fn(args, dist_env()[2]))
            det.write()
            return
    run_gb300(args, w)


if __name__ == "__main__":
    main()
