#!/usr/bin/env python
"""Benchmark of the shallow-water hot path on GB300 (one JSON line on rank 0).

A step is one SSP-RK3 step (three fused stage kernels) of the whole grid.  The
workload is the 8192^2 FP64 drop-in case: a seeded sum of 16 Gaussians as
bathymetry (centres U[0,1]^2, widths U[0.02,0.1], amplitudes U[-0.3,0.3]), a dam
break in the free surface (eta = 1.5 for x < 0.4, else 1), u = v = 0, transmissive
walls, adaptive CFL dt (0.45) reduced on the device every step.  All inputs are
synthetic and generated on the host.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun (N > 1) every rank advances its own grid on its own GPU (replicas:
the path has a real halo exchange only when one grid is split, which this build
does not do on one-GPU machines); value = all ranks' cell updates / max-over-ranks time.
``--impl reference`` times the reference algorithm on the host cores instead (the
CPU restatement of HPC_solver/omp_solver in oracle/, all host threads), rank 0 only.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GCUPS & % HBM roofline: FP32-mixed vs FP64 at stated L1 error; adjoint/forward"
BYTES_PER_CELL_FP64 = 216  # algorithmic bytes per cell-update: 56 + 80 + 80 (stages 1-3)
# dram bytes per stage launch per interior cell from the committed ncu capture
# (profiles/stage_f64_ncu.md); None until measured.
NCU_TRAFFIC_BYTES_PER_CELL_LAUNCH = None


def parse():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--n", type=int, default=8192, help="grid side (default 8192)")
    ap.add_argument("--e2e-steps", type=int, default=4)
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="target CPU work of the cpu_baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--seed", type=int, default=2026)
    return ap.parse_args()


class Dist:
    """Rank bookkeeping; under torchrun a gloo group gives barrier and max-reduce on the
    host (timing only, no data path)."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def workload(n: int, seed: int):
    P = importlib.import_module("shallow-water_gb300.problems")
    B, _ = P.gaussian_sum_bathymetry(n, n, n=16, seed=seed, bc="transmissive")
    h, hu, hv = P.dam_break(B)
    return h, hu, hv, B


def config(n, form="fp64_dropin"):
    return {
        "workload": f"{n}x{n} dam break over seeded 16-Gaussian bathymetry, transmissive "
                    "walls, adaptive CFL dt 0.45, MUSCL+hydrostatic+HLL+SSP-RK3",
        "grid": [n, n], "form": form, "bc": "transmissive", "dt": "adaptive (cfl 0.45)",
        "l2": "inputs larger than L2 (each step streams ~3.7 GB of state vs 129 MB L2)",
        "parallelism": "replicas (one grid per GPU)",
    }


class ClockSampler:
    """nvidia-smi samples (200 ms) of one GPU during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sms, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sms:
            return None
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sms)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return float(m["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def time_cpu_port(h, hu, hv, B, n, steps, warmup):
    """Times the CPU restatement of the reference (all host threads) on in-place copies."""
    from oracle import port
    p = port.grid(n, n, 1.0, 1.0, cfl=0.45, bc=port.BC_TRANSMISSIVE, threads=0)
    a = [np.array(x, copy=True) for x in (h, hu, hv)]
    ws = port.Workspace(p)
    if warmup:
        ws.run_inplace(a[0], a[1], a[2], B, warmup)
    t0 = time.perf_counter()
    _, _, st = ws.run_inplace(a[0], a[1], a[2], B, steps)
    dt = time.perf_counter() - t0
    ws.close()
    if st != 0:
        raise RuntimeError("CPU oracle reported a non-finite state")
    return dt


def run_reference(args, dist: Dist):
    if dist.rank != 0:
        return
    n = args.n
    h, hu, hv, B = workload(n, args.seed)
    secs = time_cpu_port(h, hu, hv, B, n, args.steps, args.warmup)
    value = n * n * args.steps / secs / 1e9
    cores = cpu_threads()
    line = {
        "metric": METRIC, "value": value, "unit": "GCUPS", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config(n, "reference_cpu"), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "GCUPS", "cores": cores, "kind": "port",
                         "sample": f"{n}^2 workload, {args.steps} full RK3 steps after "
                                   f"{args.warmup} warm-up steps, C restatement of "
                                   "HPC_solver/omp_solver (oracle/swe_oracle.c), OpenMP"},
        "e2e": {"value": value, "unit": "GCUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gb300(args, dist: Dist):
    sw = importlib.import_module("shallow-water_gb300")
    import torch

    n, K, W = args.n, args.steps, args.warmup
    dev = dist.local
    torch.cuda.set_device(dev)
    h, hu, hv, B = workload(n, args.seed + dist.rank)
    solver = sw.Solver(n, n, 1.0, 1.0, cfl=0.45, bc="transmissive", device=dev)
    solver.upload(h, hu, hv, B)
    if W:
        solver.step(W)

    launches0 = solver.kernel_launches()
    clocks = ClockSampler(dev)
    dist.barrier()
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    solver.step(K)  # synchronous; device time from events on the library's stream
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    dist.barrier()
    clk = clocks.stop()
    launches = solver.kernel_launches() - launches0
    dev_ms = solver.last_step_ms()
    ms = dist.max(dev_ms)
    cells = float(n) * n
    value = cells * K * dist.world / (ms / 1e3) / 1e9

    # End to end through the public API with pinned host buffers: per step, upload the
    # state and bathymetry, advance one RK3 step, download the state.
    nt = (n + 4) * (n + 4)
    pin = [torch.empty((n + 4, n + 4), dtype=torch.float64, pin_memory=True).numpy()
           for _ in range(7)]
    for dst, src in zip(pin[:4], (h, hu, hv, B)):
        np.copyto(dst, src)
    E = max(1, args.e2e_steps)
    solver.upload(pin[0], pin[1], pin[2], pin[3])
    solver.step(1)
    solver.download(tuple(pin[4:7]))
    dist.barrier()
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    for _ in range(E):
        solver.upload(pin[0], pin[1], pin[2], pin[3])
        solver.step(1)
        solver.download(tuple(pin[4:7]))
    torch.cuda.synchronize()
    e_secs = dist.max(time.perf_counter() - e0)
    e2e = {"value": cells * E * dist.world / e_secs / 1e9, "unit": "GCUPS",
           "h2d_bytes_per_step": 4 * nt * 8, "d2h_bytes_per_step": 3 * nt * 8,
           "steps": E, "api": "swe_upload + swe_step(1) + swe_download, pinned host buffers"}
    solver.close()

    peak, peak_kind = peaks()
    # Every launch in the timed region is a stage kernel: average launch = ms / (3K).
    launch_ms = ms / (3 * K)
    algo_bytes_launch = BYTES_PER_CELL_FP64 / 3.0 * cells
    achieved = algo_bytes_launch / (launch_ms / 1e3) / 1e9
    traffic = (NCU_TRAFFIC_BYTES_PER_CELL_LAUNCH * cells
               if NCU_TRAFFIC_BYTES_PER_CELL_LAUNCH else None)
    line = {
        "metric": METRIC, "value": value, "unit": "GCUPS", "n_gpus": dist.world, "steps": K,
        "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config(n),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "kernel": "k_stage_f64 (3 launches per step)",
                     "algorithmic_bytes_per_launch": algo_bytes_launch},
        "e2e": e2e,
        "gpu_launches": launches,
        "wall_ms_per_step": wall * 1e3 / K,
    }
    if clk:
        line["clocks"] = clk
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        # Bounded CPU sample: full-grid RK3 steps of the same workload; pick the count
        # from one timed step so the sample is ~cpu_seconds.
        one = time_cpu_port(h, hu, hv, B, n, 1, 0)
        s_cpu = int(max(1, min(50, args.cpu_seconds / max(one, 1e-3))))
        secs = time_cpu_port(h, hu, hv, B, n, s_cpu, 0)
        line["cpu_baseline"] = {
            "value": cells * s_cpu / secs / 1e9, "unit": "GCUPS", "cores": cpu_threads(),
            "kind": "port",
            "sample": f"{n}^2 workload from t=0, {s_cpu} full RK3 steps, C restatement of "
                      "HPC_solver/omp_solver (oracle/swe_oracle.c), OpenMP on all host threads"}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        else:
            run_gb300(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
