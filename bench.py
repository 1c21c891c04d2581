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
# DRAM bytes per stage launch per interior cell, mean of the three stages, from one
# ncu capture of this bench at 8192^2 (dram__bytes_read.sum + dram__bytes_write.sum).
NCU_TRAFFIC_BYTES_PER_CELL_LAUNCH = 71.7
# FP64 lane operations (DADD + DMUL + DFMA) per cell update, three stages, from the
# ncu thread-level instruction counts of the stage kernel as it runs (strips of 6 tiles:
# 446.8 on the FP64 pipe), plus the cell update's products (dt x L and the RK weights:
# 3 + 6 + 9 per cell update on this grid, whose 1/dx is a power of two), which run
# correctly rounded on the integer pipes and are counted as operations of the scheme.
# The pipe executes 2 per clock per SM, so its peak is 2 x SMs x clock.
FP64_OPS_PER_CELL_UPDATE = 464.8
FP64_OPS_ON_INTEGER_PIPES = 18
# The same count for lone 8x32 tiles (2.16 interfaces per cell instead of 2.05).
FP64_OPS_PER_CELL_UPDATE_LONE_TILES = 483.9
# Warp instructions per cell update (the three stages) of the FP32 kernels, from their
# ncu captures: the single grid's column sweeps (13.7 + 14.6 + 15.5) and the ensemble's
# column sweeps (14.5 + 16.5 + 16.9).  Both are bound by instruction issue (4 warp
# instructions per clock per SM) and load latency.
F32_WARP_INST_PER_CELL_UPDATE = 43.9
F32_ENS_WARP_INST_PER_CELL_UPDATE = 48.0


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
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the FP32-mixed, ensemble and adjoint measurements")
    ap.add_argument("--forms", default="fp32_mixed,ensemble,adjoint,sanity,slabs,modular",
                    help="comma list of the extra forms to measure")
    ap.add_argument("--fp32-n", type=int, default=16384)
    ap.add_argument("--ens-count", type=int, default=512)
    ap.add_argument("--ens-precisions", default="fp64,fp32_mixed")
    ap.add_argument("--ens-schedule", default="",
                    help="fixed SHAPE:GRID for every precision instead of the autotuner")
    ap.add_argument("--adj-n", type=int, default=1024)
    ap.add_argument("--adj-steps", type=int, default=200)
    ap.add_argument("--adj-fd-dirs", type=int, default=16,
                    help="random directions of the adjoint's finite-difference check (0: none)")
    ap.add_argument("--acc-n", type=int, default=16384,
                    help="grid of the FP32-mixed accuracy check (default: the timed size)")
    ap.add_argument("--acc-steps", type=int, default=100)
    ap.add_argument("--snap-steps", type=int, default=30)
    ap.add_argument("--snap-every", type=int, default=10)
    ap.add_argument("--snap-dir", default="",
                    help="directory for the snapshot form's files (default: a temporary one)")
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
        "l2": (f"no flush: each stage launch streams {BYTES_PER_CELL_FP64 / 3 * n * n / 1e9:.2f} GB "
               "(algorithmic bytes) against the 129 MB L2"
               if BYTES_PER_CELL_FP64 / 3 * n * n > 4 * 129e6 else
               "grid smaller than 4x L2: rates include L2 reuse (a parity or tuning size)"),
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


def fp64_pipe(gcups: float, dev: int):
    """The bound that limits the FP64 stage kernel on GB300: FP64-pipe operations per
    second against 2 per clock per SM at the maximum SM clock."""
    import torch
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            mhz = float(json.load(f)["sm_max_mhz"])
    except (OSError, KeyError, ValueError):
        mhz = 2070.0
    peak = 2.0 * sms * mhz * 1e6 / 1e9
    achieved = gcups * FP64_OPS_PER_CELL_UPDATE
    return {"achieved": achieved, "peak": peak, "unit": "G FP64 lane-ops/s",
            "frac": achieved / peak, "ops_per_cell_update": FP64_OPS_PER_CELL_UPDATE,
            "of_which_on_integer_pipes": FP64_OPS_ON_INTEGER_PIPES,
            "fp64_pipe_busy_frac": gcups * (FP64_OPS_PER_CELL_UPDATE - FP64_OPS_ON_INTEGER_PIPES) / peak,
            "frac_at_lone_tile_ops": gcups * FP64_OPS_PER_CELL_UPDATE_LONE_TILES / peak,
            "peak_source": f"2 x {sms} SMs x {mhz:.0f} MHz"}


def issue_roofline(gcups: float, inst_per_cell: float, dev: int = 0) -> dict:
    """The bound of the FP32 stage kernels: warp-instruction issue, 4 per clock per SM."""
    import torch
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            mhz = float(json.load(f)["sm_max_mhz"])
    except (OSError, KeyError, ValueError):
        mhz = 2070.0
    peak = 4.0 * sms * mhz * 1e6 / 1e9  # G warp instructions / s
    achieved = gcups * inst_per_cell
    return {"achieved": achieved, "peak": peak, "unit": "G warp instructions/s",
            "frac": achieved / peak, "warp_instructions_per_cell_update": inst_per_cell,
            "cap_gcups": peak / inst_per_cell, "peak_source": f"4 x {sms} SMs x {mhz:.0f} MHz"}


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def time_cpu_port(h, hu, hv, B, n, steps, warmup, threads=0):
    """Times the CPU restatement of the reference on in-place copies (threads 0: all host
    threads, as omp_solver; 1: one core, as HPC_solver)."""
    from oracle import port
    p = port.grid(n, n, 1.0, 1.0, cfl=0.45, bc=port.BC_TRANSMISSIVE, threads=threads)
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


def rel_l1(a, b):
    ai, bi = a[2:-2, 2:-2], b[2:-2, 2:-2]
    return float(np.abs(ai - bi).sum() / max(np.abs(bi).sum(), 1e-300))


def rel_linf(a, b):
    ai, bi = a[2:-2, 2:-2], b[2:-2, 2:-2]
    return float(np.abs(ai - bi).max() / max(np.abs(bi).max(), 1e-300))


def form_fp32(args, sw, fp64_gcups):
    """FP32-mixed throughput on the large grid, and its error against an FP64 GPU run of
    the same dam break on a grid small enough to run in seconds."""
    n = args.fp32_n
    h, hu, hv, B = workload(n, args.seed)
    with sw.Solver(n, n, bc="transmissive", precision="fp32_mixed") as s:
        s.upload(h, hu, hv, B)
        s.step(3)
        s.step(max(args.steps, 10))
        ms = s.last_step_ms() / max(args.steps, 10)
    del h, hu, hv, B
    gcups = n * n / (ms / 1e3) / 1e9
    out = {"grid": [n, n], "ms_per_step": ms, "gcups": gcups,
           "hbm_frac_of_measured": 108 * n * n / (ms / 1e3) / 1e9 / peaks()[0],
           "bytes_per_cell_update": 108, "speedup_vs_fp64": gcups / fp64_gcups,
           "issue_roofline": issue_roofline(gcups, F32_WARP_INST_PER_CELL_UPDATE)}
    # Accuracy against an FP64 run of the same grid (the timed size by default), each form
    # with its own adaptive dt; the mass drift of each over the run (the FP64 run's own
    # drift is the flow through the transmissive walls) and their difference at the end.
    m, K = args.acc_n, args.acc_steps
    h, hu, hv, B = workload(m, args.seed)
    with sw.Solver(m, m, bc="transmissive") as s64, \
            sw.Solver(m, m, bc="transmissive", precision="fp32_mixed") as s32:
        s64.upload(h, hu, hv, B)
        s32.upload(h, hu, hv, B)
        m64_0, m32_0 = s64.totals()[0], s32.totals()[0]
        s64.step(K)
        s32.step(K)
        m64_1, m32_1 = s64.totals()[0], s32.totals()[0]
        del h, hu, hv, B
        a, b = s64.download(), s32.download()
        out["accuracy_vs_fp64"] = {
            "grid": [m, m], "steps": K, "dt": "adaptive, each form its own",
            "l1_h": rel_l1(b[0], a[0]), "linf_h": rel_linf(b[0], a[0]),
            "l1_hu": rel_l1(b[1], a[1]), "linf_hu": rel_linf(b[1], a[1]),
            "l1_hv": rel_l1(b[2], a[2]), "linf_hv": rel_linf(b[2], a[2]),
            "t_fp64": s64.time, "t_fp32": s32.time,
            "mass_drift_fp32": (m32_1 - m32_0) / m32_0,
            "mass_drift_fp64": (m64_1 - m64_0) / m64_0,
            "mass_fp32_vs_fp64": (m32_1 - m64_1) / m64_1,
            "note": "norms relative to the FP64 field's L1 / Linf over the interior; the hv "
                    "field is driven by the bathymetry alone and is ~1e3 smaller than hu"}
        del a, b
    P = importlib.import_module("shallow-water_gb300.problems")
    Bl, _ = P.gaussian_sum_bathymetry(m, m, n=16, seed=args.seed, bc="transmissive")
    hl, hul, hvl = P.lake_at_rest(Bl, 1.0)
    with sw.Solver(m, m, bc="transmissive", precision="fp32_mixed") as s:
        s.upload(hl, hul, hvl, Bl)
        s.step(K, 0.5 * s.stable_dt())
        l = s.download()
        wet = hl[2:-2, 2:-2] > 1e-3
        out["lake_at_rest"] = {"grid": [m, m], "steps": K,
                               "max_abs_hu_hv_wet": float(max(np.abs(l[1][2:-2, 2:-2][wet]).max(),
                                                              np.abs(l[2][2:-2, 2:-2][wet]).max())),
                               "dry_cells": int((~wet).sum())}
    return out


def form_ensemble(args, sw):
    """Batched ensemble with the size and initial-condition distribution of the
    512-instance workload, `ens_count` members, tuned schedule, FP64 and FP32-mixed."""
    P = importlib.import_module("shallow-water_gb300.problems")
    specs = P.ensemble_instances(count=args.ens_count, seed=args.seed)
    sizes = [(n, n) for n, _ in specs]
    cells = float(sum(n * n for n, _ in specs))
    res = {"instances": len(specs), "cells": cells,
           "sides": sorted({n for n, _ in specs})}
    members = [P.ensemble_member(n, sd) for n, sd in specs]
    for prec in args.ens_precisions.split(","):
        with sw.Ensemble(sizes, precision=prec) as ens:
            for q, mbr in enumerate(members):
                ens.upload(q, *mbr)
            if args.ens_schedule:
                shape, grid = args.ens_schedule.split(":")
                ens.set_schedule(shape, int(grid))
                tune = {"shape": shape, "grid": int(grid)}
            else:
                tune = ens.tune(steps=1)
            steps = 3 if prec == "fp64" else 20
            ens.step(1)
            ens.step(steps)
            ms = ens.last_step_ms() / steps
            bpc = 216 if prec == "fp64" else 108
            res[prec] = {"ms_per_step": ms, "gcups": cells / (ms / 1e3) / 1e9,
                         "hbm_frac_of_measured": bpc * cells / (ms / 1e3) / 1e9 / peaks()[0],
                         "schedule": {"shape": tune["shape"], "grid": tune["grid"]},
                         "launches_per_step": 3, "graph_replay": True}
            g = res[prec]["gcups"]
            if prec == "fp64":
                res[prec]["fp64_pipe_roofline"] = fp64_pipe(g, 0)
            else:  # against the single-grid kernel's instruction count, and its own
                res[prec]["issue_roofline"] = issue_roofline(g, F32_WARP_INST_PER_CELL_UPDATE)
                res[prec]["issue_roofline_own_instructions"] = issue_roofline(
                    g, F32_ENS_WARP_INST_PER_CELL_UPDATE)
    return res


def form_adjoint(args, sw):
    """Adjoint/forward cost on the 1024^2 adjoint workload (seeded bathymetry, 8 seeded
    surface bumps, 64 gauges), fixed dt: binomial checkpointing with ~sqrt(steps) states,
    every state stored, and the tape mode (every state and stage state kept)."""
    P = importlib.import_module("shallow-water_gb300.problems")
    n, K = args.adj_n, args.adj_steps
    rng = np.random.default_rng(args.seed + 7)
    B, _ = P.gaussian_sum_bathymetry(n, n, n=16, rng=rng, bc="reflecting")
    bumps, _ = P.gaussian_sum_bathymetry(n, n, n=8, rng=rng, width=(0.02, 0.1),
                                         amp=(-0.05, 0.05), bc="reflecting")
    eta0 = 1.0 + bumps
    h = np.maximum(0.0, eta0 - B)
    z = np.zeros_like(h)
    gauges = np.stack([rng.integers(0, n, 64), rng.integers(0, n, 64)], axis=1)
    snaps = max(1, int(round(np.sqrt(K))))
    with sw.Solver(n, n) as s:
        s.upload(h, z, z, B)
        dt = 0.5 * s.stable_dt()
        # observations: the gauges of a forward run from a perturbed surface and bed
        s.upload(np.maximum(0.0, 1.0 + 1.05 * bumps - 1.02 * B), z, z, 1.02 * B)
        obs = sw.adjoint.gauge_series(s, K, dt, gauges)
        s.upload(h, z, z, B)
        s.step(K, dt)
        fwd_ms = s.last_step_ms()
        s.upload(h, z, z, B)
        r = sw.adjoint.gauge_misfit_gradient(s, K, dt, gauges, obs, snaps)
        r_all = sw.adjoint.gauge_misfit_gradient(s, K, dt, gauges, obs, K)
        r_tape = sw.adjoint.gauge_misfit_gradient(s, K, dt, gauges, obs, "tape")
        r_seg = sw.adjoint.gauge_misfit_gradient(s, K, dt, gauges, obs, "segments")
    seg_len = max(1, int(round(np.sqrt(K))))
    cells = (n + 4) * (n + 4)
    out = {"grid": [n, n], "steps": K, "gauges": 64, "snapshots": snaps,
           "forward_ms": fwd_ms, "adjoint_ms": r["ms"], "ratio": r["ms"] / fwd_ms,
           "snapshot_bytes": int(24 * (snaps + 1) * cells),
           "adjoint_ms_all_states_stored": r_all["ms"],
           "ratio_all_states_stored": r_all["ms"] / fwd_ms,
           "adjoint_ms_tape": r_tape["ms"], "ratio_tape": r_tape["ms"] / fwd_ms,
           "tape_bytes": int((75 * K + 400) * cells),
           "adjoint_ms_segments": r_seg["ms"], "ratio_segments": r_seg["ms"] / fwd_ms,
           "segment_steps": seg_len,
           "segments_bytes": int((24 * (-(-K // seg_len) + 1) + 75 * seg_len + 24) * cells),
           "schedules_bitwise_equal": all(
               x["J"] == r["J"] and all(np.array_equal(x[k], r[k]) for k in
                                        ("grad_h", "grad_hu", "grad_hv", "grad_B"))
               for x in (r_all, r_tape, r_seg))}
    # FP32-mixed: the same problem through the FP32 forward and the FP32 adjoint, and the
    # gradients' agreement with the FP64 adjoint (norm-wise, interior)
    with sw.Solver(n, n, precision="fp32_mixed") as s:
        s.upload(h, z, z, B)
        s.step(K, dt)
        fwd32 = s.last_step_ms()
        s.upload(h, z, z, B)
        q = sw.adjoint.gauge_misfit_gradient(s, K, dt, gauges, obs, snaps)
        q_tape = sw.adjoint.gauge_misfit_gradient(s, K, dt, gauges, obs, "tape")
        q_seg = sw.adjoint.gauge_misfit_gradient(s, K, dt, gauges, obs, "segments")

    # directional derivatives along smooth random directions (sums of Gaussian bumps):
    # the per-cell fields differ wherever a minmod or wave-speed branch flips between the
    # two trajectories, which on a smooth 1024^2 state is common; their projections agree
    dirs = []
    for _ in range(4):
        d = [P.gaussian_sum_bathymetry(n, n, n=4, rng=rng, width=(0.1, 0.3),
                                       amp=(-1.0, 1.0))[0] for _ in range(4)]
        dirs.append(d)

    def proj(res, d):
        return sum(float((res[k][2:-2, 2:-2] * x[2:-2, 2:-2]).sum())
                   for k, x in zip(("grad_h", "grad_hu", "grad_hv", "grad_B"), d))

    dir_rel = max(abs(proj(q, d) - proj(r, d)) / abs(proj(r, d)) for d in dirs)
    # the scale to read it against: the FP64 adjoint's own change when the initial depth
    # moves by 1e-7 (relative), the size of FP32 rounding
    with sw.Solver(n, n) as s:
        s.upload(h * (1.0 + 1e-7 * np.random.default_rng(1).standard_normal(h.shape)), z, z, B)
        r_pert = sw.adjoint.gauge_misfit_gradient(s, K, dt, gauges, obs, "tape")
    self_rel = max(abs(proj(r_pert, d) - proj(r_tape, d)) / abs(proj(r_tape, d)) for d in dirs)
    out["fp32_mixed"] = {
        "forward_ms": fwd32, "adjoint_ms": q["ms"], "ratio": q["ms"] / fwd32,
        "adjoint_ms_tape": q_tape["ms"], "ratio_tape": q_tape["ms"] / fwd32,
        "adjoint_ms_segments": q_seg["ms"], "ratio_segments": q_seg["ms"] / fwd32,
        "J_rel_diff_vs_fp64": abs(q["J"] - r["J"]) / abs(r["J"]),
        "directional_derivative_rel_diff_vs_fp64": dir_rel,
        "fp64_directional_change_under_1e-7_initial_perturbation": self_rel}
    if args.adj_fd_dirs > 0:
        out["fd_agreement"] = adjoint_fd(args, sw, P, n, K, dt, h, B, gauges, obs, r, q, rng)
        # the same check with 1e-3 noise in the initial surface and the bed (a fresh
        # adjoint), which removes the flat regions whose rounding-level slopes and bed
        # differences put kinks of minmod and max(b-, b+) at the evaluation point itself
        rn = np.random.default_rng(args.seed + 11)
        Bn = B + 1e-3 * rn.standard_normal(B.shape)
        P.fill_scalar_ghosts(Bn, "reflecting")
        hn = np.maximum(0.0, eta0 + 1e-3 * rn.standard_normal(B.shape) - Bn)
        with sw.Solver(n, n) as s:
            s.upload(hn, z, z, Bn)
            rr = sw.adjoint.gauge_misfit_gradient(s, K, dt, gauges, obs, "tape")
        out["fd_agreement_noise_1e-3"] = adjoint_fd(args, sw, P, n, K, dt, hn, Bn, gauges, obs,
                                                    rr, None, rng)
    return out


def adjoint_fd(args, sw, P, n, K, dt, h, B, gauges, obs, r64, r32, rng, eps=1e-6):
    """Central finite differences of J (the FP64 forward, bitwise the reference
    solver's) along random smooth directions in the initial depth and the bed, against
    the adjoints' directional derivatives: relative to |FD|, and to the sum of the
    absolute terms of the projection (the scale of the cancellation in it)."""
    z = np.zeros_like(h)
    fds, a64, a32, scale = [], [], [], []
    with sw.Solver(n, n) as s:
        for _ in range(args.adj_fd_dirs):
            dh = P.gaussian_sum_bathymetry(n, n, n=4, rng=rng, width=(0.1, 0.3), amp=(-1.0, 1.0))[0]
            dB = P.gaussian_sum_bathymetry(n, n, n=4, rng=rng, width=(0.1, 0.3), amp=(-1.0, 1.0),
                                           bc="reflecting")[0]
            dh = np.where(h > 0, dh, 0.0)  # wet cells only: h0 = max(0, eta0 - B)
            J = []
            for sg in (1.0, -1.0):
                s.upload(h + sg * eps * dh, z, z, B + sg * eps * dB)
                J.append(sw.adjoint.gauge_misfit(s, K, dt, gauges, obs)[0])
            fds.append((J[0] - J[1]) / (2 * eps))
            a64.append(float((r64["grad_h"] * dh).sum() + (r64["grad_B"] * dB).sum()))
            scale.append(float(np.abs(r64["grad_h"] * dh).sum() + np.abs(r64["grad_B"] * dB).sum()))
            if r32 is not None:
                a32.append(float((r32["grad_h"] * dh).sum() + (r32["grad_B"] * dB).sum()))
    fds = np.array(fds)
    rel = np.abs(np.array(a64) - fds) / np.abs(fds)
    rel_s = np.abs(np.array(a64) - fds) / np.array(scale)
    res = {"eps": eps, "directions": args.adj_fd_dirs, "grid": n, "steps": K,
           "median": float(np.median(rel)), "max": float(rel.max()),
           "median_vs_abs_terms": float(np.median(rel_s)), "max_vs_abs_terms": float(rel_s.max()),
           "of": "FP64 adjoint against central FD of the FP64 forward's J"}
    if a32:
        rel32 = np.abs(np.array(a32) - fds) / np.abs(fds)
        res.update({"fp32_median": float(np.median(rel32)), "fp32_max": float(rel32.max())})
    return res


def form_sanity(args, sw):
    """swe_sanity (mass, energy, h_min, first negative cell in one device pass) on the
    headline grid: its bandwidth against the HBM roofline (reads h, hu, hv, B: 32 B per
    cell), per synchronous call (launch, reduction and the copy of four numbers back)."""
    n = args.n
    h, hu, hv, B = workload(n, args.seed)
    with sw.Solver(n, n, bc="transmissive") as s:
        s.upload(h, hu, hv, B)
        s.sanity()
        reps = 10
        t0 = time.perf_counter()
        for _ in range(reps):
            r = s.sanity()
        wall = (time.perf_counter() - t0) / reps
    gbs = 32.0 * n * n / wall / 1e9
    return {"grid": [n, n], "ms_per_call_wall": wall * 1e3, "bytes_per_cell": 32,
            "achieved_gbs": gbs, "hbm_frac_of_measured": gbs / peaks()[0],
            "mass": r["mass"], "h_min": r["h_min"], "first_negative": r["first_negative"]}


def form_slabs(args, sw):
    """The headline grid as x-slabs on this one GPU, against one context: the
    single-process slab group (swe_slabs: device-side exchange overlapped with each
    stage's inner tile rows, device-side CFL max) with 2 and 4 slabs, and the host-staged
    SlabGrid (swe_stage + swe_halo through host memory) with 2."""
    n, K = args.n, 3
    h, hu, hv, B = workload(n, args.seed)
    out = {"grid": [n, n], "steps": K}
    for parts in (2, 4):
        with sw.slabs.DeviceSlabGrid(n, n, bc="transmissive", parts=parts) as grid:
            grid.upload(h, hu, hv, B)
            grid.step(1)
            l0 = grid.kernel_launches()
            grid.step(K)
            ms = grid.last_step_ms()
            out[f"device_{parts}"] = {
                "parts": parts, "ms_per_step": ms / K, "gcups": n * n * K / (ms / 1e3) / 1e9,
                "launches_per_step": (grid.kernel_launches() - l0) / K,
                "exchange": "2 rows x 3 fields per interface per stage, cudaMemcpyPeerAsync "
                            "on the sending slab's stream, overlapped with inner tile rows"}
    grid = sw.slabs.SlabGrid(n, n, bc="transmissive", parts=2)
    try:
        grid.upload(h, hu, hv, B)
        grid.step(1)
        t0 = time.perf_counter()
        grid.step(K)
        secs = time.perf_counter() - t0
    finally:
        grid.close()
    out["host_staged_2"] = {"parts": 2, "ms_per_step_wall": secs * 1e3 / K,
                            "gcups": n * n * K / secs / 1e9,
                            "exchange": "2 rows x 3 fields per interface per stage, through "
                                        "host memory"}
    return out


def form_snapshots(args, sw):
    """NetCDF snapshots of the headline grid every snap_every steps, two ways: through the
    device path (pack kernel + writer thread, overlapped with stepping) and the
    reference's way (synchronous download of the ghosted state, then packing and writing
    on the host, cuda_solver.hpp:211-219).  Reports ms per step of each against plain
    stepping; the files are deleted afterwards."""
    import shutil
    import tempfile
    n, K, every = args.n, args.snap_steps, args.snap_every
    h, hu, hv, B = workload(n, args.seed)
    root = tempfile.mkdtemp(prefix="swe_snap_", dir=args.snap_dir or None)
    out = {"grid": [n, n], "steps": K, "save_every": every, "records": K // every + 1,
           "record_bytes": 3 * n * n * 8 + 8, "dir_fs": _fs_type(root)}
    try:
        with sw.Solver(n, n, bc="transmissive") as s:
            s.upload(h, hu, hv, B)
            s.step(1)
            ms = {}
            for mode in ("none", "device", "host"):
                s.upload(h, hu, hv)
                s.time = 0.0
                path = os.path.join(root, f"{mode}.nc")
                w = None if mode == "none" else sw.output.NetCDFWriter(path, s, save_every=every)
                if w:
                    w.write_bathymetry(B)
                t0 = time.perf_counter()
                for k in range(K + 1):
                    if w and k % every == 0:
                        if mode == "device":
                            w.write_snapshot(s, s.time)
                        else:
                            w.write_snapshot(s.download(), s.time)
                    if k < K:
                        s.step(1)
                t_loop = time.perf_counter() - t0
                if w:
                    w.flush()
                t_all = time.perf_counter() - t0
                ms[mode] = {"ms_per_step_loop": t_loop * 1e3 / K, "ms_per_step_with_flush": t_all * 1e3 / K}
                if mode == "device":
                    c, wr, nb = w.stats()
                    ms[mode].update({"writer_copy_s": c, "writer_write_s": wr, "writer_bytes": nb,
                                     "file_write_gbs": nb / wr / 1e9 if wr > 0 else None})
                if w:
                    w.close()
                    os.remove(path)
            out.update(ms)
            base = ms["none"]["ms_per_step_loop"]
            for mode in ("device", "host"):
                # the stall the stepping loop sees per record, and the wait for the last
                # records to reach the file after the loop
                out[mode]["stall_ms_per_record"] = (
                    (ms[mode]["ms_per_step_loop"] - base) * K / out["records"])
                out[mode]["final_flush_ms"] = (
                    (ms[mode]["ms_per_step_with_flush"] - ms[mode]["ms_per_step_loop"]) * K)
    finally:
        shutil.rmtree(root, ignore_errors=True)
    return out


def form_modular(args, sw):
    """The modular scheme (SerialSolver's arithmetic, every reconstruction x Riemann
    solver, with and without bathymetry) on a 4096^2 wet state over seeded bathymetry:
    GCUPS per combination, fixed dt at half the Serial backend's CFL guard."""
    n, K = 4096, 3
    P = importlib.import_module("shallow-water_gb300.problems")
    B, _ = P.gaussian_sum_bathymetry(n, n, n=16, seed=args.seed)
    h, hu, hv = P.dam_break(B)
    out = {"grid": [n, n], "steps": K, "bytes_per_cell_update": 216, "gcups": {}}
    for recon in ("PiecewiseConst", "MUSCL"):
        for riemann in ("HLL", "Rusanov", "ROE"):
            for bathy in (True, False):
                with sw.Solver(n, n, scheme="modular", reconstruction=recon, riemann=riemann,
                               bathymetry=bathy) as s:
                    s.upload(h, hu, hv, B)
                    dt = 0.5 * s.stable_dt()
                    s.step(1, dt)
                    s.step(K, dt)
                    ms = s.last_step_ms()
                key = f"{recon}+{riemann}+{'bathymetry' if bathy else 'none'}"
                out["gcups"][key] = n * n * K / (ms * 1e-3) / 1e9
    if not args.no_cpu_baseline:
        # the oracle's C restatement of SerialSolver, one core, MUSCL + HLL + bathymetry
        from oracle import port
        m = 512
        Bm, _ = P.gaussian_sum_bathymetry(m, m, n=16, seed=args.seed)
        hm, hum, hvm = P.dam_break(Bm)
        g = port.grid(m, m)
        dtm = 0.5 * port.modular_stable_dt(g, hm, hum, hvm)[0]
        t0 = time.perf_counter()
        port.modular_run(g, 1, 0, 1, hm, hum, hvm, Bm, 2, dtm)
        secs = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": m * m * 2 / secs / 1e9, "unit": "GCUPS", "cores": 1,
                               "kind": "port", "sample": "512^2, 2 steps, MUSCL+HLL+bathymetry"}
    return out


def _fs_type(path):
    """Filesystem type of path's mount (from /proc/mounts), for the record."""
    try:
        best, fs = "", "unknown"
        real = os.path.realpath(path)
        with open("/proc/mounts") as f:
            for line in f:
                parts = line.split()
                if len(parts) > 2 and real.startswith(parts[1]) and len(parts[1]) > len(best):
                    best, fs = parts[1], parts[2]
        return fs
    except OSError:
        return "unknown"


def run_forms(args, sw, fp64_gcups):
    forms = {}
    wanted = set(args.forms.split(","))
    for name, fn in (("fp32_mixed", lambda: form_fp32(args, sw, fp64_gcups)),
                     ("ensemble", lambda: form_ensemble(args, sw)),
                     ("adjoint", lambda: form_adjoint(args, sw)),
                     ("sanity", lambda: form_sanity(args, sw)),
                     ("slabs", lambda: form_slabs(args, sw)),
                     ("snapshots", lambda: form_snapshots(args, sw)),
                     ("modular", lambda: form_modular(args, sw))):
        if name not in wanted:
            continue
        try:
            forms[name] = fn()
        except Exception as exc:  # keep the headline line whatever an extra does
            forms[name] = {"error": f"{type(exc).__name__}: {exc}"}
    return forms


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

    # End to end through the public API with pinned host buffers: per step, the state
    # and bathymetry go up, one RK3 step runs, the state comes back.  swe_step_host does
    # the three in one call, with the transfers overlapped with the stage kernels; the
    # three separate calls (swe_upload, swe_step, swe_download) are timed beside it.
    nt = (n + 4) * (n + 4)
    pin = [torch.empty((n + 4, n + 4), dtype=torch.float64, pin_memory=True).numpy()
           for _ in range(7)]
    for dst, src in zip(pin[:4], (h, hu, hv, B)):
        np.copyto(dst, src)
    E = max(1, args.e2e_steps)
    outs = tuple(pin[4:7])

    def one_call():
        solver.step_host(pin[0], pin[1], pin[2], pin[3], out=outs, n_steps=1)

    def three_calls():
        solver.upload(pin[0], pin[1], pin[2], pin[3])
        solver.step(1)
        solver.download(outs)

    def e2e_rate(fn):
        fn()
        dist.barrier()
        torch.cuda.synchronize()
        e0 = time.perf_counter()
        for _ in range(E):
            fn()
        torch.cuda.synchronize()
        return cells * E * dist.world / dist.max(time.perf_counter() - e0) / 1e9

    e2e_clocks = ClockSampler(dev)
    e2e = {"value": e2e_rate(one_call), "unit": "GCUPS",
           "h2d_bytes_per_step": 4 * nt * 8, "d2h_bytes_per_step": 3 * nt * 8,
           "steps": E, "api": "swe_step_host (upload, one RK3 step, download; transfers "
                              "overlapped with the stage kernels by bands of rows), pinned "
                              "host buffers"}
    # the last call's compute stream, first band's wait through the last stage band
    e2e["compute_stream_ms"] = solver.last_step_ms()
    e2e["wall_ms_per_step"] = cells * dist.world / (e2e["value"] * 1e9) * 1e3
    # Both paths advance the same input by one step: their outputs must agree bitwise.
    one = [np.array(a) for a in outs]
    e2e["three_calls_value"] = e2e_rate(three_calls)
    e2e["clocks"] = e2e_clocks.stop()
    e2e["bitwise_equal_to_three_calls"] = all(
        np.array_equal(x.view(np.uint64), y.view(np.uint64)) for x, y in zip(one, outs))
    del one
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
        "fp64_pipe_roofline": fp64_pipe(value, dev),
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
        # The single-core figure, HPC_solver's configuration: one full-grid step.
        secs1 = time_cpu_port(h, hu, hv, B, n, 1, 0, threads=1)
        line["cpu_baseline_1core"] = {
            "value": cells / secs1 / 1e9, "unit": "GCUPS", "cores": 1, "kind": "port",
            "sample": f"{n}^2 workload from t=0, 1 full RK3 step, one thread"}
    if dist.rank == 0 and dist.world == 1 and not args.no_forms:
        line["forms"] = run_forms(args, sw, value)
        # Last in the line, so that a reader keeping only the end of the output keeps it.
        line["forms_summary"] = forms_summary(line)
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def forms_summary(line: dict) -> dict:
    """The figures of the forms, flat and short, for the end of the line."""
    f = line.get("forms", {})

    def get(*path):
        d = f
        for k in path:
            if isinstance(d, list) and isinstance(k, int) and k < len(d):
                d = d[k]
            elif isinstance(d, dict) and k in d:
                d = d[k]
            else:
                return None
        return d

    def r(x, nd=4):
        return None if x is None else float(f"{x:.{nd}g}")

    fd = get("adjoint", "fd_agreement") or {}
    return {
        "fp64_gcups": r(line.get("value")),
        "fp64_pipe_frac": r(line.get("fp64_pipe_roofline", {}).get("frac")),
        "fp64_hbm_frac": r(line.get("roofline", {}).get("frac")),
        "fp32_gcups": r(get("fp32_mixed", "gcups")),
        "fp32_hbm_frac": r(get("fp32_mixed", "hbm_frac_of_measured")),
        "fp32_vs_fp64": r(get("fp32_mixed", "speedup_vs_fp64")),
        "fp32_acc_grid_steps": [get("fp32_mixed", "accuracy_vs_fp64", "grid", 0),
                                get("fp32_mixed", "accuracy_vs_fp64", "steps")],
        "fp32_l1_h": r(get("fp32_mixed", "accuracy_vs_fp64", "l1_h"), 3),
        "fp32_linf_h": r(get("fp32_mixed", "accuracy_vs_fp64", "linf_h"), 3),
        "fp32_l1_hu": r(get("fp32_mixed", "accuracy_vs_fp64", "l1_hu"), 3),
        "fp32_l1_hv": r(get("fp32_mixed", "accuracy_vs_fp64", "l1_hv"), 3),
        "fp32_mass_drift": r(get("fp32_mixed", "accuracy_vs_fp64", "mass_drift_fp32"), 3),
        "fp64_mass_drift": r(get("fp32_mixed", "accuracy_vs_fp64", "mass_drift_fp64"), 3),
        "fp32_lake_max": r(get("fp32_mixed", "lake_at_rest", "max_abs_hu_hv_wet"), 3),
        "ens_fp64_gcups": r(get("ensemble", "fp64", "gcups")),
        "ens_fp32_gcups": r(get("ensemble", "fp32_mixed", "gcups")),
        "ens_fp32_hbm_frac": r(get("ensemble", "fp32_mixed", "hbm_frac_of_measured")),
        "adj_ratio_sqrt": r(get("adjoint", "ratio")),
        "adj_ratio_tape": r(get("adjoint", "ratio_tape")),
        "adj_ratio_segments": r(get("adjoint", "ratio_segments")),
        "adj32_ratio_sqrt": r(get("adjoint", "fp32_mixed", "ratio")),
        "adj32_ratio_tape": r(get("adjoint", "fp32_mixed", "ratio_tape")),
        "adj32_ratio_segments": r(get("adjoint", "fp32_mixed", "ratio_segments")),
        "adj_fd": {k: (r(v, 3) if isinstance(v, float) else v) for k, v in fd.items()
                   if k in ("eps", "directions", "grid", "steps", "median", "max",
                            "max_vs_abs_terms", "fp32_median", "fp32_max")},
        "adj_fd_noise_1e-3": {k: r(get("adjoint", "fd_agreement_noise_1e-3", k), 3)
                              for k in ("median", "max", "max_vs_abs_terms")},
        "slabs_device_2_gcups": r(get("slabs", "device_2", "gcups")),
        "cpu_gcups": r(line.get("cpu_baseline", {}).get("value")),
        "cpu_cores": line.get("cpu_baseline", {}).get("cores"),
        "cpu_1core_gcups": r(line.get("cpu_baseline_1core", {}).get("value")),
    }


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
