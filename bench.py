#!/usr/bin/env python
"""Throughput of the sweep + hydrogen-chemistry step on GB300.

A *step* is one Sweep::run_sweeps (src/sweep/mod.rs:258-272): every level sweep of the
timestep hierarchy, the chemistry of each sweep's active cells and the level
reassignment, over a seeded synthetic workload (default: 128^3 jittered-lattice
Voronoi cells, lognormal density, 64 sources, 84 directions, 4 levels).  Both GPU
arithmetics run from identical initial conditions: the FP64 drop-in and the mixed
path (FP32 transport, FP64 chemistry); `value` is the mixed path's cell-direction
updates per second, device-timed by CUDA events on the library's launch stream,
and the error of x_HII / T between the two is reported with it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With N > 1 (under torchrun) every rank runs an independent replica on its own GPU
(the sweep does not shard on one node); value = all ranks' updates / slowest rank.
`--impl reference` times the CPU restatement of the reference algorithm (oracle/) on
the host cores instead, one process per core, on a bounded sample of the workload.
"""
from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-dir updates/s + chem cells/s, mixed vs FP64 GPU at stated x_HII/T error"
UNIT = "cell-dir updates/s"


# --------------------------------------------------------------------------- helpers
def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Dist:
    """Barrier / reductions across torchrun ranks (gloo on host tensors; replicas do not
    exchange data, so no device collective is needed)."""

    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def allreduce(self, value: float, op: str) -> float:
        if self.world == 1:
            return value
        import torch
        t = torch.tensor([value], dtype=torch.float64)
        self.td.all_reduce(t, op={"max": self.td.ReduceOp.MAX, "sum": self.td.ReduceOp.SUM}[op])
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d.get("hbm_gbs"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def mean_downwind_faces(grid, directions: np.ndarray, sample: int = 60000, seed: int = 0) -> float:
    """F_dn: mean number of faces with n.d > 0 per (cell, direction), over a random
    sample of cells (all directions)."""
    rng = np.random.default_rng(seed)
    n = grid.num_cells
    cells = rng.choice(n, size=min(sample, n), replace=False)
    counts = np.diff(grid.row_ptr)[cells]
    faces = np.concatenate([np.arange(grid.row_ptr[c], grid.row_ptr[c + 1]) for c in cells])
    dots = grid.normal[faces] @ directions.T  # faces x D
    return float((dots > 0).sum() / (len(cells) * directions.shape[0])) if counts.sum() else 0.0


# DRAM bytes per task of the pull transport kernel (nested-loop lockstep variant, the
# autotuner's choice on C2), measured by ncu (dram__bytes_read.sum +
# dram__bytes_write.sum) on a level-0 launch of the C2 grid at 64^3 (22,020,096 tasks):
# 2.411 GB per launch.  The per-launch traffic at other sizes is scaled by the tasks of
# a launch.
MEASURED_DRAM_BYTES_PER_TASK = {"mixed": 109.5}
TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of a level-0 k_sweep_pull_lock2 launch "
                  "on C2 64^3, per task")


# FP64 work of one try_timestep_update attempt of the chemistry kernel (mixed path),
# counted by ncu on a level-0 launch of C2 64^3 (about one attempt per cell): 366 DFMA,
# 63 DADD, 156 DMUL thread instructions, i.e. 2 * 366 + 63 + 156 FP64 flops.
CHEM_FP64_FLOPS_PER_ATTEMPT = 2 * 366 + 63 + 156


def chemistry_figures(d: dict, res: dict) -> dict:
    """Chemistry cells/s, attempts (substeps tried) per cell update and FP64 flop rate
    over the chemistry launches' CUDA-event time."""
    cells, attempts, ms = float(d["chem_cells"]), float(d["chem_attempts"]), float(d["chem_ms"])
    return {"cells_per_s": res["chem_cells_per_s"],
            "attempts_per_cell": attempts / cells if cells else None,
            "fp64_flops_per_attempt": CHEM_FP64_FLOPS_PER_ATTEMPT,
            "fp64_tflops": attempts * CHEM_FP64_FLOPS_PER_ATTEMPT / (ms * 1e-3) / 1e12 if ms else None,
            "kernel_ms": ms}


def bytes_per_task(f_dn: float, rate_bytes: int, counter_bytes: int = 1) -> float:
    """Algorithmic bytes of one cell-direction update: read incoming, periodic and the
    old outgoing rate, write the new one, and read-modify-write the incoming rate and
    the dependency counter of every downwind neighbour: S_r (4 + 2 F_dn) + 2 S_c F_dn."""
    return rate_bytes * (4 + 2 * f_dn) + 2 * counter_bytes * f_dn


def build_workload(name: str, n_per_side, nthreads: int, grid_device: str = "host"):
    from subsweep_gb300 import workloads
    if name == "c2":
        return workloads.c2_lognormal(n_per_side=n_per_side or 128, nthreads=nthreads, grid_device=grid_device)
    if name == "c1":
        return workloads.c1_small_periodic(n_per_side=n_per_side or 32, nthreads=nthreads, grid_device=grid_device)
    if name == "c4":
        return workloads.c4_grf(n_per_side=n_per_side or 256, nthreads=nthreads, grid_device=grid_device)
    if name == "c3":
        return workloads.c3_batched(num_boxes=n_per_side or 256, nthreads=nthreads)
    raise SystemExit(f"unknown workload {name}")


# --------------------------------------------------------------------------- CPU arm
def _cpu_worker(args):
    """One host core running the oracle on its own copy of the sample workload."""
    name, n_per_side, warmup, steps, seed_offset = args
    sys.path.insert(0, str(ROOT))
    from oracle import binding
    from subsweep_gb300.sweep import directions_from_num
    w = sample_workload(name, n_per_side, seed_offset)
    o = binding.OracleSweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
                            directions_from_num(w.params.num_directions()))
    for _ in range(warmup):
        o.run_sweeps()
    t0_tasks, t0_chem = o.work()
    t0 = time.perf_counter()
    for _ in range(steps):
        o.run_sweeps()
    dt = time.perf_counter() - t0
    t1_tasks, t1_chem = o.work()
    return t1_tasks - t0_tasks, t1_chem - t0_chem, dt


def sample_workload(name: str, n_per_side: int, seed_offset: int):
    """A bounded CPU sample of a workload: the same generator at n_per_side^3 cells (C4
    with its sources scaled to the sample's cells), or one C3 box."""
    from subsweep_gb300 import workloads
    if name == "c1":
        return workloads.c1_small_periodic(n_per_side=n_per_side, nthreads=1)
    if name == "c4":
        sources = max(1, round(1000 * (n_per_side / 256) ** 3))
        return workloads.c4_grf(n_per_side=n_per_side, seed=4 + seed_offset, num_sources=sources, nthreads=1)
    if name == "c3":
        return workloads.c3_batched(num_boxes=1, seed=3 + seed_offset, nthreads=1)
    return workloads.c2_lognormal(n_per_side=n_per_side, seed=2 + seed_offset, nthreads=1)


def sample_label(name: str, n_per_side: int) -> str:
    if name == "c3":
        return "one C3 box (512..64000 cells, 32 dirs, 2 levels) per process"
    return f"{name.upper()} generator at {n_per_side}^3 cells"


def cpu_sample(workload: str, n_per_side: int, warmup: int, steps: int, procs: int):
    from oracle import binding
    binding.build()
    if procs == 1:
        res = [_cpu_worker((workload, n_per_side, warmup, steps, 0))]
    else:
        import multiprocessing as mp
        ctx = mp.get_context("spawn")
        with ctx.Pool(procs) as pool:
            res = pool.map(_cpu_worker, [(workload, n_per_side, warmup, steps, i) for i in range(procs)])
    tasks = sum(r[0] for r in res)
    chem = sum(r[1] for r in res)
    wall = max(r[2] for r in res)
    return tasks, chem, wall


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def run_reference(args, dist: Dist):
    if dist.rank != 0:
        return
    from subsweep_gb300 import workloads
    procs = os.cpu_count() or 1
    n_side = args.cpu_sample_side
    tasks, chem, wall = cpu_sample(args.workload, n_side, 1, max(1, args.steps), procs)
    value = tasks / wall
    sample = (f"{sample_label(args.workload, n_side)}, one oracle process per host core "
              f"({procs}), each 1 warm-up + {max(1, args.steps)} timed steps")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * wall / max(1, args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workloads.label(args.workload, args.n_per_side), "cpu": cpu_model()},
        "chem_cells_per_s": chem / wall,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- GPU arm
def time_precision(w, precision: str, device: int, warmup: int, steps: int, dist: Dist, graphs: bool = False):
    from subsweep_gb300 import Sweep
    s = Sweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
              precision=precision, device=device, use_graphs=graphs and precision == "mixed")
    for _ in range(warmup):
        s.run_sweeps()
    dist.barrier()
    st0 = s.stats()
    sampler = ClockSampler(device)
    sampler.start()
    for _ in range(steps):
        s.run_sweeps()
    clocks = sampler.stop()
    st1 = s.stats()
    dist.barrier()
    d = {k: st1[k] - st0[k] for k in st1}
    return s, d, clocks


def run_ours(args, dist: Dist):
    from subsweep_gb300 import build as native_build
    native_build.build()
    from subsweep_gb300.sweep import directions_from_num

    device = dist.local
    t0 = time.perf_counter()
    # the grids of the GPU arm are built on the GPU (csrc/voronoi_gpu.cu)
    w = build_workload(args.workload, args.n_per_side, nthreads=os.cpu_count() or 1, grid_device=f"gpu:{device}")
    grid_s = time.perf_counter() - t0
    directions = directions_from_num(w.params.num_directions())
    f_dn = mean_downwind_faces(w.grid, directions)

    results = {}
    handles = {}
    precisions = ("fp64", "mixed") if args.precision == "both" else (args.precision,)
    for precision in precisions:
        s, d, clocks = time_precision(w, precision, device, args.warmup, args.steps, dist, graphs=args.graphs)
        handles[precision] = s
        step_s = d["step_ms"] / 1e3
        max_step_s = dist.allreduce(step_s, "max")
        tasks = dist.allreduce(float(d["tasks"]), "sum")
        chem = dist.allreduce(float(d["chem_cells"]), "sum")
        results[precision] = {
            "cell_dir_updates_per_s": tasks / max_step_s,
            "chem_cells_per_s": chem / max_step_s,
            "ms_per_step": 1e3 * max_step_s / args.steps,
            "tasks": tasks, "chem_cells": chem, "d": d, "clocks": clocks,
        }
    # error of the mixed path against the FP64 drop-in after identical steps
    head = "mixed" if "mixed" in results else "fp64"
    sched_levels = int(handles[head].stats()["schedule_levels"])
    pull_variant = int(handles[head].stats()["pull_variant"])
    err = None
    if len(results) == 2:
        fm, ff = handles["mixed"].fields(), handles["fp64"].fields()
        err = {
            "max_abs_dx_HII": float(np.abs(fm["ionized_hydrogen_fraction"] - ff["ionized_hydrogen_fraction"]).max()),
            "max_rel_dT": float((np.abs(fm["temperature"] - ff["temperature"]) / ff["temperature"]).max()),
            "levels_equal_fraction": float((handles["mixed"].cell_state()["level"] ==
                                            handles["fp64"].cell_state()["level"]).mean()),
            # FP32 rates are stored in units of 2^-96 of the total source: rates below
            # 1e-20 of the total luminosity are compared against that floor
            "max_rel_photon_rate": float((np.abs(fm["photon_rate"] - ff["photon_rate"]) /
                                          np.maximum(np.abs(ff["photon_rate"]), 1e-20 * float(w.source.sum()))).max()),
        }
        handles["fp64"].close()

    # end to end through the C ABI: each step = sw_step + field write-back to host memory
    s = handles[head]
    n = w.grid.num_cells
    out = {k: np.empty(n) for k in ("ionized_hydrogen_fraction", "temperature", "timestep", "photon_rate")}
    s.fields(out)  # untimed: the caller's buffers are mapped once, then reused every step
    st0 = s.stats()
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.run_sweeps()
        s.fields(out)
    e2e_s = time.perf_counter() - t0
    st1 = s.stats()
    e2e_max = dist.allreduce(e2e_s, "max")
    e2e_tasks = dist.allreduce(float(st1["tasks"] - st0["tasks"]), "sum")
    s.close()

    mixed = results[head]
    d = mixed["d"]
    peaks = measured_peaks()
    b_task = bytes_per_task(f_dn, 4 if head == "mixed" else 8)
    achieved_gbs = d["tasks"] * b_task / (d["transport_kernel_ms"] / 1e3) / 1e9 if d["transport_kernel_ms"] else None
    launches = d["transport_launches"]
    traffic = (MEASURED_DRAM_BYTES_PER_TASK[head] * d["tasks"] / launches
               if head in MEASURED_DRAM_BYTES_PER_TASK and launches else None)
    cpu = None
    if dist.rank == 0 and args.gpus == 1 and not args.no_cpu_baseline:
        c_tasks, c_chem, c_wall = cpu_sample(args.workload, args.cpu_sample_side, 1, 1, 1)
        cpu = {"value": c_tasks / c_wall, "unit": UNIT, "cores": 1, "kind": "port", "cpu": cpu_model(),
               "sample": f"{sample_label(args.workload, args.cpu_sample_side)}, oracle, "
                         f"1 warm-up + 1 timed step ({c_tasks} tasks, {c_wall:.1f} s)",
               "chem_cells_per_s": c_chem / c_wall}
    if dist.rank != 0:
        return
    line = {
        "metric": METRIC,
        "value": mixed["cell_dir_updates_per_s"],
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": mixed["ms_per_step"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 transport + f64 chemistry" if head == "mixed" else "f64",
        "data": "synthetic",
        "config": dict(w.describe(), precision=head, replicas=args.gpus, cuda_graph_steps=bool(args.graphs),
                       l2="per-(cell,dir) state of %.1f GB per array > 129 MB L2; no flush needed" %
                          (n * ((w.params.num_directions() + 7) // 8 * 8) * 4 / 1e9),
                       grid_build_s=round(grid_s, 1), grid_builder="gpu"),
        "chem_cells_per_s": mixed["chem_cells_per_s"],
        "chemistry": chemistry_figures(d, mixed),
        "fp64": ({k: results["fp64"][k] for k in ("cell_dir_updates_per_s", "chem_cells_per_s", "ms_per_step")}
                 if "fp64" in results else None),
        "speedup_mixed_vs_fp64": (results["fp64"]["ms_per_step"] / mixed["ms_per_step"]
                                  if len(results) == 2 else None),
        "error_mixed_vs_fp64": err,
        "e2e": {"value": e2e_tasks / e2e_max, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 4 * 8 * n},
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": (achieved_gbs / peaks["hbm_gbs"]) if achieved_gbs else None,
                     "traffic": traffic, "traffic_unit": "bytes per launch",
                     "traffic_source": TRAFFIC_SOURCE if traffic else None,
                     # the measured DRAM bytes over the same CUDA-event time
                     "traffic_gbs": (traffic * launches / (d["transport_kernel_ms"] / 1e3) / 1e9
                                     if traffic and d["transport_kernel_ms"] else None),
                     "kernel": "k_sweep_pull" if head == "mixed" else "k_sweep_sched<double>",
                     "bytes_per_task": b_task, "f_dn": f_dn, "launches": launches,
                     # face geometry, 16 B per face, reported beside B_task and not in it
                     # (the mixed sweep reads its precomputed records and slots instead)
                     "geometry_bytes_per_cell": 16.0 * w.grid.num_faces / w.grid.num_cells,
                     "peak_source": peaks["source"]},
        "gpu_launches": int(d["kernel_launches"]),
        "clocks": mixed["clocks"],
        "clocks_fp64": results["fp64"]["clocks"] if "fp64" in results else None,
        "cpu_baseline": cpu,
        "stats": {"tasks": d["tasks"], "levelled_sweeps": d["levelled_sweeps"],
                  "transport_attempts": d["transport_attempts"],
                  "pull_variant": pull_variant,
                  "sweeps": d["level_sweeps"], "schedule_levels": sched_levels,
                  "chem_attempts": d["chem_attempts"], "transport_kernel_ms": d["transport_kernel_ms"],
                  "sweep_ms": d["sweep_ms"], "chem_ms": d["chem_ms"], "level_ms": d["level_ms"],
                  "fp64_transport_kernel_ms": (results["fp64"]["d"]["transport_kernel_ms"]
                                               if "fp64" in results else None),
                  "fp64_chem_ms": results["fp64"]["d"]["chem_ms"] if "fp64" in results else None},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["c1", "c2", "c3", "c4"], default="c2")
    ap.add_argument("--n-per-side", type=int, default=None)
    ap.add_argument("--cpu-sample-side", type=int, default=40)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--graphs", action="store_true", help="replay each mixed-path step as one CUDA graph")
    ap.add_argument("--precision", choices=["both", "fp64", "mixed"], default="both",
                    help="GPU arithmetic(s) to time; value reports the mixed path when it runs")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
