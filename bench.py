#!/usr/bin/env python
"""Throughput of the sweep + hydrogen-chemistry step on GB300.

A *step* is one Sweep::run_sweeps (src/sweep/mod.rs:258-272): every level sweep of the
timestep hierarchy, the chemistry of each sweep's active cells and the level
reassignment, over a seeded synthetic workload (default: 256^3 jittered-lattice
Voronoi cells of 750 pc, density the exponential of a Gaussian random field, 1000
sources at the density peaks, 84 directions, 4 levels).  Both GPU arithmetics run
from identical initial conditions, one after the other: the FP64 drop-in and the
mixed path (FP32 transport, FP64 chemistry); `value` is the mixed path's
cell-direction updates per second, device-timed by CUDA events on the library's
launch stream, and the error of x_HII / T between the two is reported with it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With N > 1 (under torchrun) every rank runs an independent replica on its own GPU
(the sweep does not shard on one node); value = all ranks' updates / slowest rank.
`--impl reference` times the CPU restatement of the reference algorithm (oracle/) on
every host core instead, over the same full workload built by the oracle alone; each
step is a bounded sample of a level-0 sweep (a subset of the directions).
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


# DRAM bytes per task of the pull transport kernel (lockstep kernel with 2 lanes per
# task, variant 122, the autotuner's choice on C4 256^3), measured by ncu
# (dram__bytes_read.sum + dram__bytes_write.sum, one pass) on a level-0 launch of the
# C4 generator at 256^3 (1,409,286,144 tasks): 142.04 + 20.99 GB per launch.  The
# per-launch traffic of other launches is scaled by their tasks.
MEASURED_DRAM_BYTES_PER_TASK = {"mixed": 115.7}
TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of a level-0 k_sweep_pull_lockg<2,2,1> "
                  "launch on C4 256^3, per task")


# FP64 work of one try_timestep_update attempt of the chemistry kernel (mixed path: rate
# fits in FP32, the update in FP64), counted by ncu on the second chemistry launch of
# the C4 generator at 64^3 (60.18 M attempts by the sweep trace): 55.2 DFMA, 41.1 DMUL
# and 9.0 DADD thread instructions per attempt, i.e. 2 * 55 + 41 + 9 FP64 flops.
CHEM_FP64_FLOPS_PER_ATTEMPT = 2 * 55 + 41 + 9


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


def build_workload(name: str, n_per_side, nthreads: int, grid_device: str = "host", thick: bool = False,
                   voronoi=None):
    from subsweep_gb300 import workloads
    kw = {"nthreads": nthreads, "voronoi": voronoi}
    if name == "c1":
        return workloads.c1_small_periodic(n_per_side=n_per_side or 32, grid_device=grid_device, **kw)
    if name == "c2":
        return workloads.c2_lognormal(n_per_side=n_per_side or 128, grid_device=grid_device, thick=thick, **kw)
    if name == "c4":
        return workloads.c4_grf(n_per_side=n_per_side or 256, grid_device=grid_device, thick=thick, **kw)
    if name == "c5":
        return workloads.c5_grf(n_per_side=n_per_side or 384, grid_device=grid_device, thick=thick, **kw)
    if name == "c3":
        return workloads.c3_batched(num_boxes=n_per_side or 256, thick=thick, **kw)
    raise SystemExit(f"unknown workload {name}")


def workload_config(w) -> dict:
    """The `config` of both arms' lines: the workload and its inputs."""
    return dict(w.describe(), l2="per-(cell,dir) state of %.1f GB per FP32 array > 129 MB L2; no flush needed" %
                (w.grid.num_cells * ((w.params.num_directions() + 7) // 8 * 8) * 4 / 1e9))


# --------------------------------------------------------------------------- CPU arm
def oracle_voronoi(threads: int):
    """Grid builder for the CPU arm: the oracle's own Voronoi producer, wrapped in the
    grid record the workload generators fill (a plain dataclass: no library of the
    package is loaded)."""
    from oracle import binding
    from subsweep_gb300 import grid as gridmod

    def build(points, box):
        g = binding.voronoi(points, box, threads)
        if g["failed_cells"] or g["dropped_faces"]:
            raise RuntimeError(f"oracle Voronoi: {g['failed_cells']} failed cells, {g['dropped_faces']} dropped faces")
        return gridmod.Grid(row_ptr=g["row_ptr"], nbr=g["nbr"], kind=g["kind"], area=g["area"], normal=g["normal"],
                            volume=g["volume"], size=g["size"], position=np.asarray(points, np.float64),
                            box_size=np.full(3, float(box)), periodic=True)
    return build


class OracleSample:
    """The oracle (the reference's algorithm restated, FP64) on the host cores, over the
    whole workload grid.  A step is a bounded sample of a level-0 sweep: the transport
    of `k` of the D directions over every cell, in the reference's task order (its
    BinaryHeap keyed by direction), one direction per worker thread (directions are
    independent within a level sweep), followed by the chemistry of k/D of the cells;
    successive steps take the next directions and cells."""

    def __init__(self, w, threads: int):
        from oracle import binding
        self.D = w.params.num_directions()
        self.k = max(1, min(threads, self.D))
        self.threads = threads
        self.n = w.grid.num_cells
        self.o = binding.OracleSweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature,
                                     w.source, binding.directions_from_num(self.D), order=binding.ORDER_HEAP,
                                     num_threads=threads, partition=binding.PARTITION_DIRECTIONS)
        self.index = 0

    def step(self) -> tuple:
        i = self.index
        self.index += 1
        return self.o.sample_sweep(0, i * self.k, self.k, i * (self.n * self.k // self.D))

    def describe(self, steps: int) -> str:
        return (f"the full grid ({self.n} cells); each step the level-0 transport of {self.k} of the {self.D} "
                f"directions (rotating) over every cell in the reference's BinaryHeap task order plus the chemistry "
                f"of {self.k}/{self.D} of the cells, {self.threads} threads (one direction each), {steps} timed steps")

    def close(self):
        self.o.close()


def time_oracle(sample: OracleSample, warmup: int, steps: int) -> tuple:
    for _ in range(warmup):
        sample.step()
    tasks = chem = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        a, b = sample.step()
        tasks += a
        chem += b
    return tasks, chem, time.perf_counter() - t0


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
    """CPU arm: the reference's algorithm (the oracle restatement; the reference itself
    cannot be built) on every host core, over the same full workload, built by the
    oracle alone (its own Voronoi producer and direction tables)."""
    if dist.rank != 0:
        return
    from oracle import binding
    binding.build()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    w = build_workload(args.workload, args.n_per_side, threads, thick=args.thick, voronoi=oracle_voronoi(threads))
    sample = OracleSample(w, threads)
    setup_s = time.perf_counter() - t0
    tasks, chem, wall = time_oracle(sample, args.warmup, args.steps)
    value = tasks / wall
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(workload_config(w), cpu=cpu_model(), setup_s=round(setup_s, 1)),
        "chem_cells_per_s": chem / wall,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample.describe(args.steps)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    sample.close()
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- GPU arm
def time_precision(w, precision: str, device: int, warmup: int, steps: int, dist: Dist, graphs: bool = False,
                   e2e: bool = False, snapshot_after: int = 0):
    """W untimed steps, then `steps` timed ones: the device time of each sw_step from the
    library's CUDA events and, with `e2e`, the host wall time of sw_step followed by the
    write-back of x_HII, T, the species timestep and the photon rate into the caller's
    host arrays (the same steps).  The fields and levels after `snapshot_after` timed
    steps are kept (outside the timed region) for the comparison of precisions."""
    from subsweep_gb300 import Sweep
    t_create = time.perf_counter()
    s = Sweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
              precision=precision, device=device, use_graphs=graphs and precision == "mixed")
    create_s = time.perf_counter() - t_create
    for _ in range(warmup):
        s.run_sweeps()
    n = w.grid.num_cells
    out = {k: np.empty(n) for k in ("ionized_hydrogen_fraction", "temperature", "timestep", "photon_rate")}
    if e2e:
        s.fields(out)  # the caller's buffers are mapped once, then reused every step
    dist.barrier()
    st0 = s.stats()
    per_step, wall, snap = [], 0.0, None
    sampler = ClockSampler(device)
    sampler.start()
    for k in range(steps):
        before = s.stats()["step_ms"]
        t0 = time.perf_counter()
        s.run_sweeps()
        if e2e:
            s.fields(out)
        wall += time.perf_counter() - t0
        per_step.append(s.stats()["step_ms"] - before)
        if k + 1 == snapshot_after:
            snap = (s.fields(), s.cell_state()["level"])
    clocks = sampler.stop()
    st1 = s.stats()
    dist.barrier()
    d = {k: st1[k] - st0[k] for k in st1}
    for k in ("task_spaces", "device_bytes", "pull_variant", "schedule_levels"):  # states, not counters
        d[k] = st1[k]
    return s, d, clocks, {"per_step_ms": per_step, "wall_s": wall, "snapshot": snap, "create_s": create_s}


def precision_errors(mixed: dict, fp64: dict, lv_mixed, lv_fp64, total_source: float) -> dict:
    """Mixed path against the FP64 drop-in after the same steps from the same inputs:
    over every cell and over the cells the radiation reaches (photon rate above 1e-6
    of the total source).  x_HII is compared absolutely and relative to x_HII and to
    the neutral fraction 1 - x_HII."""
    x_m, x_f = mixed["ionized_hydrogen_fraction"], fp64["ionized_hydrogen_fraction"]
    t_m, t_f = mixed["temperature"], fp64["temperature"]
    r_m, r_f = mixed["photon_rate"], fp64["photon_rate"]
    lit = r_f > 1e-6 * total_source

    def on(mask):
        if not mask.any():
            return None
        dx = np.abs(x_m[mask] - x_f[mask])
        rel_t = np.abs(t_m[mask] - t_f[mask]) / t_f[mask]
        rel_x, rel_n = dx / x_f[mask], dx / (1.0 - x_f[mask])
        return {
            "cells": int(mask.sum()),
            "max_abs_dx_HII": float(dx.max()),
            "max_rel_dx_HII": float(rel_x.max()),
            "max_rel_d_neutral": float(rel_n.max()),
            "max_rel_dT": float(rel_t.max()),
            # how many cells exceed 1e-4, and the error that all but 1e-5 of the cells meet
            "cells_above_1e-4": {"abs_dx_HII": int((dx > 1e-4).sum()), "rel_dx_HII": int((rel_x > 1e-4).sum()),
                                 "rel_d_neutral": int((rel_n > 1e-4).sum()), "rel_dT": int((rel_t > 1e-4).sum())},
            "quantile_1e-5": {"rel_dx_HII": float(np.quantile(rel_x, 1 - 1e-5)),
                              "rel_d_neutral": float(np.quantile(rel_n, 1 - 1e-5)),
                              "rel_dT": float(np.quantile(rel_t, 1 - 1e-5))},
            "levels_equal_fraction": float((lv_mixed[mask] == lv_fp64[mask]).mean()),
            # FP32 rates are stored in units of 2^-96 of the total source: below 1e-20
            # of it the comparison is against that floor
            "max_rel_photon_rate": float((np.abs(r_m[mask] - r_f[mask]) /
                                          np.maximum(np.abs(r_f[mask]), 1e-20 * total_source)).max()),
        }
    all_cells = on(np.ones_like(lit))
    worst = int(np.argmax(np.abs(t_m - t_f) / t_f))
    return dict(all_cells, lit_cells=on(lit), lit_fraction=float(lit.mean()),
                worst_T_cell={"x_HII": float(x_f[worst]), "T": float(t_f[worst]), "T_mixed": float(t_m[worst]),
                              "level": int(lv_fp64[worst]), "photon_rate_rel": float(r_f[worst] / total_source)})


def write_back_split(s, reps: int = 3) -> dict:
    """The e2e write-back after the timed steps, split (median ms of `reps` calls on the
    state of the last timed step, outside the timed region): sw_get_fields with the
    photon rate, and without it (the three per-cell copies alone); the difference is the
    photon-rate export.  With it, the number of cells at each timestep level.  Diagnostic
    only: an error is reported, never raised."""
    try:
        n = s.num_cells
        out = {k: np.empty(n) for k in ("ionized_hydrogen_fraction", "temperature", "timestep", "photon_rate")}
        s.fields(out)  # the buffers' pages touched once, as in the timed steps

        def median_ms(photon_rate: bool) -> float:
            times = []
            for _ in range(reps):
                t0 = time.perf_counter()
                s.fields(out, photon_rate=photon_rate)
                times.append(1e3 * (time.perf_counter() - t0))
            return float(np.median(times))

        split = {"fields_ms": median_ms(True), "fields_without_photon_rate_ms": median_ms(False), "calls": reps}
        # the export's cost follows the cells left behind by later sweeps: the level mix
        split["cells_per_level"] = np.bincount(s.cell_state()["level"]).tolist()
        return split
    except Exception as e:  # noqa: BLE001
        return {"error": repr(e)}


def radiation_field(s, w) -> dict:
    """How far the radiation reaches: the fraction of (cell, direction) incoming rates
    above 1e-6 of the total source per direction, of cells whose photon rate is above
    1e-6 of the total source, and of ionized cells."""
    total = float(w.source.sum())
    d = w.params.num_directions()
    frac_cd = None
    if w.grid.num_cells * d < 1 << 31:  # C5's per-task rates would take 38 GB of host memory
        inc = s.rates(which=("incoming",))["incoming"]
        frac_cd = float((inc > 1e-6 * total / d).mean())
        del inc
    f = s.fields()
    return {"cell_dir_above_1e-6_of_source": frac_cd,
            "cells_above_1e-6_of_source": float((f["photon_rate"] > 1e-6 * total).mean()),
            "cells_x_HII_above_0.5": float((f["ionized_hydrogen_fraction"] > 0.5).mean()),
            "cells_x_HII_above_1e-3": float((f["ionized_hydrogen_fraction"] > 1e-3).mean())}


def periodic_semantics(name: str, n_side: int, steps: int, device: int) -> dict:
    """The library's periodic semantics (a correction through a periodic face becomes
    visible in the next sweep) against the reference's (visible at once, in the order
    its BinaryHeap pops tasks): the FP64 drop-in against the oracle in the reference's
    literal order, on the workload's generator at n_side^3 cells."""
    from oracle import binding
    from subsweep_gb300 import Sweep
    sources = {"c4": {"num_sources": max(1, round(1000 * (n_side / 256) ** 3))}}.get(name, {})
    from subsweep_gb300 import workloads
    make = {"c1": workloads.c1_small_periodic, "c2": workloads.c2_lognormal, "c4": workloads.c4_grf}[name]
    w = make(n_per_side=n_side, nthreads=4, **sources)
    args = (w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source)
    lit = binding.OracleSweep(*args, binding.directions_from_num(w.params.num_directions()),
                              periodic_mode=binding.PERIODIC_IMMEDIATE, order=binding.ORDER_HEAP)
    gpu = Sweep(*args, precision="fp64", device=device)
    for _ in range(steps):
        lit.run_sweeps()
        gpu.run_sweeps()
    fl, fg = lit.fields(), gpu.fields()
    levels_gpu = gpu.cell_state()["level"]
    gpu.close()
    lit.close()
    total = float(w.source.sum())
    return {"sample": f"{w.name}, {steps} steps",
            "max_abs_dx_HII": float(np.abs(fg["ionized_hydrogen_fraction"] - fl["ionized_hydrogen_fraction"]).max()),
            "max_rel_dT": float((np.abs(fg["temperature"] - fl["temperature"]) / fl["temperature"]).max()),
            "max_rel_photon_rate": float((np.abs(fg["photon_rate"] - fl["photon_rate"]) /
                                          np.maximum(np.abs(fl["photon_rate"]), 1e-20 * total)).max()),
            "levels_equal_fraction": float((levels_gpu == fl["level"]).mean())}


def run_ours(args, dist: Dist):
    from subsweep_gb300 import build as native_build
    native_build.build()
    from subsweep_gb300.sweep import directions_from_num

    device = dist.local
    t0 = time.perf_counter()
    # the grids of the GPU arm are built on the GPU (csrc/voronoi_gpu.cu)
    w = build_workload(args.workload, args.n_per_side, nthreads=os.cpu_count() or 1,
                       grid_device=f"gpu:{device}", thick=args.thick)
    grid_s = time.perf_counter() - t0
    directions = directions_from_num(w.params.num_directions())
    f_dn = mean_downwind_faces(w.grid, directions)
    total_source = float(w.source.sum())

    # FP64 drop-in first, alone on the device (its downwind records then fit), then the
    # mixed path from the same inputs.  The FP64 drop-in is timed over the first
    # min(K, 4) of the K steps (a 256^3 FP64 step takes seconds); the speed-up and the
    # field comparison are taken over those common steps.
    results, snaps = {}, {}
    precisions = ("fp64", "mixed") if args.precision == "both" else (args.precision,)
    if args.workload == "c5":  # 4.76 G tasks: beyond the FP64 path's 32-bit task ids
        precisions = ("mixed",)
    head = precisions[-1]
    k_common = min(args.steps, 4) if len(precisions) == 2 else args.steps
    s = None
    for precision in precisions:
        steps = args.steps if precision == head else k_common
        s, d, clocks, timing = time_precision(w, precision, device, args.warmup, steps, dist, graphs=args.graphs,
                                              e2e=precision == head, snapshot_after=k_common)
        step_s = d["step_ms"] / 1e3
        max_step_s = dist.allreduce(step_s, "max")
        tasks = dist.allreduce(float(d["tasks"]), "sum")
        chem = dist.allreduce(float(d["chem_cells"]), "sum")
        results[precision] = {
            "cell_dir_updates_per_s": tasks / max_step_s,
            "chem_cells_per_s": chem / max_step_s,
            "ms_per_step": 1e3 * max_step_s / steps,
            "tasks_per_step": tasks / steps / args.gpus,
            "transport_tasks_per_s": (d["tasks"] / (d["transport_kernel_ms"] / 1e3)
                                      if d["transport_kernel_ms"] else None),
            "common_steps_ms": float(sum(timing["per_step_ms"][:k_common])),
            "tasks": tasks, "chem_cells": chem, "d": d, "clocks": clocks, "timing": timing,
        }
        snaps[precision] = timing["snapshot"]
        if precision != head:
            s.close()
    sched_levels = int(s.stats()["schedule_levels"])
    pull_variant = int(s.stats()["pull_variant"])
    err = None
    if len(results) == 2:
        (fm, lm), (ff, lf) = snaps["mixed"], snaps["fp64"]
        err = dict(precision_errors(fm, ff, lm, lf, total_source), after_timed_steps=k_common)
    field = radiation_field(s, w) if dist.rank == 0 else None
    write_back = write_back_split(s) if dist.rank == 0 else None
    n = w.grid.num_cells
    e2e_max = dist.allreduce(results[head]["timing"]["wall_s"], "max")
    e2e_tasks = dist.allreduce(float(results[head]["d"]["tasks"]), "sum")
    s.close()

    main = results[head]
    d = main["d"]
    peaks = measured_peaks()
    b_task = bytes_per_task(f_dn, 4 if head == "mixed" else 8)
    achieved_gbs = d["tasks"] * b_task / (d["transport_kernel_ms"] / 1e3) / 1e9 if d["transport_kernel_ms"] else None
    launches = d["transport_launches"]
    # the measured bytes per task are the full state's lockstep kernel's; the compact
    # state (C5) runs the geometry kernel, whose traffic is not captured
    traffic = (MEASURED_DRAM_BYTES_PER_TASK[head] * d["tasks"] / launches
               if head in MEASURED_DRAM_BYTES_PER_TASK and launches and not d.get("task_spaces") else None)
    cpu = semantics = None
    # C5's full-grid CPU sample would hold its per-task FP64 state (4.76 G tasks) in host memory
    if dist.rank == 0 and args.gpus == 1 and not args.no_cpu_baseline and args.workload != "c5":
        threads = os.cpu_count() or 1
        sample = OracleSample(w, threads)
        c_tasks, c_chem, c_wall = time_oracle(sample, 1, 1)
        cpu = {"value": c_tasks / c_wall, "unit": UNIT, "cores": threads, "kind": "port", "cpu": cpu_model(),
               "sample": sample.describe(1) + f" ({c_tasks} tasks, {c_wall:.1f} s), after 1 warm-up step",
               "chem_cells_per_s": c_chem / c_wall}
        sample.close()
        if args.workload in ("c1", "c2", "c4"):
            semantics = periodic_semantics(args.workload, 16, 4, device)
    if dist.rank != 0:
        return
    fp64 = results.get("fp64")
    line = {
        "metric": METRIC,
        "value": main["cell_dir_updates_per_s"],
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": main["ms_per_step"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 transport + f64 chemistry" if head == "mixed" else "f64",
        "data": "synthetic",
        "config": dict(workload_config(w), precision=head, replicas=args.gpus, cuda_graph_steps=bool(args.graphs),
                       grid_build_s=round(grid_s, 1), grid_builder="gpu",
                       # sw_create: upload, schedule, records and slots (outside the timed steps)
                       handle_create_s={p: round(r["timing"]["create_s"], 1) for p, r in results.items()}),
        "chem_cells_per_s": main["chem_cells_per_s"],
        "chemistry": chemistry_figures(d, main),
        "fp64": ({**{k: fp64[k] for k in ("cell_dir_updates_per_s", "chem_cells_per_s", "ms_per_step",
                                          "tasks_per_step", "transport_tasks_per_s")}, "timed_steps": k_common}
                 if fp64 and head != "fp64" else None),
        "speedup_mixed_vs_fp64": ({"per_step": fp64["common_steps_ms"] / main["common_steps_ms"],
                                   "common_steps": k_common,
                                   "per_task": main["cell_dir_updates_per_s"] / fp64["cell_dir_updates_per_s"],
                                   "transport_kernel_per_task": (main["transport_tasks_per_s"] /
                                                                 fp64["transport_tasks_per_s"]),
                                   "tasks_per_step_ratio": main["tasks_per_step"] / fp64["tasks_per_step"]}
                                  if fp64 and head != "fp64" else None),
        "error_mixed_vs_fp64": err,
        "radiation_field": field,
        "periodic_semantics_vs_reference_order": semantics,
        # the same timed steps, host wall time of sw_step + the field write-back
        "e2e": {"value": e2e_tasks / e2e_max, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 4 * 8 * n, "write_back": write_back},
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
        "clocks": main["clocks"],
        "clocks_fp64": fp64["clocks"] if fp64 and head != "fp64" else None,
        "cpu_baseline": cpu,
        "stats": {"tasks": d["tasks"], "levelled_sweeps": d["levelled_sweeps"],
                  "transport_attempts": d["transport_attempts"],
                  "pull_variant": pull_variant,
                  "sweeps": d["level_sweeps"], "schedule_levels": sched_levels,
                  "chem_attempts": d["chem_attempts"], "transport_kernel_ms": d["transport_kernel_ms"],
                  "sweep_ms": d["sweep_ms"], "chem_ms": d["chem_ms"], "level_ms": d["level_ms"],
                  "fp64_transport_kernel_ms": fp64["d"]["transport_kernel_ms"] if fp64 else None,
                  "fp64_chem_ms": fp64["d"]["chem_ms"] if fp64 else None,
                  "fp64_tasks": fp64["d"]["tasks"] if fp64 else None,
                  "task_spaces": d.get("task_spaces"), "device_bytes": d.get("device_bytes")},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["c1", "c2", "c3", "c4", "c5"], default="c4",
                    help="c5: the stress configuration, mixed path only (its FP64 state would not fit)")
    ap.add_argument("--n-per-side", type=int, default=None,
                    help="cells per side (C1, C2, C4) or boxes (C3); default the configuration's")
    ap.add_argument("--thick", action="store_true", help="C2-C4 at C1's 1 Mpc / 32 cell size")
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
