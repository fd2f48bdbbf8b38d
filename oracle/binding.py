"""ctypes binding of the CPU FP64 oracle (oracle/sweep_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB = HERE / "build" / "liboracle.so"

c_int32, c_int64, c_double, c_void_p = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p

PERIODIC_SNAPSHOT = 0
PERIODIC_IMMEDIATE = 1
ORDER_FIFO = 0
ORDER_HEAP = 1
PARTITION_DIRECTIONS = 0
PARTITION_DOMAINS = 1


class OrcGrid(ctypes.Structure):
    _fields_ = [("num_cells", c_int64), ("row_ptr", c_void_p), ("nbr", c_void_p), ("kind", c_void_p),
                ("area", c_void_p), ("normal", c_void_p), ("volume", c_void_p), ("size", c_void_p)]


class OrcParams(ctypes.Structure):
    _fields_ = [("num_directions", c_int32), ("directions", c_void_p), ("num_timestep_levels", c_int32),
                ("max_timestep", c_double), ("significant_rate_threshold", c_double),
                ("timestep_safety_factor", c_double), ("chemistry_timestep_safety_factor", c_double),
                ("prevent_cooling", c_int32), ("scale_factor", c_double), ("periodic_mode", c_int32),
                ("order", c_int32), ("num_threads", c_int32), ("partition", c_int32)]


# names of the reference's time-series outputs (src/sweep/time_series.rs:26-48)
TIME_SERIES_NAMES = ("hydrogen_ionization_mass_average", "hydrogen_ionization_volume_average",
                     "temperature_mass_average", "temperature_volume_average",
                     "photoionization_rate_volume_average", "weighted_photoionization_rate_volume_average")


def build() -> pathlib.Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        build()
    lib = ctypes.CDLL(str(LIB))
    lib.orc_sim_create.restype = c_void_p
    lib.orc_sim_create.argtypes = [ctypes.POINTER(OrcParams), ctypes.POINTER(OrcGrid)] + [c_void_p] * 4
    lib.orc_sim_destroy.argtypes = [c_void_p]
    lib.orc_sim_step.argtypes = [c_void_p, ctypes.POINTER(c_double)]
    lib.orc_sim_step.restype = ctypes.c_int
    lib.orc_sim_get_fields.argtypes = [c_void_p] + [c_void_p] * 6
    lib.orc_sim_get_rates.argtypes = [c_void_p] + [c_void_p] * 3
    lib.orc_sim_time_series.argtypes = [c_void_p, c_void_p]
    lib.orc_sim_init_counts.argtypes = [c_void_p, c_int32, c_void_p]
    lib.orc_sim_init_counts.restype = c_int64
    lib.orc_sim_level_counts.argtypes = [c_void_p, c_void_p]
    lib.orc_sim_work.argtypes = [c_void_p, c_void_p, c_void_p]
    lib.orc_sim_sweep_order.argtypes = [c_void_p, c_void_p, c_int32]
    lib.orc_sim_sweep_order.restype = c_int32
    lib.orc_sim_single_sweep.argtypes = [c_void_p, c_int32]
    lib.orc_sim_single_sweep.restype = c_int64
    lib.orc_sim_sample_sweep.argtypes = [c_void_p, c_int32, c_int32, c_int32, c_int64, ctypes.POINTER(c_int64)]
    lib.orc_sim_sample_sweep.restype = c_int64
    lib.orc_timestep_level.argtypes = [c_int32, c_double, c_double]
    lib.orc_timestep_level.restype = c_int32
    lib.orc_sweep_order_after.argtypes = [c_int32, c_int32, c_void_p, c_int32]
    lib.orc_sweep_order_after.restype = c_int32
    lib.orc_lowest_allowed_after.argtypes = [c_int32, c_int32]
    lib.orc_lowest_allowed_after.restype = c_int32
    lib.orc_rate_fit.argtypes = [c_int32, c_double, c_double]
    lib.orc_rate_fit.restype = c_double
    lib.orc_solver_perform_timestep.argtypes = [ctypes.POINTER(c_double), ctypes.POINTER(c_double)] + \
        [c_double] * 5 + [c_int32, c_double, c_double, c_double, c_double, ctypes.POINTER(c_double),
                          ctypes.POINTER(c_int32)]
    lib.orc_solver_perform_timestep.restype = c_int32
    lib.orc_voronoi_build.restype = c_void_p
    lib.orc_voronoi_build.argtypes = [c_void_p, c_int64, c_double, c_int32]
    for name in ("orc_voronoi_num_faces", "orc_voronoi_failed_cells", "orc_voronoi_dropped_faces"):
        getattr(lib, name).restype = c_int64
        getattr(lib, name).argtypes = [c_void_p]
    lib.orc_voronoi_copy.argtypes = [c_void_p] * 8
    lib.orc_voronoi_free.argtypes = [c_void_p]
    lib.orc_directions_from_num.argtypes = [c_int32, c_void_p]
    lib.orc_directions_from_num.restype = c_int32
    lib.orc_heap_replay.argtypes = [c_void_p, c_int64, c_void_p, c_int64, c_void_p]
    lib.orc_heap_replay.restype = c_int64
    lib.orc_outgoing_rate.argtypes = [c_double] * 5
    lib.orc_outgoing_rate.restype = c_double
    _lib = lib
    return lib


def directions_from_num(num: int) -> np.ndarray:
    """The reference's direction table for `num` directions (Directions::from_num)."""
    out = np.zeros((num, 3))
    if load().orc_directions_from_num(num, out.ctypes.data) != 0:
        raise ValueError(f"no direction table for {num} directions")
    return out


def voronoi(points: np.ndarray, box: float, num_threads: int = 1) -> dict:
    """Periodic Voronoi tessellation of `points` in [0, box)^3 by the oracle's own
    producer (voronoi_oracle.cpp): the CSR arrays as a dict (the fields of a sweep
    grid) plus the counts of failed cells and dropped one-sided faces."""
    lib = load()
    pts = np.ascontiguousarray(points, dtype=np.float64)
    n = pts.shape[0]
    h = lib.orc_voronoi_build(pts.ctypes.data, n, float(box), int(num_threads))
    if not h:
        raise ValueError("invalid Voronoi arguments")
    try:
        e = lib.orc_voronoi_num_faces(h)
        g = {"row_ptr": np.zeros(n + 1, np.int64), "nbr": np.zeros(e, np.int32), "kind": np.zeros(e, np.uint8),
             "area": np.zeros(e), "normal": np.zeros((e, 3)), "volume": np.zeros(n), "size": np.zeros(n)}
        lib.orc_voronoi_copy(h, *(g[k].ctypes.data for k in ("row_ptr", "nbr", "kind", "area", "normal",
                                                              "volume", "size")))
        g["failed_cells"] = lib.orc_voronoi_failed_cells(h)
        g["dropped_faces"] = lib.orc_voronoi_dropped_faces(h)
        return g
    finally:
        lib.orc_voronoi_free(h)


class OracleSweep:
    """The oracle's Sweep<HydrogenOnly>, built from the same inputs as subsweep_gb300.Sweep."""

    def __init__(self, params, grid, density, xhii, temperature, source, directions: np.ndarray,
                 scale_factor: float = 1.0, periodic_mode: int = PERIODIC_SNAPSHOT, order: int = ORDER_FIFO,
                 num_threads: int = 1, partition: int = PARTITION_DIRECTIONS):
        lib = load()
        self._lib = lib
        n = grid.num_cells
        self.num_cells = n
        self.num_directions = directions.shape[0]
        self.num_levels = params.num_timestep_levels
        keep = []

        def arr(a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return a.ctypes.data

        self._dirs = np.ascontiguousarray(directions, dtype=np.float64)
        p = OrcParams(num_directions=self._dirs.shape[0], directions=self._dirs.ctypes.data,
                      num_timestep_levels=params.num_timestep_levels, max_timestep=params.max_timestep,
                      significant_rate_threshold=params.significant_rate_threshold,
                      timestep_safety_factor=params.timestep_safety_factor,
                      chemistry_timestep_safety_factor=params.chemistry_timestep_safety_factor,
                      prevent_cooling=int(params.prevent_cooling), scale_factor=scale_factor,
                      periodic_mode=periodic_mode, order=order, num_threads=num_threads,
                      partition=partition)
        g = OrcGrid(num_cells=n, row_ptr=arr(grid.row_ptr, np.int64), nbr=arr(grid.nbr, np.int32),
                    kind=arr(grid.kind, np.uint8), area=arr(grid.area, np.float64),
                    normal=arr(grid.normal.reshape(-1), np.float64), volume=arr(grid.volume, np.float64),
                    size=arr(grid.size, np.float64))
        self._h = lib.orc_sim_create(ctypes.byref(p), ctypes.byref(g),
                                     arr(np.broadcast_to(density, (n,)), np.float64),
                                     arr(np.broadcast_to(xhii, (n,)), np.float64),
                                     arr(np.broadcast_to(temperature, (n,)), np.float64),
                                     arr(np.broadcast_to(source, (n,)), np.float64))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.orc_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def run_sweeps(self) -> float:
        te = c_double()
        st = self._lib.orc_sim_step(self._h, ctypes.byref(te))
        if st != 0:
            raise RuntimeError(f"oracle step failed with status {st}")
        return te.value

    def fields(self) -> dict:
        n = self.num_cells
        out = {k: np.empty(n) for k in ("ionized_hydrogen_fraction", "temperature", "timestep", "photon_rate",
                                        "change_timescale")}
        lvl = np.empty(n, np.uint8)
        self._lib.orc_sim_get_fields(self._h, out["ionized_hydrogen_fraction"].ctypes.data,
                                     out["temperature"].ctypes.data, out["timestep"].ctypes.data,
                                     out["photon_rate"].ctypes.data, out["change_timescale"].ctypes.data,
                                     lvl.ctypes.data)
        out["level"] = lvl
        return out

    def rates(self) -> dict:
        shape = (self.num_cells, self.num_directions)
        inc, outg, per = np.empty(shape), np.empty(shape), np.empty(shape)
        self._lib.orc_sim_get_rates(self._h, inc.ctypes.data, outg.ctypes.data, per.ctypes.data)
        return {"incoming": inc, "outgoing": outg, "periodic": per}

    def time_series(self) -> dict:
        out = np.empty(6)
        self._lib.orc_sim_time_series(self._h, out.ctypes.data)
        return dict(zip(TIME_SERIES_NAMES, (float(v) for v in out)))

    def dependency_counts(self, level: int) -> np.ndarray:
        out = np.zeros((self.num_cells, self.num_directions), np.uint8)
        self._lib.orc_sim_init_counts(self._h, level, out.ctypes.data)
        return out

    def level_counts(self) -> np.ndarray:
        out = np.zeros(self.num_levels, np.int64)
        self._lib.orc_sim_level_counts(self._h, out.ctypes.data)
        return out

    def work(self) -> tuple:
        t, c = c_int64(), c_int64()
        self._lib.orc_sim_work(self._h, ctypes.byref(t), ctypes.byref(c))
        return t.value, c.value

    def single_sweep(self, level: int) -> int:
        return self._lib.orc_sim_single_sweep(self._h, level)

    def sample_sweep(self, level: int, dir_first: int, dir_count: int, chem_first: int) -> tuple:
        """(tasks, chemistry updates) of a bounded sample of one level sweep."""
        chem = c_int64()
        tasks = self._lib.orc_sim_sample_sweep(self._h, level, dir_first, dir_count, chem_first, ctypes.byref(chem))
        if tasks < 0:
            raise ValueError("invalid sample")
        return tasks, chem.value
