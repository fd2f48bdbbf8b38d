"""Python mirror of the reference's sweep plugin interface over the C ABI.

The reference's Rust host calls the library through `extern "C"`; this module is
the same boundary seen from Python (used by the tests and the benchmark):

* :class:`SweepParameters` mirrors ``SweepParameters`` (src/sweep/parameters.rs:8-46)
  with the same field names and serde defaults;
* :class:`Sweep` mirrors ``Sweep<HydrogenOnly>``: construction is
  ``init_sweep_system`` (src/sweep/mod.rs:634-692), :meth:`Sweep.run_sweeps` is
  ``Sweep::run_sweeps`` (258-272) and :meth:`Sweep.fields` the write-back of
  ``run_sweep_system`` (718-738).

Errors the reference would panic on raise :class:`SweepError`.
"""
from __future__ import annotations

import ctypes
import dataclasses
from typing import Optional, Sequence, Union

import numpy as np

from . import _native
from .grid import Grid

# src/units/mod.rs
PROTON_MASS = 1.67262192369e-27      # kg
YEAR = 3.15576e7                      # s
MEGAYEAR = 1e6 * YEAR
PARSEC = 3.0857e16                    # m
MEGAPARSEC = 1e6 * PARSEC
PER_CUBIC_CENTIMETER = 1.0 / 1e-6     # m^-3


def mass_density_from_number_density(n_h_per_cm3):
    """Hydrogen number density in cm^-3 -> mass density in kg/m^3."""
    return np.asarray(n_h_per_cm3, np.float64) * PER_CUBIC_CENTIMETER * PROTON_MASS


class SweepError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_native.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


@dataclasses.dataclass
class SweepParameters:
    """`sweep:` parameter section (src/sweep/parameters.rs:8-46, defaults 64-78)."""
    directions: Union[int, Sequence[Sequence[float]]]
    num_timestep_levels: int
    periodic: bool
    max_timestep: float
    rotate_directions: bool = False
    significant_rate_threshold: float = 0.0
    timestep_safety_factor: float = 0.1
    chemistry_timestep_safety_factor: float = 0.1
    check_deadlock: bool = False
    prevent_cooling: bool = True
    num_tasks_to_solve_before_send_receive: int = 10000

    def num_directions(self) -> int:
        return self.directions if isinstance(self.directions, int) else len(self.directions)


def directions_from_num(num: int) -> np.ndarray:
    """Directions::from_num (src/sweep/direction/mod.rs:58-75) as a (num, 3) array."""
    lib = _native.load_gpu()
    out = np.zeros((num, 3))
    st = lib.sw_directions_from_num(num, out.ctypes.data)
    if st != _native.SW_OK:
        raise SweepError(st, f"no direction table for {num} directions")
    return out


class Sweep:
    """One device-resident sweep (grid, per-cell species, per-(cell, dir) rates)."""

    def __init__(self, params: SweepParameters, grid: Grid, density, ionized_hydrogen_fraction,
                 temperature, source, precision: str = "fp64", scale_factor: float = 1.0,
                 device: int = -1, use_graphs: bool = False, autotune: bool = True):
        self._setup(params, precision, scale_factor, device, use_graphs, autotune)
        g, init = self._csr(grid, density, ionized_hydrogen_fraction, temperature, source)
        self._finish(self._lib.sw_create(ctypes.byref(self._p), ctypes.byref(g), ctypes.byref(init),
                                         ctypes.byref(self._hnew)), grid.num_cells)

    @classmethod
    def batch(cls, params: SweepParameters, boxes, precision: str = "fp64", scale_factor: float = 1.0,
              device: int = -1, use_graphs: bool = False, autotune: bool = True) -> "Sweep":
        """One handle over independent boxes (sw_create_batch): `boxes` holds
        (grid, density, ionized_hydrogen_fraction, temperature, source) per box; per-cell
        results are concatenated in box order."""
        self = cls.__new__(cls)
        self._setup(params, precision, scale_factor, device, use_graphs, autotune)
        parts = [self._csr(*box) for box in boxes]
        grids = (_native.SwGridCsr * len(parts))(*[g for g, _ in parts])
        inits = (_native.SwCellInit * len(parts))(*[i for _, i in parts])
        self._finish(self._lib.sw_create_batch(ctypes.byref(self._p), len(parts), grids, inits,
                                               ctypes.byref(self._hnew)), sum(b[0].num_cells for b in boxes))
        return self

    def _setup(self, params, precision, scale_factor, device, use_graphs, autotune):
        self._lib = _native.load_gpu()
        self.params = params
        self.num_directions = params.num_directions()
        self.precision = precision
        p = _native.SwParams()
        self._lib.sw_default_params(ctypes.byref(p))
        self._keep = []
        if isinstance(params.directions, int):
            p.num_directions = params.directions
        else:
            dirs = np.ascontiguousarray(params.directions, dtype=np.float64).reshape(-1, 3)
            self._keep.append(dirs)
            p.num_directions = dirs.shape[0]
            p.explicit_directions = dirs.ctypes.data_as(_native.P_double)
        p.num_timestep_levels = params.num_timestep_levels
        p.periodic = int(params.periodic)
        p.max_timestep = params.max_timestep
        p.rotate_directions = int(params.rotate_directions)
        p.significant_rate_threshold = params.significant_rate_threshold
        p.timestep_safety_factor = params.timestep_safety_factor
        p.chemistry_timestep_safety_factor = params.chemistry_timestep_safety_factor
        p.check_deadlock = int(params.check_deadlock)
        p.prevent_cooling = int(params.prevent_cooling)
        p.num_tasks_to_solve_before_send_receive = params.num_tasks_to_solve_before_send_receive
        p.scale_factor = scale_factor
        p.precision = {"fp64": _native.SW_PRECISION_FP64, "mixed": _native.SW_PRECISION_MIXED}[precision]
        p.use_graphs = int(use_graphs)
        p.autotune = int(autotune)
        p.device = device
        self._p = p
        self._hnew = ctypes.c_void_p()

    def _csr(self, grid, density, ionized_hydrogen_fraction, temperature, source):
        def arr(a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            self._keep.append(a)
            return a.ctypes.data

        n = grid.num_cells
        g = _native.SwGridCsr(
            num_cells=n, row_ptr=arr(grid.row_ptr, np.int64), nbr=arr(grid.nbr, np.int32),
            kind=arr(grid.kind, np.uint8), area=arr(grid.area, np.float64),
            normal=arr(grid.normal.reshape(-1), np.float64), volume=arr(grid.volume, np.float64),
            size=arr(grid.size, np.float64))
        init = _native.SwCellInit(
            density=arr(np.broadcast_to(density, (n,)), np.float64),
            ionized_hydrogen_fraction=arr(np.broadcast_to(ionized_hydrogen_fraction, (n,)), np.float64),
            temperature=arr(np.broadcast_to(temperature, (n,)), np.float64),
            source=arr(np.broadcast_to(source, (n,)), np.float64))
        return g, init

    def _finish(self, st, num_cells):
        self._keep = []
        if st != _native.SW_OK:
            raise SweepError(st, self._lib.sw_last_error(None).decode())
        self._h = self._hnew
        self.num_cells = num_cells

    # -- lifecycle -------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._lib.sw_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, st):
        if st != _native.SW_OK:
            raise SweepError(st, self._lib.sw_last_error(self._h).decode())

    # -- the hot path ----------------------------------------------------------
    def run_sweeps(self) -> float:
        """Sweep::run_sweeps: one full step; returns the elapsed simulation time (s)."""
        te = ctypes.c_double()
        self._check(self._lib.sw_step(self._h, ctypes.byref(te)))
        return te.value

    # -- fields ----------------------------------------------------------------
    def fields(self, out: Optional[dict] = None, photon_rate: bool = True) -> dict:
        """x_HII, T, species timestep and PhotonRate per cell (run_sweep_system write-back);
        with photon_rate=False the photon rate (a device reduction over the directions) is
        neither formed nor copied."""
        n = self.num_cells
        keys = ("ionized_hydrogen_fraction", "temperature", "timestep") + (("photon_rate",) if photon_rate else ())
        if out is None:
            out = {k: np.empty(n) for k in keys}
        self._check(self._lib.sw_get_fields(
            self._h, out["ionized_hydrogen_fraction"].ctypes.data, out["temperature"].ctypes.data,
            out["timestep"].ctypes.data, out["photon_rate"].ctypes.data if photon_rate else None))
        return out

    def cell_state(self) -> dict:
        n = self.num_cells
        cts, lvl, ion = np.empty(n), np.empty(n, np.uint8), np.empty(n)
        self._check(self._lib.sw_get_cell_state(self._h, cts.ctypes.data, lvl.ctypes.data, ion.ctypes.data))
        return {"change_timescale": cts, "level": lvl, "ionization_time": ion}

    def set_fields(self, ionized_hydrogen_fraction=None, temperature=None):
        x = None if ionized_hydrogen_fraction is None else np.ascontiguousarray(ionized_hydrogen_fraction, np.float64)
        t = None if temperature is None else np.ascontiguousarray(temperature, np.float64)
        self._check(self._lib.sw_set_fields(self._h, None if x is None else x.ctypes.data,
                                            None if t is None else t.ctypes.data))

    def level_counts(self) -> np.ndarray:
        out = np.zeros(self.params.num_timestep_levels, np.int64)
        self._check(self._lib.sw_get_level_counts(self._h, out.ctypes.data))
        return out

    def dependency_counts(self, level: int) -> np.ndarray:
        out = np.zeros((self.num_cells, self.num_directions), np.uint8)
        self._check(self._lib.sw_get_dependency_counts(self._h, level, out.ctypes.data))
        return out

    def rates(self, which=("incoming", "outgoing", "periodic")) -> dict:
        """Per-(cell, direction) incoming, outgoing and periodic rates in photons/s
        ([cell][dir]); `which` names the arrays to export."""
        shape = (self.num_cells, self.num_directions)
        out = {k: np.empty(shape) for k in which}
        self._check(self._lib.sw_get_rates(self._h, *(out[k].ctypes.data if k in out else None
                                                      for k in ("incoming", "outgoing", "periodic"))))
        return out

    def time_series(self) -> dict:
        """Global averages of the current state (the reference's time-series outputs,
        src/sweep/time_series.rs:61-155), reduced on the device."""
        s = _native.SwTimeSeries()
        self._check(self._lib.sw_get_time_series(self._h, ctypes.byref(s)))
        return {name: getattr(s, name) for name, _ in s._fields_}

    def save_state(self) -> np.ndarray:
        """Checkpoint of the evolving state as a byte array (see sw_save_state)."""
        n = ctypes.c_size_t(0)
        self._check(self._lib.sw_checkpoint_size(self._h, ctypes.byref(n)))
        buf = np.empty(n.value, np.uint8)
        self._check(self._lib.sw_save_state(self._h, buf.ctypes.data, buf.nbytes))
        return buf

    def load_state(self, buf: np.ndarray) -> None:
        """Restore a checkpoint written by save_state of a handle with the same inputs."""
        buf = np.ascontiguousarray(buf, np.uint8)
        self._check(self._lib.sw_load_state(self._h, buf.ctypes.data, buf.nbytes))

    def stats(self) -> dict:
        s = _native.SwStats()
        self._check(self._lib.sw_get_stats(self._h, ctypes.byref(s)))
        return {name: getattr(s, name) for name, _ in s._fields_}
