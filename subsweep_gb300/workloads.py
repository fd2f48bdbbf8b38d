"""Seeded synthetic workloads of the sweep benchmark configurations.

All inputs are generated here (no external dataset): periodic boxes of fixed cell
size (the box grows with the cell count), jittered-lattice or Poisson Voronoi
generators, hydrogen number densities (uniform, uncorrelated lognormal, or the
exponential of a Gaussian random field with P(k) ~ k^-2), T = 1e4 K, x_HII = 1e-10
and point sources placed on their nearest cell.

Cell size.  C1's 1 Mpc box of 32^3 cells is part of its definition.  For C2-C4 the
cell size is chosen so that a neutral cell of median density is optically thin to
moderately thick (tau = n_H sigma size of order 0.3-1, size = the radius of the sphere
of the cell's volume, as the sweep attenuates), so the sweep carries a radiation field
across many cells; at C1's 31 kpc cells the same densities give tau ~ 100-400 per cell
and the field ends at the source cells.  `thick=True` keeps that
1 Mpc / 32 cell size as a second case.

  C1  32^3, uniform n_H = 1e-3 cm^-3, one 5e48 photons/s source at the centre,
      84 directions, 1 level, max_timestep 1 Myr, threshold 1e-5 photons/s
  C2  128^3 cells of 200 pc, lognormal n_H (ln-sigma 1, mean 1e-3: median tau 0.7),
      64 sources log-uniform in 1e48..1e50 at random positions, 84 directions,
      4 levels, safety 0.1, threshold 1e-5 photons/s
  C3  256 independent periodic Poisson-point boxes of N log-uniform in 8^3..40^3
      cells of 100 pc, each with a uniform n_H log-uniform in 1e-4..1e-2 (tau
      0.06..6) and 1-4 sources log-uniform in 1e48..1e49 photons/s, 32 directions,
      2 levels, threshold 1e-5 photons/s; run as one grid (block-diagonal union),
      so one sweep launch covers every box
  C4  256^3 cells of 750 pc, n_H = exp(GRF), P(k) ~ k^-2, ln-sigma 1.5, mean 2e-4
      (median tau 0.3), 1000 sources at the densest cells with rates proportional
      to density (1e52 total), 84 directions, 4 levels, threshold 1e-5 photons/s
  C5  384^3 cells of 750 pc, C4's field with ln-sigma 2.0, 4000 sources (4e52
      total), 84 directions, 6 levels, threshold 1e-5 photons/s, 20 steps of 1 Myr
Any configuration can be scaled down (`n_per_side`) for tests.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import grid as gridmod
from .sweep import (MEGAPARSEC, MEGAYEAR, PARSEC, PER_CUBIC_CENTIMETER, PROTON_MASS, SweepParameters,
                    mass_density_from_number_density)

# cell sizes (m): C1's is fixed by its 1 Mpc / 32^3 definition, also the thick case
THICK_CELL = MEGAPARSEC / 32.0
C2_CELL = 200.0 * PARSEC
C3_CELL = 100.0 * PARSEC
C4_CELL = 750.0 * PARSEC
# photons/s: C1's and the stress configuration's stated threshold, used by every workload
THRESHOLD = 1e-5
# photoionization cross section (cm^2), for the optical depths a workload reports
SIGMA_CM2 = 2.9580524545305314e-18


@dataclasses.dataclass
class Workload:
    name: str
    params: SweepParameters
    grid: gridmod.Grid
    density: np.ndarray
    ionized_hydrogen_fraction: np.ndarray
    temperature: np.ndarray
    source: np.ndarray
    steps: int

    def describe(self) -> dict:
        return {
            "workload": self.name,
            "cells": self.grid.num_cells,
            "faces_per_cell": round(self.grid.num_faces / self.grid.num_cells, 3),
            "directions": self.params.num_directions(),
            "timestep_levels": self.params.num_timestep_levels,
            "periodic": self.params.periodic,
            "significant_rate_threshold": self.params.significant_rate_threshold,
            "optical_depth_neutral": optical_depths(self.grid, self.density / (PROTON_MASS * PER_CUBIC_CENTIMETER)),
        }


def _voronoi(pts: np.ndarray, box: float, nthreads: int, grid_device: str, voronoi=None) -> gridmod.Grid:
    """Periodic Voronoi grid of the generators on the host (`nthreads` threads) or on
    a GPU (`grid_device="gpu"` or `"gpu:<index>"`, same topology, geometry equal to
    rounding); `voronoi(points, box) -> Grid`, when given, builds it instead."""
    if voronoi is not None:
        return voronoi(pts, box)
    if grid_device.startswith("gpu"):
        index = int(grid_device.split(":")[1]) if ":" in grid_device else 0
        return gridmod.voronoi_gpu(pts, box, periodic=True, device=index)
    return gridmod.voronoi(pts, box, periodic=True, nthreads=nthreads)


def _cell(thick: bool, cell_size: float) -> float:
    return THICK_CELL if thick else cell_size


def optical_depths(grid: gridmod.Grid, n_h_per_cm3: np.ndarray) -> dict:
    """Optical depth of each cell when neutral, tau = n_H sigma size (cell size =
    volume^(1/3), as the sweep attenuates): median, mean and 90th percentile."""
    tau = np.asarray(n_h_per_cm3) * SIGMA_CM2 * (grid.size * 100.0)
    return {"median": float(np.median(tau)), "mean": float(tau.mean()), "p90": float(np.percentile(tau, 90))}


def label(name: str, n_per_side: int | None = None, num_directions: int | None = None,
          num_levels: int | None = None, thick: bool = False) -> str:
    """The name a workload carries (`Workload.name`), from its parameters alone: the
    CPU reference arm of the benchmark names the full-size workload it samples without
    building it.  `n_per_side` is the cells per side (C1, C2, C4) or the number of boxes
    (C3); None takes the workload's default; `thick` names the 1 Mpc / 32 cell size."""
    if name == "c1":
        n, d = n_per_side or 32, num_directions or 84
        return f"C1 periodic jittered-lattice Voronoi {n}^3, {d} dirs, 1 level"
    if name == "c2":
        n, d, lv = n_per_side or 128, num_directions or 84, num_levels or 4
        return f"C2 periodic jittered-lattice Voronoi {n}^3 lognormal{_cells(thick, C2_CELL)}, {d} dirs, {lv} levels"
    if name == "c3":
        return _c3_label(n_per_side or 256, 512, 64000, num_directions or 32, num_levels or 2, thick)
    if name == "c4":
        n, d, lv = n_per_side or 256, num_directions or 84, num_levels or 4
        return f"C4 periodic jittered-lattice Voronoi {n}^3 GRF{_cells(thick, C4_CELL)}, {d} dirs, {lv} levels"
    if name == "c5":
        n, d, lv = n_per_side or 384, num_directions or 84, num_levels or 6
        return (f"C5 periodic jittered-lattice Voronoi {n}^3 GRF ln-sigma 2.0{_cells(thick, C4_CELL)}, {d} dirs, "
                f"{lv} levels")
    raise ValueError(f"unknown workload {name}")


def _cells(thick: bool, cell_size: float) -> str:
    return f" ({_cell(thick, cell_size) / PARSEC:.0f} pc cells)"


def _c3_label(num_boxes: int, min_cells: int, max_cells: int, num_directions: int, num_levels: int,
              thick: bool = False) -> str:
    return (f"C3 {num_boxes} periodic Poisson Voronoi boxes of {min_cells}..{max_cells} cells"
            f"{_cells(thick, C3_CELL)}, {num_directions} dirs, {num_levels} levels")


def c1_small_periodic(n_per_side: int = 32, seed: int = 1, num_directions: int = 84,
                      nthreads: int = 0, grid_device: str = "host", voronoi=None) -> Workload:
    box = THICK_CELL * n_per_side
    pts = gridmod.jittered_lattice(n_per_side, box, 0.25, seed)
    g = _voronoi(pts, box, nthreads, grid_device, voronoi)
    n = g.num_cells
    src = gridmod.place_sources(g, np.array([[box / 2, box / 2, box / 2]]), np.array([5e48]))
    params = SweepParameters(directions=num_directions, num_timestep_levels=1, periodic=True,
                             max_timestep=1.0 * MEGAYEAR, significant_rate_threshold=THRESHOLD)
    return Workload(label("c1", n_per_side, num_directions), params, g,
                    np.full(n, float(mass_density_from_number_density(1e-3))), np.full(n, 1e-10),
                    np.full(n, 1e4), src, steps=10)


def c2_lognormal(n_per_side: int = 128, seed: int = 2, num_directions: int = 84, num_levels: int = 4,
                 nthreads: int = 0, grid_device: str = "host", thick: bool = False, voronoi=None) -> Workload:
    box = _cell(thick, C2_CELL) * n_per_side
    rng = np.random.default_rng(seed)
    pts = gridmod.jittered_lattice(n_per_side, box, 0.25, seed)
    g = _voronoi(pts, box, nthreads, grid_device, voronoi)
    n = g.num_cells
    sigma = 1.0
    n_h = 1e-3 * np.exp(sigma * rng.standard_normal(n) - 0.5 * sigma * sigma)
    pos = rng.uniform(0.0, box, size=(64, 3))
    rates = 10.0 ** rng.uniform(48.0, 50.0, size=64)
    src = gridmod.place_sources(g, pos, rates)
    params = SweepParameters(directions=num_directions, num_timestep_levels=num_levels, periodic=True,
                             max_timestep=1.0 * MEGAYEAR, timestep_safety_factor=0.1,
                             significant_rate_threshold=THRESHOLD)
    return Workload(label("c2", n_per_side, num_directions, num_levels, thick), params, g,
                    mass_density_from_number_density(n_h), np.full(n, 1e-10),
                    np.full(n, 1e4), src, steps=4)


def c3_box(rng: np.random.Generator, seed: int, min_cells: int = 512, max_cells: int = 64000,
           nthreads: int = 0, thick: bool = False, voronoi=None):
    """One box of the C3 batch: (grid, n_H per cell, source per cell)."""
    n = int(round(np.exp(rng.uniform(np.log(min_cells), np.log(max_cells)))))
    box = _cell(thick, C3_CELL) * n ** (1.0 / 3.0)
    g = _voronoi(gridmod.poisson_points(n, box, seed), box, nthreads, "host", voronoi)
    n_h = np.full(g.num_cells, 10.0 ** rng.uniform(-4.0, -2.0))
    k = int(rng.integers(1, 5))
    src = gridmod.place_sources(g, rng.uniform(0.0, box, size=(k, 3)), 10.0 ** rng.uniform(48.0, 49.0, size=k))
    return g, n_h, src


def c3_batched(num_boxes: int = 256, seed: int = 3, min_cells: int = 512, max_cells: int = 64000,
               num_directions: int = 32, num_levels: int = 2, nthreads: int = 0, boxes=None,
               thick: bool = False, voronoi=None) -> Workload:
    """C3: independent boxes run as one block-diagonal grid.  `boxes` may pass
    precomputed (grid, n_H, source) triples."""
    rng = np.random.default_rng(seed)
    if boxes is None:
        boxes = [c3_box(rng, seed * 100003 + b, min_cells, max_cells, nthreads, thick, voronoi)
                 for b in range(num_boxes)]
    g = gridmod.concatenate([b[0] for b in boxes])
    n_h = np.concatenate([b[1] for b in boxes])
    src = np.concatenate([b[2] for b in boxes])
    n = g.num_cells
    params = SweepParameters(directions=num_directions, num_timestep_levels=num_levels, periodic=True,
                             max_timestep=1.0 * MEGAYEAR, timestep_safety_factor=0.1,
                             significant_rate_threshold=THRESHOLD)
    return Workload(_c3_label(len(boxes), min_cells, max_cells, num_directions, num_levels, thick), params, g,
                    mass_density_from_number_density(n_h), np.full(n, 1e-10), np.full(n, 1e4), src, steps=4)


def gaussian_random_field(m: int, ln_sigma: float, seed: int) -> np.ndarray:
    """Gaussian random field on an m^3 lattice with P(k) ~ k^-2, unit-normalised to
    standard deviation ln_sigma (the field whose exponential gives the density)."""
    rng = np.random.default_rng(seed)
    white = rng.standard_normal((m, m, m))
    k = np.fft.fftfreq(m)
    kz = np.fft.rfftfreq(m)
    k2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + kz[None, None, :] ** 2
    amp = np.zeros_like(k2)
    amp[k2 > 0] = 1.0 / np.sqrt(k2[k2 > 0])  # sqrt(P) with P ~ k^-2
    field = np.fft.irfftn(np.fft.rfftn(white) * amp, s=(m, m, m), axes=(0, 1, 2))
    field -= field.mean()
    return field * (ln_sigma / field.std())


def c4_grf(n_per_side: int = 256, seed: int = 4, ln_sigma: float = 1.5, num_sources: int = 1000,
           num_directions: int = 84, num_levels: int = 4, nthreads: int = 0, grid_device: str = "host",
           thick: bool = False, voronoi=None, total_rate: float = 1e52, steps: int = 4,
           name: str = "c4") -> Workload:
    box = _cell(thick, C4_CELL) * n_per_side
    pts = gridmod.jittered_lattice(n_per_side, box, 0.25, seed)
    g = _voronoi(pts, box, nthreads, grid_device, voronoi)
    n = g.num_cells
    field = gaussian_random_field(n_per_side, ln_sigma, seed)
    ijk = np.minimum((g.position / box * n_per_side).astype(np.int64), n_per_side - 1)
    ln_n = field[ijk[:, 0], ijk[:, 1], ijk[:, 2]]
    n_h = np.exp(ln_n)
    n_h *= 2e-4 / n_h.mean()
    peaks = np.argsort(n_h)[-num_sources:]
    src = np.zeros(n)
    src[peaks] = n_h[peaks] / n_h[peaks].sum() * total_rate
    params = SweepParameters(directions=num_directions, num_timestep_levels=num_levels, periodic=True,
                             max_timestep=1.0 * MEGAYEAR, significant_rate_threshold=THRESHOLD)
    return Workload(label(name, n_per_side, num_directions, num_levels, thick), params, g,
                    mass_density_from_number_density(n_h), np.full(n, 1e-10),
                    np.full(n, 1e4), src, steps=steps)


def c5_grf(n_per_side: int = 384, seed: int = 5, num_directions: int = 84, num_levels: int = 6,
           nthreads: int = 0, grid_device: str = "host", thick: bool = False, voronoi=None) -> Workload:
    """C5, the stress configuration: C4's generator (750 pc cells, exp of a Gaussian random
    field with P(k) ~ k^-2, mean n_H 2e-4 cm^-3, sources at the density peaks with rates
    proportional to the local density) at 384^3 with ln-sigma 2.0, 4000 sources (their
    total scaled with the count from C4's 1e52 photons/s for 1000), 84 directions, 6
    levels, threshold 1e-5 photons/s, 20 steps of 1 Myr (final time 20 Myr).  Its 4.76 G
    tasks exceed 32-bit task ids: the mixed path runs it in the compact state."""
    return c4_grf(n_per_side=n_per_side, seed=seed, ln_sigma=2.0, num_sources=4000, num_directions=num_directions,
                  num_levels=num_levels, nthreads=nthreads, grid_device=grid_device, thick=thick, voronoi=voronoi,
                  total_rate=4e52, steps=20, name="c5")


def cartesian_column(n: int, cell_size: float, n_h: float, source_rate: float, num_levels: int = 1,
                     max_timestep: float = 1.0 * MEGAYEAR) -> Workload:
    """1-D column along x (n x 1 x 1 cartesian cells, non-periodic, 1 direction (1,0,0)):
    the setting of the reference's examples/sweep_1d.rs."""
    g = gridmod.cartesian(n, 1, 1, cell_size, periodic=False)
    src = np.zeros(n)
    src[0] = source_rate
    params = SweepParameters(directions=1, num_timestep_levels=num_levels, periodic=False,
                             max_timestep=max_timestep)
    return Workload(f"cartesian column {n}", params, g,
                    np.full(n, float(mass_density_from_number_density(n_h))), np.full(n, 1e-10),
                    np.full(n, 1e4), src, steps=1)
