"""Arepo Voronoi grids as sweep CSR grids.

Restates the single-rank path of the reference's grid read-in
(src/arepo_postprocess/read_grid/mod.rs): an Arepo grid file lists every face once as
a *connection* {Id1, Id2, ConnectionType, Area, Normal}; the snapshot gives each gas
cell's unique particle id, mass and density.  `from_connections` turns those arrays
into the face-neighbour CSR that `Sweep` takes:

* ConnectionType -1 and connections with a boundary bit, or with both periodic bits,
  are dropped (`TryFrom<ConnectionTypeInt>`, mod.rs:143-163; bits 0/1: periodic /
  boundary of Id1, bits 2/3: the same for Id2).
* A connection adds one face to each cell (`add_connections`, mod.rs:340-370): Id1
  gets {area, -Normal} towards Id2, Id2 gets {area, +Normal} towards Id1.  A connection
  with a periodic bit gives LOCAL_PERIODIC faces when the sweep is periodic and BOUNDARY
  faces when it is not, else LOCAL faces (`get_particle_type`, mod.rs:309-338).  The
  reference takes each face's kind from the neighbour's bit alone, so a periodic
  connection comes out periodic (or boundary) on one side and LOCAL on the other: its
  periodic branch ends in `get_periodic_wrap_type` (`todo!()`, mod.rs:395-400), and in a
  non-periodic sweep the LOCAL side would wait for a flux the boundary side never sends.
  Here both faces of a periodic connection take the periodic kind, as the sweep's own
  grids have them (and as `sw_create`'s reciprocal-face check requires).
* Faces of a cell are kept in connection order (id1's face before id2's for one
  connection), cells in the order of the particle ids given; volume = mass / density
  and size = volume^(1/3) (`Constructor::new`, mod.rs:273-301).
* Connections whose ids are both unknown are ignored (`filter_relevant_connections`);
  a connection with exactly one unknown id is an error (the reference's single-rank
  lookup `unwrap`s it).

Arepo's face normals are not the exact bisector normals of the generators, so the
upwind graph of a direction can contain cycles; `dependency_cycles` counts the tasks
that no topological order reaches (`Sweep` would report SW_ERR_STALLED on them).

`read_grid_file` reads the grid file and the snapshot with the package's own HDF5
reader (subsweep_gb300.hdf5; no libhdf5 needed), converting Arepo's units to SI as the
reference does; `read_initial_conditions` reads the gas state the sweep starts from.
"""
from __future__ import annotations

import dataclasses
import pathlib
import re
from typing import Optional

import numpy as np

from . import bpass_table, hdf5
from .cosmology import YEAR
from .grid import Grid
from .sweep import PROTON_MASS

FACE_LOCAL, FACE_LOCAL_PERIODIC, FACE_BOUNDARY = 0, 1, 2


def connection_flags(connection_type: np.ndarray):
    """(valid, periodic1, periodic2) per connection (mod.rs:130-163)."""
    t = np.asarray(connection_type, dtype=np.int64)
    periodic1 = (t & 1) != 0
    boundary1 = (t & 2) != 0
    periodic2 = ((t >> 2) & 1) != 0
    boundary2 = ((t >> 2) & 2) != 0
    valid = (t != -1) & ~(boundary1 | boundary2 | (periodic1 & periodic2))
    return valid, periodic1, periodic2


def from_connections(unique_ids, volume, id1, id2, connection_type, area, normal, periodic: bool,
                     position=None, box_size=None) -> Grid:
    """CSR grid of the cells `unique_ids` (in that order) from a connection list.

    unique_ids: int [N] Arepo ParticleIDs of the gas cells; volume: [N] cell volumes
    (mass / density, SI); id1, id2, connection_type: int [M]; area: [M]; normal: [M, 3].
    """
    uid = np.asarray(unique_ids, dtype=np.int64)
    n = uid.shape[0]
    if n == 0:
        raise ValueError("no cells")
    order = np.argsort(uid, kind="stable")
    sorted_ids = uid[order]
    if np.any(sorted_ids[1:] == sorted_ids[:-1]):
        raise ValueError("duplicate particle ids")

    def index_of(ids):
        ids = np.asarray(ids, dtype=np.int64)
        pos = np.searchsorted(sorted_ids, ids)
        pos = np.minimum(pos, n - 1)
        known = sorted_ids[pos] == ids
        return np.where(known, order[pos], -1), known

    valid, p1, p2 = connection_flags(connection_type)
    a1, k1 = index_of(id1)
    a2, k2 = index_of(id2)
    relevant = valid & (k1 | k2)
    if np.any(relevant & ~(k1 & k2)):
        bad = int(np.flatnonzero(relevant & ~(k1 & k2))[0])
        raise ValueError(f"connection {bad} links a known cell to an unknown particle id")
    sel = np.flatnonzero(relevant)
    area = np.asarray(area, dtype=np.float64)[sel]
    nrm = np.asarray(normal, dtype=np.float64).reshape(-1, 3)[sel]
    a1, a2, p1, p2 = a1[sel], a2[sel], p1[sel], p2[sel]
    m = sel.shape[0]

    kind_c = np.full(m, FACE_LOCAL, np.uint8)
    kind_c[p1 | p2] = FACE_LOCAL_PERIODIC if periodic else FACE_BOUNDARY

    # face 2k: cell id1 -> neighbour id2 (normal -N); face 2k + 1: cell id2 -> id1 (+N)
    owner = np.empty(2 * m, np.int64)
    owner[0::2], owner[1::2] = a1, a2
    nbr = np.empty(2 * m, np.int64)
    nbr[0::2], nbr[1::2] = a2, a1
    kind = np.empty(2 * m, np.uint8)
    kind[0::2], kind[1::2] = kind_c, kind_c
    normals = np.empty((2 * m, 3))
    normals[0::2], normals[1::2] = -nrm, nrm
    areas = np.repeat(area, 2)
    by_cell = np.argsort(owner, kind="stable")  # per cell in connection order
    row_ptr = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(owner, minlength=n), out=row_ptr[1:])
    # a BOUNDARY face keeps no neighbour (sweep::grid::ParticleType::Boundary)
    nbr_sorted = nbr[by_cell]
    kind_sorted = kind[by_cell]
    nbr_sorted = np.where(kind_sorted == FACE_BOUNDARY, -1, nbr_sorted)
    vol = np.asarray(volume, dtype=np.float64)
    if vol.shape != (n,) or np.any(~(vol > 0)):
        raise ValueError("volume must be positive, one per cell")
    return Grid(row_ptr=row_ptr, nbr=nbr_sorted.astype(np.int32), kind=kind_sorted,
                area=areas[by_cell], normal=normals[by_cell], volume=vol, size=np.cbrt(vol),
                position=(np.zeros((n, 3)) if position is None else np.asarray(position, np.float64)),
                box_size=(np.zeros(3) if box_size is None else np.asarray(box_size, np.float64)),
                periodic=bool(periodic))


def read_grid_file(grid_path, snapshot_paths, periodic: bool, cosmology: Optional[hdf5.Cosmology] = None) -> Grid:
    """Grid of an Arepo grid file and the gas cells of a snapshot, in SI units.

    Follows `ReadSweepGridPlugin` and `read_grid_system`
    (src/arepo_postprocess/read_grid/mod.rs:165-195, 213-256, 402-437): the snapshot's
    PartType0/ParticleIDs (no units), PartType0/Masses and PartType0/Density (Arepo's
    units) give each cell's id and volume = mass / density; the grid file's Id1, Id2,
    ConnectionType (no units), Area and Normal (Arepo's units) give the connections.
    `snapshot_paths`: a file, a directory of `*.hdf5` files, or a list of them (read in
    order, as one set of cells).  `cosmology` converts datasets with a or h exponents
    (a file that has them and no cosmology is an error, as in the reference)."""
    units = hdf5.ArepoUnits(cosmology)
    ids = hdf5.read_dataset(snapshot_paths, "PartType0/ParticleIDs", hdf5.NONE, hdf5.IdUnits())
    mass = hdf5.read_dataset(snapshot_paths, "PartType0/Masses", hdf5.MASS, units)
    density = hdf5.read_dataset(snapshot_paths, "PartType0/Density", hdf5.DENSITY, units)
    if not (ids.shape[0] == mass.shape[0] == density.shape[0]):
        raise hdf5.H5Error(f"Different lengths of datasets: PartType0/ParticleIDs ({ids.shape[0]}), "
                           f"PartType0/Masses ({mass.shape[0]}), PartType0/Density ({density.shape[0]})")
    id1 = hdf5.read_dataset(grid_path, "Id1", hdf5.NONE, hdf5.IdUnits())
    id2 = hdf5.read_dataset(grid_path, "Id2", hdf5.NONE, hdf5.IdUnits())
    ctype = hdf5.read_dataset(grid_path, "ConnectionType", hdf5.NONE, hdf5.IdUnits())
    area = hdf5.read_dataset(grid_path, "Area", hdf5.AREA, units)
    normal = hdf5.read_dataset(grid_path, "Normal", hdf5.NONE, units)
    return from_connections(ids, mass / density, id1, id2, ctype, area, normal.reshape(-1, 3), periodic)


# src/units/mod.rs:101-104
BOLTZMANN_CONSTANT = 1.380649e-23  # J/K
GAMMA = 5.0 / 3.0
HYDROGEN_MASS_FRACTION = 0.76  # src/main.rs:214, the assumed X_H


def temperature_from_internal_energy(internal_energy, ionized_hydrogen_fraction, density):
    """Temperature::from_internal_energy_density_hydrogen_only
    (src/units/specific_impls.rs:46-60) of the energy density u * rho, as
    src/main.rs:159-166 forms it: ((u * rho) / rho) * mu * (gamma - 1) * m_p / k_B with
    mu = 1 / (x_HII + 1), evaluated left to right as there."""
    rho = np.asarray(density, np.float64)
    per_mass = (np.asarray(internal_energy, np.float64) * rho) / rho
    mu = 1.0 / (np.asarray(ionized_hydrogen_fraction, np.float64) + 1.0)
    return per_mass * mu * (GAMMA - 1.0) * PROTON_MASS / BOLTZMANN_CONSTANT


def snapshot_folders(remap_from):
    """(first, last) output folders of an earlier run: the subdirectories of `remap_from`
    with the lowest and the highest number (`get_highest_or_lowest_snapshot_dir`,
    src/arepo_postprocess/remap.rs:318-353).  Every subdirectory must be named by a
    number."""
    root = pathlib.Path(remap_from)
    if not root.is_dir():
        raise hdf5.H5Error(f"remap path {root} is not a directory")
    folders = []
    for sub in sorted(q for q in root.iterdir() if q.is_dir()):
        if not re.fullmatch(r"\+?[0-9]+", sub.name):
            raise hdf5.H5Error(f"Unexpected folder in snapshot dir: {sub}")
        folders.append((int(sub.name), sub))
    if not folders:
        raise hdf5.H5Error("No snapshot folder exists. Failed to remap")
    return min(folders, key=lambda f: f[0])[1], max(folders, key=lambda f: f[0])[1]


def remap_abundances_and_temperatures(remap_from, position, ionized_hydrogen_fraction, temperature,
                                      cosmology: Optional[hdf5.Cosmology]):
    """The reference's `remap_from` (src/arepo_postprocess/remap.rs:82-125, 380-383) on one
    rank: each cell takes the larger of its own x_HII and T and those of the nearest cell
    of an earlier run.  The earlier run's positions come from its first output folder
    (dataset `position`, with the root attributes `scale_factor` and `little_h`) and are
    scaled by (a / a_first); its x_HII and T (`ionized_hydrogen_fraction`, `temperature`)
    from its last.  The reference requires a cosmological run here (its non-cosmological
    branch panics); so does this.  Nearest means least Euclidean distance; among equally
    near cells the choice is the search tree's, as in the reference.  Returns the new
    (x_HII, T)."""
    from scipy.spatial import cKDTree

    if cosmology is None:
        raise hdf5.H5Error("remapping needs the cosmology of the run (the reference supports only cosmological runs)")
    first, last = snapshot_folders(remap_from)
    first_files, last_files = hdf5.input_files(first), hdf5.input_files(last)
    if not first_files or not last_files:
        raise hdf5.H5Error(f"no *.hdf5 files in {first if not first_files else last}")
    old_pos = hdf5.read_dataset(first_files, "position", hdf5.LENGTH).reshape(-1, 3)
    old_x = hdf5.read_dataset(last_files, "ionized_hydrogen_fraction", hdf5.NONE)
    old_t = hdf5.read_dataset(last_files, "temperature", hdf5.TEMPERATURE)
    if not (old_pos.shape[0] == old_x.shape[0] == old_t.shape[0]):
        raise hdf5.H5Error(f"remap data of different lengths: position {old_pos.shape[0]}, "
                           f"ionized_hydrogen_fraction {old_x.shape[0]}, temperature {old_t.shape[0]}")
    with hdf5.File(first_files[0]) as f:
        attrs = f.attrs
        for key in ("scale_factor", "little_h"):
            if attrs.get(key) is None:
                raise hdf5.H5Error(f"no attribute '{key}' in {first_files[0]}")
        a_first = float(attrs["scale_factor"])
    old_pos = old_pos * (cosmology.a / a_first) ** hdf5.LENGTH.length  # get_scale_factor_difference
    _, nearest = cKDTree(old_pos).query(np.asarray(position, np.float64).reshape(-1, 3), k=1)
    # Temperature / IonizedHydrogenFraction max: f64::max, which ignores a NaN
    x = np.fmax(np.asarray(ionized_hydrogen_fraction, np.float64), old_x[nearest])
    t = np.fmax(np.asarray(temperature, np.float64), old_t[nearest])
    return x, t


SOLAR_MASS = 1.988477e30  # kg, src/units/mod.rs:55


def _linear_interpolate(x1, x2, y1, y2, x):
    return y1 + (x - x1) / (x2 - x1) * (y2 - y1)


def bpass_lookup(age, metallicity, mass):
    """Ionizing photon rate (photons/s) of stars of the given age (s), metallicity and
    mass (kg) from the BPASS table (`bpass_lookup`, src/arepo_postprocess/bpass.rs:11-55):
    age (in years) and metallicity clamped into the table's range shrunk by 1.00001,
    bilinear interpolation of the per-solar-mass output in age, then metallicity, times
    the mass in solar masses.  Elementwise over arrays."""
    ages = np.asarray(bpass_table.AGE_BINS)
    mets = np.asarray(bpass_table.METALLICITY_BINS)
    table = np.asarray(bpass_table.TABLE)
    safety = 1.00001
    age_yr = np.clip(np.asarray(age, np.float64) / YEAR, ages[0] * safety, ages[-1] / safety)
    met = np.clip(np.asarray(metallicity, np.float64), mets[0] * safety, mets[-1] / safety)
    # binary_search_by_key: an exact hit at i gives i + 1, a miss its insertion point
    mi = np.searchsorted(mets, met, side="right")
    ai = np.searchsorted(ages, age_yr, side="right")
    l1 = _linear_interpolate(ages[ai - 1], ages[ai], table[ai - 1, mi - 1], table[ai, mi - 1], age_yr)
    l2 = _linear_interpolate(ages[ai - 1], ages[ai], table[ai - 1, mi], table[ai, mi], age_yr)
    per_mass = _linear_interpolate(mets[mi - 1], mets[mi], l1, l2, met)
    return per_mass * (np.asarray(mass, np.float64) / SOLAR_MASS)


def read_sources(snapshot_paths, cosmology: hdf5.Cosmology, escape_fraction: float):
    """Star particles of a snapshot as point sources (`read_sources`,
    src/arepo_postprocess/sources.rs:54-128): PartType4/Coordinates, GFM_Metallicity,
    GFM_StellarFormationTime (the scale factor of formation) and Masses in Arepo's units;
    particles with a formation scale factor that is not positive (wind particles) are
    dropped; each star's rate is `bpass_lookup` of its age (the cosmic time from its
    formation to the cosmology's scale factor) times the escape fraction.  Returns
    (positions [n, 3] in m, rates in photons/s); `grid.place_sources` or
    `source_rates` adds each to its nearest cell."""
    units = hdf5.ArepoUnits(cosmology)
    pos = hdf5.read_dataset(snapshot_paths, "PartType4/Coordinates", hdf5.LENGTH, units).reshape(-1, 3)
    met = hdf5.read_dataset(snapshot_paths, "PartType4/GFM_Metallicity", hdf5.NONE, units)
    a_form = hdf5.read_dataset(snapshot_paths, "PartType4/GFM_StellarFormationTime", hdf5.NONE, units)
    mass = hdf5.read_dataset(snapshot_paths, "PartType4/Masses", hdf5.MASS, units)
    if not (pos.shape[0] == met.shape[0] == a_form.shape[0] == mass.shape[0]):
        raise hdf5.H5Error("Different lengths of datasets: PartType4/Coordinates, GFM_Metallicity, "
                           "GFM_StellarFormationTime, Masses")
    stars = a_form > 0.0
    age = np.array([cosmology.time_difference_between_scalefactors(float(a), cosmology.a) for a in a_form[stars]])
    rates = bpass_lookup(age, met[stars], mass[stars]) * float(escape_fraction)
    return pos[stars], rates


def source_rates(cell_positions, source_positions, rates) -> np.ndarray:
    """Per-cell source rates: each source's rate added, in order, to the cell whose
    position is nearest (`set_source_terms_system`, src/source_systems.rs:48-80)."""
    from scipy.spatial import cKDTree

    out = np.zeros(np.asarray(cell_positions).reshape(-1, 3).shape[0])
    if len(rates):
        _, idx = cKDTree(np.asarray(cell_positions, np.float64).reshape(-1, 3)).query(
            np.asarray(source_positions, np.float64).reshape(-1, 3), k=1)
        np.add.at(out, idx, np.asarray(rates, np.float64))
    return out


def read_initial_conditions(snapshot_paths, initial_fraction_ionized_hydrogen: Optional[float] = None,
                            cosmology: Optional[hdf5.Cosmology] = None, remap_from=None) -> dict:
    """The gas state of an Arepo snapshot as the sweep takes it, in SI units (src/main.rs:71-235):

    * density: PartType0/Density;
    * ionized_hydrogen_fraction: `initial_fraction_ionized_hydrogen` for every cell if
      given, else 0.76 * PartType0/ElectronAbundance clamped to [1e-10, 1 - 1e-10]
      (`set_initial_ionized_fraction_from_electron_abundance_system`);
    * temperature: from PartType0/InternalEnergy and that fraction
      (`insert_missing_components_system`, `temperature_from_internal_energy`);
    * position: PartType0/Coordinates [N, 3], m;
    * with `remap_from` (an earlier run's output folder), x_HII and T raised to those of
      the nearest cell of that run (`remap_abundances_and_temperatures`).
    """
    units = hdf5.ArepoUnits(cosmology)
    density = hdf5.read_dataset(snapshot_paths, "PartType0/Density", hdf5.DENSITY, units)
    energy = hdf5.read_dataset(snapshot_paths, "PartType0/InternalEnergy", hdf5.ENERGY_PER_MASS, units)
    position = hdf5.read_dataset(snapshot_paths, "PartType0/Coordinates", hdf5.LENGTH, units).reshape(-1, 3)
    if initial_fraction_ionized_hydrogen is None:
        xe = hdf5.read_dataset(snapshot_paths, "PartType0/ElectronAbundance", hdf5.NONE, units)
        x = np.clip(HYDROGEN_MASS_FRACTION * xe, 1e-10, 1.0 - 1e-10)
    else:
        x = np.full(density.shape[0], float(initial_fraction_ionized_hydrogen))
    n = density.shape[0]
    if not (energy.shape[0] == position.shape[0] == x.shape[0] == n):
        raise hdf5.H5Error("Different lengths of datasets: PartType0/Density, InternalEnergy, Coordinates, "
                           "ElectronAbundance")
    temperature = temperature_from_internal_energy(energy, x, density)
    if remap_from is not None:
        x, temperature = remap_abundances_and_temperatures(remap_from, position, x, temperature, cosmology)
    return {"density": density, "ionized_hydrogen_fraction": x, "temperature": temperature, "position": position}


def dependency_cycles(grid: Grid, directions: np.ndarray) -> int:
    """Number of (cell, direction) tasks that no topological order of the upwind graph
    reaches (on a cycle or downstream of one), over all directions.  The dependency of
    a task is as the sweep counts it (`Sweep::init_counts`, src/sweep/mod.rs:346-386):
    LOCAL faces with n . d < 0."""
    n = grid.num_cells
    owner = np.repeat(np.arange(n), np.diff(grid.row_ptr))
    local = grid.kind == FACE_LOCAL
    stuck = 0
    for d in np.asarray(directions, dtype=np.float64).reshape(-1, 3):
        up = local & (grid.normal @ d < 0)
        src, dst = grid.nbr[up].astype(np.int64), owner[up]
        missing = np.bincount(dst, minlength=n)
        order = np.argsort(src, kind="stable")
        s_sorted, d_sorted = src[order], dst[order]
        starts = np.searchsorted(s_sorted, np.arange(n + 1))
        frontier = np.flatnonzero(missing == 0)
        reached = frontier.size
        while frontier.size:
            lens = starts[frontier + 1] - starts[frontier]
            idx = np.repeat(starts[frontier] - np.cumsum(np.concatenate(([0], lens[:-1]))), lens) + \
                np.arange(lens.sum())
            down = d_sorted[idx]
            np.subtract.at(missing, down, 1)
            cand = np.unique(down)
            frontier = cand[missing[cand] == 0]
            reached += frontier.size
        stuck += n - reached
    return int(stuck)


def read_postprocess_inputs(grid_file, snapshot_paths, cosmology: Optional[hdf5.Cosmology], periodic: bool,
                            escape_fraction: Optional[float] = None, sources=None,
                            initial_fraction_ionized_hydrogen: Optional[float] = None, remap_from=None) -> dict:
    """Everything `Sweep` takes for post-processing an Arepo run with a grid file, in the
    snapshot's cell order, as the reference's post-processing startup assembles it
    (src/main.rs:30-140): the grid (`read_grid_file`), the gas state
    (`read_initial_conditions`, with `remap_from`), and the per-cell source rates, from
    the star particles (`read_sources`, `escape_fraction` given) or from explicit
    `sources` = (positions [n, 3] in m, rates in photons/s), each on its nearest cell.
    Returns a dict with grid, density, ionized_hydrogen_fraction, temperature, source
    and position."""
    if (escape_fraction is None) == (sources is None):
        raise ValueError("give either escape_fraction (sources from the star particles) or explicit sources")
    grid = read_grid_file(grid_file, snapshot_paths, periodic, cosmology)
    ic = read_initial_conditions(snapshot_paths, initial_fraction_ionized_hydrogen, cosmology, remap_from)
    if ic["density"].shape[0] != grid.num_cells:
        raise hdf5.H5Error(f"the snapshot has {ic['density'].shape[0]} gas cells, its grid {grid.num_cells}")
    if sources is None:
        src_pos, src_rates = read_sources(snapshot_paths, cosmology, escape_fraction)
    else:
        src_pos, src_rates = (np.asarray(a, np.float64) for a in sources)
    grid = dataclasses.replace(grid, position=ic["position"])
    return {"grid": grid, "density": ic["density"], "ionized_hydrogen_fraction": ic["ionized_hydrogen_fraction"],
            "temperature": ic["temperature"], "source": source_rates(ic["position"], src_pos, src_rates),
            "position": ic["position"]}
