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

Reading the HDF5 files needs h5py, which is not installed on these machines;
`read_grid_file` raises ImportError then, and `from_connections` works on the arrays.
"""
from __future__ import annotations

import numpy as np

from .grid import Grid

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


def read_grid_file(grid_path, snapshot_path, periodic: bool, density=None) -> Grid:
    """Grid of an Arepo grid file (Id1, Id2, ConnectionType, Area, Normal) and the gas
    cells of a snapshot (PartType0/ParticleIDs, Masses, and Density unless given).
    Lengths, areas and volumes are returned as stored (code units); areas and normals
    only enter the sweep through ratios, volumes through the cell size."""
    import h5py  # not installed on these machines: ImportError

    with h5py.File(snapshot_path, "r") as f:
        gas = f["PartType0"]
        ids = gas["ParticleIDs"][...]
        mass = gas["Masses"][...]
        rho = gas["Density"][...] if density is None else np.asarray(density)
    with h5py.File(grid_path, "r") as f:
        return from_connections(ids, mass / rho, f["Id1"][...], f["Id2"][...], f["ConnectionType"][...],
                                f["Area"][...], f["Normal"][...], periodic)


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
