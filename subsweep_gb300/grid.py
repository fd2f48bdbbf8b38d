"""Face-neighbour CSR grids for the sweep, built on the host.

The sweep library takes any grid as CSR (row_ptr, neighbour, kind, area, normal,
volume, size).  This module wraps the native producers in csrc/grid_host.cpp:
Voronoi tessellations of generator points (periodic or bounded box) and the
reference's cartesian test grid (src/sweep/grid/cartesian.rs), and places point
sources on their nearest cell as src/source_systems.rs:48-80 does.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import _native


@dataclasses.dataclass
class Grid:
    row_ptr: np.ndarray   # int64 [N+1]
    nbr: np.ndarray       # int32 [E]
    kind: np.ndarray      # uint8 [E]
    area: np.ndarray      # float64 [E]
    normal: np.ndarray    # float64 [E, 3]
    volume: np.ndarray    # float64 [N]
    size: np.ndarray      # float64 [N]
    position: np.ndarray  # float64 [N, 3] generator positions
    box_size: np.ndarray  # float64 [3]
    periodic: bool

    @property
    def num_cells(self) -> int:
        return int(self.row_ptr.shape[0] - 1)

    @property
    def num_faces(self) -> int:
        return int(self.nbr.shape[0])

    def faces_per_cell(self) -> np.ndarray:
        return np.diff(self.row_ptr)


def _from_handle(lib, h, box_size, periodic) -> Grid:
    if not h:
        raise RuntimeError("grid construction failed")
    try:
        failed = lib.sw_grid_failed_cells(h)
        if failed:
            raise RuntimeError(f"Voronoi construction failed for {failed} cells")
        n = lib.sw_grid_num_cells(h)
        e = lib.sw_grid_num_faces(h)
        g = Grid(
            row_ptr=np.zeros(n + 1, np.int64), nbr=np.zeros(e, np.int32), kind=np.zeros(e, np.uint8),
            area=np.zeros(e), normal=np.zeros((e, 3)), volume=np.zeros(n), size=np.zeros(n),
            position=np.zeros((n, 3)), box_size=np.asarray(box_size, np.float64), periodic=bool(periodic))
        lib.sw_grid_copy(h, g.row_ptr.ctypes.data, g.nbr.ctypes.data, g.kind.ctypes.data, g.area.ctypes.data,
                         g.normal.ctypes.data, g.volume.ctypes.data, g.size.ctypes.data, g.position.ctypes.data)
        return g
    finally:
        lib.sw_grid_free(h)


def voronoi(points: np.ndarray, box_size, periodic: bool = True, nthreads: int = 0) -> Grid:
    """Voronoi grid of `points` (N x 3, inside [0, box)) in a periodic or walled box."""
    lib = _native.load_grid()
    pts = np.ascontiguousarray(points, dtype=np.float64)
    box = np.ascontiguousarray(np.broadcast_to(np.asarray(box_size, np.float64), (3,)))
    h = lib.sw_grid_voronoi(pts.ctypes.data, pts.shape[0], box.ctypes.data, int(periodic), int(nthreads))
    return _from_handle(lib, h, box, periodic)


def voronoi_gpu(points: np.ndarray, box_size, periodic: bool = True, device: int = 0) -> Grid:
    """Voronoi grid of `points` built on the GPU (csrc/voronoi_gpu.cu), one thread per
    cell: the CSR conventions of `voronoi`, the same faces and neighbours; areas and
    volumes equal to rounding (the clipping order can differ in its last bits)."""
    lib = _native.load_gpu()
    pts = np.ascontiguousarray(points, dtype=np.float64)
    box = np.ascontiguousarray(np.broadcast_to(np.asarray(box_size, np.float64), (3,)))
    n = pts.shape[0]
    h = lib.sw_gpu_grid_voronoi(pts.ctypes.data, n, box.ctypes.data, int(periodic), int(device))
    if not h:
        raise RuntimeError("GPU grid construction rejected its arguments")
    try:
        st = lib.sw_gpu_grid_status(h)
        if st:
            raise RuntimeError(f"GPU grid construction failed with CUDA error {st}")
        failed = lib.sw_gpu_grid_failed_cells(h)
        if failed:
            raise RuntimeError(f"Voronoi construction failed for {failed} cells")
        e = lib.sw_gpu_grid_num_faces(h)
        g = Grid(
            row_ptr=np.zeros(n + 1, np.int64), nbr=np.zeros(e, np.int32), kind=np.zeros(e, np.uint8),
            area=np.zeros(e), normal=np.zeros((e, 3)), volume=np.zeros(n), size=np.zeros(n),
            position=pts.copy(), box_size=box.copy(), periodic=bool(periodic))
        lib.sw_gpu_grid_copy(h, g.row_ptr.ctypes.data, g.nbr.ctypes.data, g.kind.ctypes.data, g.area.ctypes.data,
                             g.normal.ctypes.data, g.volume.ctypes.data, g.size.ctypes.data)
        return g
    finally:
        lib.sw_gpu_grid_free(h)


def cartesian(nx: int, ny: int, nz: int, cell_size: float, periodic: bool) -> Grid:
    """The reference's cartesian grid (cartesian.rs:220-395) for one rank."""
    lib = _native.load_grid()
    h = lib.sw_grid_cartesian(nx, ny, nz, float(cell_size), int(periodic))
    return _from_handle(lib, h, np.array([nx, ny, nz], np.float64) * cell_size, periodic)


def _part1by2(v: np.ndarray) -> np.ndarray:
    v = v.astype(np.uint64) & np.uint64(0x1FFFFF)
    v = (v | (v << np.uint64(32))) & np.uint64(0x1F00000000FFFF)
    v = (v | (v << np.uint64(16))) & np.uint64(0x1F0000FF0000FF)
    v = (v | (v << np.uint64(8))) & np.uint64(0x100F00F00F00F00F)
    v = (v | (v << np.uint64(4))) & np.uint64(0x10C30C30C30C30C3)
    v = (v | (v << np.uint64(2))) & np.uint64(0x1249249249249249)
    return v


def morton_order(ijk: np.ndarray) -> np.ndarray:
    """Permutation sorting integer coordinates along a Morton (Z-order) curve."""
    code = _part1by2(ijk[:, 0]) | (_part1by2(ijk[:, 1]) << np.uint64(1)) | (_part1by2(ijk[:, 2]) << np.uint64(2))
    return np.argsort(code, kind="stable")


def jittered_lattice(n_per_side: int, box: float, jitter: float = 0.25, seed: int = 1) -> np.ndarray:
    """Cubic lattice of n^3 generators at cell centres with uniform jitter of +-jitter
    spacings, ordered along a Morton curve so that neighbouring cells have nearby ids."""
    rng = np.random.default_rng(seed)
    m = n_per_side
    ijk = np.stack(np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij"), -1).reshape(-1, 3)
    ijk = ijk[morton_order(ijk)]
    pts = (ijk + 0.5 + rng.uniform(-jitter, jitter, size=ijk.shape)) * (box / m)
    return np.mod(pts, box)


def poisson_points(n: int, box: float, seed: int) -> np.ndarray:
    """n uniform random generators in [0, box)^3, Morton-ordered by bucket."""
    rng = np.random.default_rng(seed)
    pts = rng.uniform(0.0, box, size=(n, 3))
    b = max(1, int(round(n ** (1.0 / 3.0))))
    ijk = np.minimum((pts / box * b).astype(np.int64), b - 1)
    return pts[morton_order(ijk)]


def concatenate(grids: list) -> Grid:
    """Block-diagonal union of independent grids: one CSR whose components never share a
    face (LOCAL and LOCAL_PERIODIC neighbour ids are offset into each grid's own cell
    range; boundary faces keep their id).  A sweep over the union computes, for every
    component, what a sweep over that grid alone computes.  Generator positions are
    shifted along x so the components do not overlap in space."""
    offsets = np.cumsum([0] + [g.num_cells for g in grids])
    face_offsets = np.cumsum([0] + [g.num_faces for g in grids])
    row_ptr = np.concatenate([g.row_ptr[:-1] + fo for g, fo in zip(grids, face_offsets[:-1])] +
                             [np.array([face_offsets[-1]], np.int64)]).astype(np.int64)
    nbr = np.concatenate([np.where(g.kind <= 1, g.nbr + np.int32(o), g.nbr) for g, o in zip(grids, offsets[:-1])])
    shift = np.cumsum([0.0] + [float(g.box_size[0]) for g in grids])
    position = np.concatenate([g.position + np.array([sx, 0.0, 0.0]) for g, sx in zip(grids, shift[:-1])])
    return Grid(row_ptr=row_ptr, nbr=nbr.astype(np.int32), kind=np.concatenate([g.kind for g in grids]),
                area=np.concatenate([g.area for g in grids]), normal=np.concatenate([g.normal for g in grids]),
                volume=np.concatenate([g.volume for g in grids]), size=np.concatenate([g.size for g in grids]),
                position=position, box_size=np.array([shift[-1], max(float(g.box_size[1]) for g in grids),
                                                      max(float(g.box_size[2]) for g in grids)]),
                periodic=all(g.periodic for g in grids))


def nearest_cells(grid: Grid, positions: np.ndarray) -> np.ndarray:
    """Index of the cell whose generator is nearest to each position (Euclidean, not
    periodic, like the kd-tree lookup of src/source_systems.rs:61-72)."""
    from scipy.spatial import cKDTree

    tree = cKDTree(grid.position)
    _, idx = tree.query(np.atleast_2d(positions))
    return np.asarray(idx, dtype=np.int64)


def place_sources(grid: Grid, positions: np.ndarray, rates: np.ndarray) -> np.ndarray:
    """Per-cell source rates: each point source's rate added to its nearest cell."""
    src = np.zeros(grid.num_cells)
    np.add.at(src, nearest_cells(grid, positions), np.asarray(rates, np.float64))
    return src
