"""Two transport designs that the benchmark grids rule out, measured on the CPU.

Direction bundles.  A bundle task (c, B) would solve every direction of B for cell c
after the union of their upwind neighbours.  A LOCAL face whose normal n separates two
directions of B (n . d1 < 0 < n . d2) makes its neighbour upwind of c for d1 and
downwind for d2, so the union graph holds a 2-cycle on that face.  On the
jittered-lattice Voronoi grids of the benchmark (~15 faces per cell, 84 directions ~22
degrees apart) nearly every cell has such a face and the union graph has no usable
topological order, while every single direction has a complete one.

Cluster-local chunks.  Contiguous Morton chunks of cells keep most faces inside a chunk
(so a thread-block cluster owning a chunk could exchange most upwind words through
distributed shared memory), but a chunk's own upwind chains are long: the dependent
exchanges per chunk and direction grow with the chunk's edge in cells.

CPU only; `PYTHONPATH=. python tests/test_transport_alternatives.py 32` prints the
figures for a 32^3 grid.
"""
import sys

import numpy as np

from subsweep_gb300 import arepo, workloads
from subsweep_gb300.sweep import directions_from_num


def ordered_fraction(n_cells, src, dst):
    """Fraction of cells a Kahn sort of the edges src -> dst orders (the rest lie on a
    cycle or downstream of one)."""
    missing = np.bincount(dst, minlength=n_cells)
    order = np.argsort(src, kind="stable")
    s_sorted, d_sorted = src[order], dst[order]
    starts = np.searchsorted(s_sorted, np.arange(n_cells + 1))
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
    return reached / n_cells


def bundle_figures(n_per_side: int, k: int):
    """Means over the 84 bundles {d, its k - 1 nearest directions}: the fraction of LOCAL
    faces that separate two members, of cells with such a face, and of bundle tasks the
    union graph orders; and the least ordered fraction of a single direction."""
    w = workloads.c4_grf(n_per_side=n_per_side, num_sources=4, nthreads=4)
    g = w.grid
    dirs = directions_from_num(84)
    owner = np.repeat(np.arange(g.num_cells), np.diff(g.row_ptr))
    local = g.kind == arepo.FACE_LOCAL
    src, dst = g.nbr[local].astype(np.int64), owner[local]
    upwind = (g.normal[local] @ dirs.T) < 0  # [faces, directions]: the neighbour is upstream
    angle = np.arccos(np.clip(dirs @ dirs.T, -1.0, 1.0))
    np.fill_diagonal(angle, np.inf)
    sep_faces, sep_cells, ordered = [], [], []
    for d in range(dirs.shape[0]):
        members = [d] + list(np.argsort(angle[d])[:k - 1])
        up = upwind[:, members]
        separating = up.any(1) & ~up.all(1)
        sep_faces.append(separating.mean())
        sep_cells.append(np.isin(np.arange(g.num_cells), dst[separating]).mean())
        union = up.any(1)
        ordered.append(ordered_fraction(g.num_cells, src[union], dst[union]))
    single = min(ordered_fraction(g.num_cells, src[upwind[:, d]], dst[upwind[:, d]]) for d in range(dirs.shape[0]))
    return float(np.mean(sep_faces)), float(np.mean(sep_cells)), float(np.mean(ordered)), single


def ordered_depth(n_cells, src, dst, mask):
    """Kahn depth (number of levels) of the edges src -> dst between cells of `mask`."""
    keep = mask[src] & mask[dst]
    src, dst = src[keep], dst[keep]
    missing = np.bincount(dst, minlength=n_cells)
    order = np.argsort(src, kind="stable")
    s_sorted, d_sorted = src[order], dst[order]
    starts = np.searchsorted(s_sorted, np.arange(n_cells + 1))
    frontier = np.flatnonzero((missing == 0) & mask)
    levels = 0
    while frontier.size:
        lens = starts[frontier + 1] - starts[frontier]
        idx = np.repeat(starts[frontier] - np.cumsum(np.concatenate(([0], lens[:-1]))), lens) + \
            np.arange(lens.sum())
        down = d_sorted[idx]
        np.subtract.at(missing, down, 1)
        cand = np.unique(down)
        frontier = cand[missing[cand] == 0]
        levels += 1
    return levels


def chunk_figures(n_per_side: int, chunk: int, directions=(0, 20, 41, 63)):
    """For Morton chunks of `chunk` cells: the fraction of LOCAL faces inside a chunk, the
    upwind depth of the first chunk for a few directions, and of the whole grid for the
    first of them."""
    w = workloads.c4_grf(n_per_side=n_per_side, num_sources=4, nthreads=4)
    g = w.grid
    dirs = directions_from_num(84)
    owner = np.repeat(np.arange(g.num_cells), np.diff(g.row_ptr))
    local = g.kind == arepo.FACE_LOCAL
    inside = float(np.mean(owner[local] // chunk == g.nbr[local].astype(np.int64) // chunk))
    first = np.zeros(g.num_cells, bool)
    first[:chunk] = True
    everything = np.ones(g.num_cells, bool)
    depths, whole = [], None
    for k in directions:
        up = local & (g.normal @ dirs[k] < 0)
        src, dst = g.nbr[up].astype(np.int64), owner[up]
        depths.append(ordered_depth(g.num_cells, src, dst, first))
        if whole is None:
            whole = ordered_depth(g.num_cells, src, dst, everything)
    return inside, depths, whole


def test_bundles_of_neighbouring_directions_have_no_order():
    faces, cells, ordered, single = bundle_figures(12, 2)
    assert single == 1.0               # every direction alone: a complete order
    assert 0.05 < faces < 0.25         # an eighth of the faces separate the two directions
    assert cells > 0.7                 # most cells have such a face
    assert ordered < 0.02              # the union graph orders almost nothing


def test_chunks_keep_faces_but_not_short_chains():
    inside, depths, whole = chunk_figures(16, 512)
    assert inside > 0.75                 # most faces stay inside an 8^3-cell chunk
    assert min(depths) > 30              # but its chains are tens of levels deep
    assert whole > max(depths)


if __name__ == "__main__":
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 32
    for k in (2, 4):
        faces, cells, ordered, single = bundle_figures(n, k)
        print(f"{n}^3, bundles of {k}: separating faces {faces:.3f}, cells with one {cells:.3f}, "
              f"bundle tasks ordered {ordered:.4f}; single directions ordered (min) {single:.4f}")
    for chunk in (512, 4096):
        if chunk < n ** 3:
            inside, depths, whole = chunk_figures(n, chunk)
            print(f"{n}^3, Morton chunks of {chunk} cells: faces inside {inside:.3f}, chunk depth {depths} "
                  f"(whole grid {whole})")
