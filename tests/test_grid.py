"""Host grid producers: Voronoi geometry against scipy and the reference's Voronoi KAT,
and the cartesian grid's conventions."""
import numpy as np
import pytest

from subsweep_gb300 import grid as gridmod


def test_voronoi_reference_kat(kats):
    """right_volume_and_face_areas_three_d (src/voronoi/mod.rs:191-244), points shifted
    into a large walled box so that no wall touches the tested cell."""
    k = kats["voronoi_kat"]
    pts = np.array(k["points"]) + 1.0
    g = gridmod.voronoi(pts, 3.0, periodic=False, nthreads=1)
    c = k["cell"]
    assert g.volume[c] == pytest.approx(k["volume"], rel=1e-12)
    faces = range(g.row_ptr[c], g.row_ptr[c + 1])
    assert len(faces) == len(k["faces"])
    by_nbr = {int(g.nbr[f]): f for f in faces}
    for kf in k["faces"]:
        f = by_nbr[kf["neighbour"]]
        assert g.kind[f] == gridmod._native.SW_FACE_LOCAL
        assert g.area[f] == pytest.approx(kf["area"], rel=1e-12)
        np.testing.assert_allclose(g.normal[f], kf["normal"], atol=1e-15)
    assert g.size[c] == pytest.approx((3 * k["volume"] / (4 * np.pi)) ** (1 / 3), rel=1e-12)


def test_voronoi_matches_scipy():
    from scipy.spatial import ConvexHull, Voronoi
    rng = np.random.default_rng(5)
    pts = rng.uniform(0, 1, size=(800, 3))
    g = gridmod.voronoi(pts, 1.0, periodic=False, nthreads=2)
    v = Voronoi(pts)
    checked = 0
    for i in range(len(pts)):
        reg = v.regions[v.point_region[i]]
        if -1 in reg or not reg:
            continue
        verts = v.vertices[reg]
        if (verts < 0).any() or (verts > 1).any():
            continue
        assert g.volume[i] == pytest.approx(ConvexHull(verts).volume, rel=1e-9)
        checked += 1
    assert checked > 200
    ridge = {(min(a, b), max(a, b)) for a, b in v.ridge_points}
    mine = {(min(i, int(g.nbr[f])), max(i, int(g.nbr[f]))) for i in range(len(pts))
            for f in range(g.row_ptr[i], g.row_ptr[i + 1]) if g.kind[f] == 0}
    assert mine <= ridge
    assert g.volume.sum() == pytest.approx(1.0, rel=1e-12)


@pytest.mark.parametrize("maker", ["lattice", "poisson"])
def test_periodic_voronoi_invariants(maker):
    box = 2.0
    pts = gridmod.jittered_lattice(10, box, 0.25, 3) if maker == "lattice" else gridmod.poisson_points(600, box, 7)
    g = gridmod.voronoi(pts, box, periodic=True, nthreads=2)
    n = g.num_cells
    assert g.volume.sum() == pytest.approx(box ** 3, rel=1e-12)
    assert (g.kind != gridmod._native.SW_FACE_BOUNDARY).all()
    # closed cells: sum of area-weighted normals vanishes
    closure = np.zeros((n, 3))
    for a in range(3):
        closure[:, a] = np.add.reduceat(g.area * g.normal[:, a], g.row_ptr[:-1])
    assert np.abs(closure).max() < 1e-12 * box ** 2
    # every face has a reciprocal face with the bitwise negated normal and equal area
    for c in range(n):
        for f in range(g.row_ptr[c], g.row_ptr[c + 1]):
            nb = g.nbr[f]
            rec = [q for q in range(g.row_ptr[nb], g.row_ptr[nb + 1])
                   if g.nbr[q] == c and (g.normal[q] == -g.normal[f]).all()]
            assert len(rec) == 1 and g.area[rec[0]] == g.area[f]
    assert g.faces_per_cell().max() <= 64


@pytest.mark.parametrize("periodic", [False, True])
def test_cartesian_grid_conventions(periodic):
    """cartesian.rs:220-395: 6 faces per cell, neighbour order x-,x+,y-,y+,z-,z+,
    area s^2, volume s^3, periodic faces LocalPeriodic or Boundary."""
    s = 2.5
    g = gridmod.cartesian(3, 4, 5, s, periodic)
    assert g.num_cells == 60
    assert (g.faces_per_cell() == 6).all()
    assert (g.area == s * s).all() and (g.volume == s ** 3).all() and (g.size == s).all()
    expected = np.array([[-1, 0, 0], [1, 0, 0], [0, -1, 0], [0, 1, 0], [0, 0, -1], [0, 0, 1]], float)
    np.testing.assert_array_equal(g.normal.reshape(-1, 6, 3), np.broadcast_to(expected, (60, 6, 3)))
    wrapped = g.kind != 0
    assert wrapped.sum() == 2 * (4 * 5 + 3 * 5 + 3 * 4)
    assert (g.kind[wrapped] == (1 if periodic else 2)).all()


def test_source_placement_nearest_cell():
    g = gridmod.cartesian(4, 4, 4, 1.0, False)
    src = gridmod.place_sources(g, np.array([[0.1, 0.1, 0.1], [0.2, 0.0, 0.0], [3.0, 3.0, 3.0]]),
                                np.array([1.0, 2.0, 5.0]))
    assert src[0] == 3.0 and src[-1] == 5.0 and src.sum() == 8.0
