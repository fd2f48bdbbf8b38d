"""Arepo connection lists -> sweep CSR (subsweep_gb300.arepo).

The conversion restates the reference's single-rank grid read-in
(src/arepo_postprocess/read_grid/mod.rs).  CPU: the ConnectionType rules, face order
and kinds on hand-made lists; a Voronoi grid written out as a shuffled connection list
with fresh particle ids comes back face for face; the dependency-cycle count; and the
oracle driven by the converted grid evolves like the original.  GPU: the mixed sweep on
the converted grid against the original grid.
"""
import numpy as np
import pytest

from oracle import binding
from subsweep_gb300 import arepo, grid as gridmod, workloads
from subsweep_gb300.sweep import Sweep, directions_from_num

from test_gpu_parity import oracle_dirs


def test_connection_type_bits():
    t = np.array([0, 1, 4, 5, 2, 8, -1, 6])
    valid, p1, p2 = arepo.connection_flags(t)
    np.testing.assert_array_equal(valid, [True, True, True, False, False, False, False, False])
    np.testing.assert_array_equal(p1[:3], [False, True, False])
    np.testing.assert_array_equal(p2[:3], [False, False, True])


def test_faces_in_connection_order_with_negated_normals():
    ids = np.array([30, 10, 20])  # cell order: ids as given
    vol = np.array([8.0, 27.0, 1.0])
    n1, n2, n3 = [1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0]
    g = arepo.from_connections(ids, vol, id1=[10, 20, 30, 10], id2=[20, 30, 10, 99],
                               connection_type=[0, 0, 0, -1], area=[1.0, 2.0, 3.0, 4.0],
                               normal=[n1, n2, n3, n1], periodic=False)
    np.testing.assert_array_equal(g.row_ptr, [0, 2, 4, 6])
    # cell 0 (id 30): connection 1 as id2 (+N, towards 20), connection 2 as id1 (-N, towards 10)
    np.testing.assert_array_equal(g.nbr[0:2], [2, 1])
    np.testing.assert_array_equal(g.normal[0:2], [n2, np.negative(n3)])
    np.testing.assert_array_equal(g.area[0:2], [2.0, 3.0])
    # cell 1 (id 10): connection 0 as id1 (-N to 20), connection 2 as id2 (+N to 30)
    np.testing.assert_array_equal(g.nbr[2:4], [2, 0])
    np.testing.assert_array_equal(g.normal[2:4], [np.negative(n1), n3])
    np.testing.assert_array_equal(g.kind, 0)
    np.testing.assert_allclose(g.size, [2.0, 3.0, 1.0])


def test_periodic_connections():
    ids, vol = np.array([1, 2]), np.ones(2)
    args = dict(id1=[1], id2=[2], connection_type=[4], area=[1.0], normal=[[1.0, 0, 0]])
    gp = arepo.from_connections(ids, vol, periodic=True, **args)
    np.testing.assert_array_equal(gp.kind, [arepo.FACE_LOCAL_PERIODIC] * 2)
    np.testing.assert_array_equal(gp.nbr, [1, 0])
    gb = arepo.from_connections(ids, vol, periodic=False, **args)
    np.testing.assert_array_equal(gb.kind, [arepo.FACE_BOUNDARY] * 2)
    np.testing.assert_array_equal(gb.nbr, [-1, -1])


def test_unknown_ids():
    ids, vol = np.array([1, 2]), np.ones(2)
    g = arepo.from_connections(ids, vol, id1=[1, 7], id2=[2, 8], connection_type=[0, 0], area=[1.0, 1.0],
                               normal=[[1.0, 0, 0]] * 2, periodic=False)
    assert g.num_faces == 2  # the connection between two unknown ids is not this grid's
    with pytest.raises(ValueError, match="unknown particle id"):
        arepo.from_connections(ids, vol, id1=[1], id2=[8], connection_type=[0], area=[1.0],
                               normal=[[1.0, 0, 0]], periodic=False)
    with pytest.raises(ValueError, match="duplicate"):
        arepo.from_connections(np.array([1, 1]), vol, id1=[1], id2=[1], connection_type=[0], area=[1.0],
                               normal=[[1.0, 0, 0]], periodic=False)


def to_connections(g, uid, rng):
    """The grid's faces as an Arepo connection list: one connection per reciprocal face
    pair, in random order, Id1 / Id2 in random roles."""
    owner = np.repeat(np.arange(g.num_cells), np.diff(g.row_ptr))
    keep = (g.kind != arepo.FACE_BOUNDARY) & (owner < g.nbr)
    f = np.flatnonzero(keep)
    swap = rng.random(f.size) < 0.5
    a, b = owner[f], g.nbr[f].astype(np.int64)
    id1 = np.where(swap, uid[b], uid[a])
    id2 = np.where(swap, uid[a], uid[b])
    # id1's face gets -Normal: Normal = -(outward normal of id1's face)
    normal = np.where(swap[:, None], g.normal[f], -g.normal[f])
    ctype = np.where(g.kind[f] == arepo.FACE_LOCAL_PERIODIC, np.where(swap, 1, 4), 0)
    perm = rng.permutation(f.size)
    return id1[perm], id2[perm], ctype[perm], g.area[f][perm], normal[perm]


def face_table(g, c):
    sl = slice(g.row_ptr[c], g.row_ptr[c + 1])
    rows = sorted(zip(g.nbr[sl].tolist(), g.kind[sl].tolist(), g.area[sl].tolist(),
                      map(tuple, g.normal[sl].tolist())))
    return rows


@pytest.fixture(scope="module")
def voronoi_pair():
    w = workloads.c1_small_periodic(n_per_side=8, num_directions=16, nthreads=2)
    g = w.grid
    rng = np.random.default_rng(3)
    uid = rng.choice(10 ** 9, size=g.num_cells, replace=False).astype(np.int64)
    conv = arepo.from_connections(uid, g.volume, *to_connections(g, uid, rng), periodic=True,
                                  position=g.position, box_size=g.box_size)
    return w, conv


def test_voronoi_round_trip(voronoi_pair):
    w, conv = voronoi_pair
    g = w.grid
    assert conv.num_cells == g.num_cells and conv.num_faces == g.num_faces
    for c in range(g.num_cells):
        assert face_table(conv, c) == face_table(g, c), c
    np.testing.assert_allclose(conv.size, np.cbrt(g.volume))


def test_dependency_cycles():
    from test_abi import _cyclic_grid
    assert arepo.dependency_cycles(_cyclic_grid(), np.array([[0.0, 0.0, 1.0]])) == 3
    g = workloads.c1_small_periodic(n_per_side=6, num_directions=16, nthreads=2).grid
    assert arepo.dependency_cycles(g, directions_from_num(16)) == 0


def test_read_grid_file_needs_h5py():
    try:
        import h5py  # noqa: F401
    except ImportError:
        with pytest.raises(ImportError):
            arepo.read_grid_file("grid.hdf5", "snap.hdf5", periodic=True)
    else:
        pytest.skip("h5py present: the file reader is exercised by from_connections' tests")


def _with_grid(w, grid):
    return dict(params=w.params, grid=grid, density=w.density, x=w.ionized_hydrogen_fraction,
                T=w.temperature, src=w.source)


def test_oracle_on_converted_grid(voronoi_pair):
    """Same simulation: only each cell's face order differs, i.e. the order of the
    oracle's FP64 additions."""
    w, conv = voronoi_pair
    size = np.cbrt(w.grid.volume)
    base = gridmod.Grid(**{**w.grid.__dict__, "size": size})

    def run(g):
        o = binding.OracleSweep(w.params, g, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
                                oracle_dirs(w.params))
        for _ in range(3):
            o.run_sweeps()
        return o.fields()

    fa, fb = run(conv), run(base)
    for k in ("ionized_hydrogen_fraction", "temperature"):
        np.testing.assert_allclose(fa[k], fb[k], rtol=1e-9, err_msg=k)


@pytest.mark.gpu
def test_gpu_sweep_on_converted_grid(voronoi_pair):
    w, conv = voronoi_pair
    base = gridmod.Grid(**{**w.grid.__dict__, "size": np.cbrt(w.grid.volume)})
    out = []
    for g in (conv, base):
        s = Sweep(w.params, g, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source, precision="mixed")
        for _ in range(3):
            s.run_sweeps()
        out.append(s.fields())
        s.close()
    for k in ("ionized_hydrogen_fraction", "temperature"):
        np.testing.assert_allclose(out[0][k], out[1][k], rtol=1e-5, err_msg=k)
