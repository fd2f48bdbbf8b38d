"""Arepo connection lists -> sweep CSR (subsweep_gb300.arepo).

The conversion restates the reference's single-rank grid read-in
(src/arepo_postprocess/read_grid/mod.rs).  CPU: the ConnectionType rules, face order
and kinds on hand-made lists; a Voronoi grid written out as a shuffled connection list
with fresh particle ids comes back face for face, also through HDF5 grid and snapshot
files in Arepo's comoving code units; the initial gas state of a snapshot; the
dependency-cycle count; and the oracle driven by the converted grid evolves like the
original.  GPU: the mixed sweep on
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


KPC = 3.085678e21      # cm
MSUN10 = 1.989e43      # 1e10 solar masses in g


def _arepo_attrs(to_cgs, length=0, mass=0, velocity=0, a=0, h=0):
    return {"to_cgs": np.float64(to_cgs), "length_scaling": np.float64(length), "mass_scaling": np.float64(mass),
            "velocity_scaling": np.float64(velocity), "a_scaling": np.float64(a), "h_scaling": np.float64(h)}


def _arepo_factor(to_cgs, length=0, mass=0, a=0, h=0, cosmo=(0.5, 0.7)):
    """SI factor of a dataset with these exponents (src/arepo_postprocess/unit_reader.rs:97-115)."""
    ca, ch = cosmo
    return (1.0 / (ca ** -a * ch ** -h)) * (0.01 ** length * 0.001 ** mass) * to_cgs


def test_read_grid_file_from_hdf5(voronoi_pair, tmp_path):
    """A snapshot (split over two files) and a grid file written in Arepo's comoving code
    units read back as the grid from_connections builds from the SI arrays."""
    from hdf5_writer import H5Writer
    from subsweep_gb300 import hdf5

    w, _ = voronoi_pair
    g = w.grid
    rng = np.random.default_rng(11)
    uid = rng.choice(10 ** 12, size=g.num_cells, replace=False).astype(np.uint64)
    id1, id2, ctype, area, normal = to_connections(g, uid.astype(np.int64), rng)
    a_mass = dict(mass=1, h=-1)
    a_rho = dict(length=-3, mass=1, a=-3, h=2)
    a_area = dict(length=2, a=2, h=-2)
    rho_code = rng.uniform(1e-3, 1e-1, g.num_cells)
    mass_code = g.volume * (rho_code * _arepo_factor(6.77e-22, **a_rho)) / _arepo_factor(MSUN10, **a_mass)
    area_code = area / _arepo_factor(KPC ** 2, **a_area)

    snap = tmp_path / "snap"
    snap.mkdir()
    half = g.num_cells // 2
    for i, sl in enumerate((slice(0, half), slice(half, None))):
        s = H5Writer()
        s.group("Header", {"Time": np.float64(0.5)})
        s.dataset("PartType0/ParticleIDs", uid[sl])
        s.dataset("PartType0/Masses", mass_code[sl].astype(np.float32), attrs=_arepo_attrs(MSUN10, **a_mass))
        s.dataset("PartType0/Density", rho_code[sl].astype(np.float32), attrs=_arepo_attrs(6.77e-22, **a_rho))
        s.write(snap / f"snap_010.{i}.hdf5")
    gw = H5Writer()
    gw.dataset("Id1", id1.astype(np.uint64), layout="chunked", chunks=(1000,), filters=("shuffle", "deflate"))
    gw.dataset("Id2", id2.astype(np.uint64), layout="chunked", chunks=(1000,), filters=("shuffle", "deflate"))
    gw.dataset("ConnectionType", ctype.astype(np.int32))
    gw.dataset("Area", area_code, attrs=_arepo_attrs(KPC ** 2, **a_area))
    gw.dataset("Normal", normal, attrs=_arepo_attrs(0.0))
    gw.write(tmp_path / "grid.hdf5")

    cosmo = hdf5.Cosmology(a=0.5, h=0.7)
    got = arepo.read_grid_file(tmp_path / "grid.hdf5", snap, periodic=True, cosmology=cosmo)
    mass_si = mass_code.astype(np.float32).astype(np.float64) * _arepo_factor(MSUN10, **a_mass)
    rho_si = rho_code.astype(np.float32).astype(np.float64) * _arepo_factor(6.77e-22, **a_rho)
    want = arepo.from_connections(uid.astype(np.int64), mass_si / rho_si, id1, id2, ctype,
                                  area_code * _arepo_factor(KPC ** 2, **a_area), normal, periodic=True)
    for field in ("row_ptr", "nbr", "kind", "area", "normal", "volume", "size"):
        np.testing.assert_array_equal(getattr(got, field), getattr(want, field), err_msg=field)
    # the geometry is the original grid's to the float32 rounding of the snapshot's fields
    np.testing.assert_allclose(got.volume, g.volume, rtol=1e-6)
    np.testing.assert_allclose(got.area, want.area, rtol=0)
    for c in range(0, g.num_cells, 37):
        assert [r[:2] for r in face_table(got, c)] == [r[:2] for r in face_table(g, c)]
    with pytest.raises(hdf5.H5Error, match="no cosmology given"):
        arepo.read_grid_file(tmp_path / "grid.hdf5", snap, periodic=True)


def test_read_initial_conditions(tmp_path):
    """Density, x_HII from the electron abundance (0.76 x_e clamped) or a fixed fraction,
    and T from the internal energy, in SI (src/main.rs:159-219)."""
    from hdf5_writer import H5Writer
    from subsweep_gb300 import hdf5
    from subsweep_gb300.sweep import PROTON_MASS

    rng = np.random.default_rng(5)
    n = 50
    rho = rng.uniform(1e-4, 1e-2, n)
    u = rng.uniform(10.0, 1e3, n)       # (km/s)^2
    xe = np.concatenate([[0.0, 2.0], rng.uniform(0, 1.2, n - 2)])
    pos = rng.uniform(0, 1e4, (n, 3))  # kpc
    s = H5Writer()
    s.dataset("PartType0/Density", rho, attrs=_arepo_attrs(6.77e-22, length=-3, mass=1))
    s.dataset("PartType0/InternalEnergy", u, attrs=_arepo_attrs(1e10, velocity=2))
    s.dataset("PartType0/ElectronAbundance", xe, attrs=_arepo_attrs(0.0))
    s.dataset("PartType0/Coordinates", pos, attrs=_arepo_attrs(KPC, length=1))
    s.write(tmp_path / "snap.hdf5")
    ic = arepo.read_initial_conditions(tmp_path / "snap.hdf5")
    rho_si = rho * (0.01 ** -3 * 0.001 * 6.77e-22)
    u_si = u * (0.01 ** 2 * 1e10)
    x = np.clip(0.76 * xe, 1e-10, 1 - 1e-10)
    np.testing.assert_array_equal(ic["density"], rho_si)
    np.testing.assert_array_equal(ic["ionized_hydrogen_fraction"], x)
    assert ic["ionized_hydrogen_fraction"][0] == 1e-10 and ic["ionized_hydrogen_fraction"][1] == 1 - 1e-10
    np.testing.assert_array_equal(ic["position"], pos * (0.01 * KPC))
    want_t = (u_si * rho_si) / rho_si * (1.0 / (x + 1.0)) * (5.0 / 3.0 - 1.0) * PROTON_MASS / 1.380649e-23
    np.testing.assert_array_equal(ic["temperature"], want_t)
    # u of 10 to 1000 (km/s)^2 is some 10^2.5 to 10^5 K
    assert 1e2 < ic["temperature"].min() and ic["temperature"].max() < 1e6
    fixed = arepo.read_initial_conditions(tmp_path / "snap.hdf5", initial_fraction_ionized_hydrogen=0.5)
    assert np.all(fixed["ionized_hydrogen_fraction"] == 0.5)
    np.testing.assert_array_equal(fixed["temperature"],
                                  (u_si * rho_si) / rho_si * (1.0 / 1.5) * (5.0 / 3.0 - 1.0) * PROTON_MASS / 1.380649e-23)


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


def _ref_attrs(factor, length=0, mass=0, time=0, temperature=0):
    return {"scale_factor_si": np.float64(factor), "scaling_length": np.int32(length),
            "scaling_mass": np.int32(mass), "scaling_time": np.int32(time),
            "scaling_temperature": np.int32(temperature)}


def _write_run(folder, rng, n_old, a_first, vector="array"):
    """Output folders 0, 3 and 12 of an earlier run: positions in the first (as an
    array-typed or compound-typed 1-D dataset), x_HII and T in every folder (the last
    one's differ), the cosmology attributes on the root group."""
    from hdf5_writer import H5Writer
    pos = rng.uniform(0, 1e21, (n_old, 3))
    fields = {}
    for k in (0, 3, 12):
        sub = folder / f"{k}"
        sub.mkdir(parents=True)
        x = rng.uniform(0, 1, n_old)
        t = rng.uniform(1e3, 1e5, n_old)
        fields[k] = (x, t)
        w = H5Writer()
        w.group("/", {"scale_factor": np.float64(a_first + 0.01 * k), "little_h": np.float64(0.7),
                      "time": np.float64(k)})
        if vector == "array":
            w.dataset("position", pos, dtype=np.dtype(("<f8", (3,))), attrs=_ref_attrs(1.0, length=1))
        else:
            xyz = np.zeros(n_old, dtype=[("x", "<f8"), ("y", "<f8"), ("z", "<f8")])
            xyz["x"], xyz["y"], xyz["z"] = pos.T
            w.dataset("position", xyz, attrs=_ref_attrs(1.0, length=1))
        w.dataset("ionized_hydrogen_fraction", x, attrs=_ref_attrs(1.0))
        w.dataset("temperature", t, attrs=_ref_attrs(1.0, temperature=1))
        w.write(sub / "snapshot.hdf5")
    return pos, fields


@pytest.mark.parametrize("vector", ["array", "compound"])
def test_remap_from_earlier_run(tmp_path, vector):
    """remap_from (src/arepo_postprocess/remap.rs): positions of the first folder scaled
    by a / a_first, x_HII and T of the last folder (12, not 3: folders go by number),
    each cell raised to its nearest old cell's values; a NaN is ignored as f64::max does."""
    from subsweep_gb300 import hdf5
    rng = np.random.default_rng(21)
    pos_old, fields = _write_run(tmp_path / "run", rng, 400, a_first=0.25, vector=vector)
    cosmo = hdf5.Cosmology(a=0.5, h=0.7)
    assert [p.name for p in arepo.snapshot_folders(tmp_path / "run")] == ["0", "12"]
    pos_new = rng.uniform(0, 2e21, (300, 3))
    x0 = rng.uniform(0, 1, 300)
    t0 = rng.uniform(1e3, 1e5, 300)
    x0[5], t0[7] = np.nan, np.nan
    x, t = arepo.remap_abundances_and_temperatures(tmp_path / "run", pos_new, x0, t0, cosmo)
    scaled = pos_old * (0.5 / 0.25)
    d2 = ((pos_new[:, None, :] - scaled[None, :, :]) ** 2).sum(-1)
    nearest = d2.argmin(1)
    old_x, old_t = fields[12]
    np.testing.assert_array_equal(x, np.fmax(x0, old_x[nearest]))
    np.testing.assert_array_equal(t, np.fmax(t0, old_t[nearest]))
    assert x[5] == old_x[nearest[5]] and t[7] == old_t[nearest[7]]
    assert np.all(x >= np.nan_to_num(x0)) and np.any(x > x0)


def test_remap_errors(tmp_path):
    from subsweep_gb300 import hdf5
    rng = np.random.default_rng(2)
    cosmo = hdf5.Cosmology(a=0.5, h=0.7)
    pos = np.zeros((1, 3))
    with pytest.raises(hdf5.H5Error, match="No snapshot folder exists"):
        (tmp_path / "empty").mkdir()
        arepo.remap_abundances_and_temperatures(tmp_path / "empty", pos, [0.1], [1e4], cosmo)
    _write_run(tmp_path / "run", rng, 10, a_first=0.25)
    with pytest.raises(hdf5.H5Error, match="needs the cosmology"):
        arepo.remap_abundances_and_temperatures(tmp_path / "run", pos, [0.1], [1e4], None)
    (tmp_path / "run" / "latest").mkdir()
    with pytest.raises(hdf5.H5Error, match="Unexpected folder in snapshot dir"):
        arepo.remap_abundances_and_temperatures(tmp_path / "run", pos, [0.1], [1e4], cosmo)


def test_read_initial_conditions_with_remap(tmp_path):
    """The snapshot's own x_HII and T, then the remap on top, as src/main.rs orders the
    startup stages (derived components before the remap)."""
    from hdf5_writer import H5Writer
    from subsweep_gb300 import hdf5
    rng = np.random.default_rng(4)
    _write_run(tmp_path / "run", rng, 200, a_first=0.5)
    n = 60
    s = H5Writer()
    s.dataset("PartType0/Density", rng.uniform(1e-4, 1e-2, n), attrs=_arepo_attrs(6.77e-22, length=-3, mass=1))
    s.dataset("PartType0/InternalEnergy", rng.uniform(10.0, 1e3, n), attrs=_arepo_attrs(1e10, velocity=2))
    s.dataset("PartType0/ElectronAbundance", rng.uniform(0, 1, n), attrs=_arepo_attrs(0.0))
    s.dataset("PartType0/Coordinates", rng.uniform(0, 1e21 / (0.01 * KPC), (n, 3)), attrs=_arepo_attrs(KPC, length=1))
    s.write(tmp_path / "snap.hdf5")
    cosmo = hdf5.Cosmology(a=0.5, h=0.7)
    plain = arepo.read_initial_conditions(tmp_path / "snap.hdf5", cosmology=cosmo)
    remapped = arepo.read_initial_conditions(tmp_path / "snap.hdf5", cosmology=cosmo, remap_from=tmp_path / "run")
    x, t = arepo.remap_abundances_and_temperatures(tmp_path / "run", plain["position"],
                                                   plain["ionized_hydrogen_fraction"], plain["temperature"], cosmo)
    np.testing.assert_array_equal(remapped["ionized_hydrogen_fraction"], x)
    np.testing.assert_array_equal(remapped["temperature"], t)
    np.testing.assert_array_equal(remapped["density"], plain["density"])


def test_read_postprocess_inputs_runs_on_the_oracle(voronoi_pair, tmp_path):
    """Grid file + snapshot (gas and stars) -> the inputs of a sweep, in the snapshot's
    cell order; they equal the pieces read one by one, and the oracle steps them."""
    from hdf5_writer import H5Writer
    from subsweep_gb300 import hdf5
    from subsweep_gb300.cosmology import Cosmology

    w, _ = voronoi_pair
    g = w.grid
    rng = np.random.default_rng(31)
    n = g.num_cells
    uid = rng.choice(10 ** 9, size=n, replace=False).astype(np.uint64)
    id1, id2, ctype, area, normal = to_connections(g, uid.astype(np.int64), rng)
    cosmo = Cosmology(a=0.5, h=0.7, omega_0=0.3, omega_lambda=0.7)
    one = dict(a=0, h=0)
    rho = rng.uniform(0.5, 2.0, n) * w.density
    s = H5Writer()
    s.dataset("PartType0/ParticleIDs", uid)
    s.dataset("PartType0/Masses", rho * g.volume * 1e3, attrs=_arepo_attrs(1.0, mass=1, **one))
    s.dataset("PartType0/Density", rho * 1e-3, attrs=_arepo_attrs(1.0, length=-3, mass=1, **one))
    s.dataset("PartType0/InternalEnergy", rng.uniform(1e11, 1e12, n), attrs=_arepo_attrs(1.0, velocity=2, **one))
    s.dataset("PartType0/ElectronAbundance", rng.uniform(0, 1e-3, n), attrs=_arepo_attrs(0.0))
    s.dataset("PartType0/Coordinates", g.position * 100.0, attrs=_arepo_attrs(1.0, length=1, **one))
    stars = g.position[rng.choice(n, 5, replace=False)] * 100.0
    s.dataset("PartType4/Coordinates", stars, attrs=_arepo_attrs(1.0, length=1, **one))
    s.dataset("PartType4/GFM_Metallicity", np.full(5, 0.01), attrs=_arepo_attrs(0.0))
    s.dataset("PartType4/GFM_StellarFormationTime", np.array([0.49, 0.495, 0.48, -1.0, 0.499]),
              attrs=_arepo_attrs(0.0))
    s.dataset("PartType4/Masses", np.full(5, 1e5 * 1.988477e33), attrs=_arepo_attrs(1.0, mass=1, **one))
    s.write(tmp_path / "snap.hdf5")
    gw = H5Writer()
    for name, arr in (("Id1", id1.astype(np.uint64)), ("Id2", id2.astype(np.uint64)), ("ConnectionType", ctype)):
        gw.dataset(name, arr)
    gw.dataset("Area", area * 1e4, attrs=_arepo_attrs(1.0, length=2, **one))
    gw.dataset("Normal", normal, attrs=_arepo_attrs(0.0))
    gw.write(tmp_path / "grid.hdf5")

    inp = arepo.read_postprocess_inputs(tmp_path / "grid.hdf5", tmp_path / "snap.hdf5", cosmo, periodic=True,
                                        escape_fraction=0.1)
    grid = arepo.read_grid_file(tmp_path / "grid.hdf5", tmp_path / "snap.hdf5", True, cosmo)
    ic = arepo.read_initial_conditions(tmp_path / "snap.hdf5", cosmology=cosmo)
    pos, rates = arepo.read_sources(tmp_path / "snap.hdf5", cosmo, 0.1)
    assert pos.shape == (4, 3)  # the wind particle is dropped
    for field in ("row_ptr", "nbr", "kind", "area", "normal", "volume"):
        np.testing.assert_array_equal(getattr(inp["grid"], field), getattr(grid, field))
    np.testing.assert_array_equal(inp["grid"].position, ic["position"])
    for k in ("density", "ionized_hydrogen_fraction", "temperature"):
        np.testing.assert_array_equal(inp[k], ic[k])
    np.testing.assert_array_equal(inp["source"], arepo.source_rates(ic["position"], pos, rates))
    assert np.count_nonzero(inp["source"]) == 4 and inp["source"].sum() == pytest.approx(rates.sum(), rel=1e-12)
    np.testing.assert_allclose(inp["grid"].volume, g.volume, rtol=1e-12)
    with pytest.raises(ValueError, match="either escape_fraction"):
        arepo.read_postprocess_inputs(tmp_path / "grid.hdf5", tmp_path / "snap.hdf5", cosmo, True)

    def run(source):
        o = binding.OracleSweep(w.params, inp["grid"], inp["density"], inp["ionized_hydrogen_fraction"],
                                inp["temperature"], source, oracle_dirs(w.params))
        for _ in range(2):
            o.run_sweeps()
        return o.fields()["ionized_hydrogen_fraction"]

    lit, dark = run(inp["source"]), run(np.zeros(n))
    assert np.all(np.isfinite(lit)) and np.all(lit >= dark)
    assert np.all(lit[inp["source"] > 0] > dark[inp["source"] > 0])
