"""The package's HDF5 reader (subsweep_gb300.hdf5) and the reference's dataset input on
top of it, on the CPU.

Pinned to the reference's own input fixtures (tests/golden/hdf5/, copied by
tests/golden/gen_reference_hdf5.py from the reference's tests/input/): the known answers
of src/io/input/tests.rs:23-50.  The structures those two files lack (nested groups,
chunked and filtered data, continuation blocks, user blocks, other types and layout
versions) are covered by files from the test writer tests/hdf5_writer.py; the unit
readers (src/io/unit_reader.rs, src/arepo_postprocess/unit_reader.rs) on both.
"""
import pathlib
import zlib

import numpy as np
import pytest

from subsweep_gb300 import hdf5
from hdf5_writer import H5Writer

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "hdf5"
SOLAR_MASS = 1.988477e30  # src/units/mod.rs:55, kg


# ---------------------------------------------------------------------------------------
# the reference's fixtures

def test_reference_fixture_respects_scale_factor():
    """respect_scale_factor (src/io/input/tests.rs:23-42): one particle stored with the
    value of 1 solar mass and `scale_factor_si` 5 reads as 5 solar masses; the reference
    compares with an absolute tolerance of f64 epsilon, so the value is exact."""
    mass = hdf5.read_dataset(GOLDEN / "respect_scale_factor.hdf5", "mass", hdf5.MASS)
    assert mass.shape == (1,) and mass.dtype == np.float64
    assert abs(mass[0] - 5.0 * SOLAR_MASS) < np.finfo(np.float64).eps
    assert mass[0] == 5.0 * SOLAR_MASS


def test_reference_fixture_dimension_mismatch():
    """panic_on_dimension_mismatch (src/io/input/tests.rs:44-51): the dataset is stored
    with length exponent 1 beside mass 1, which is not a mass."""
    with pytest.raises(hdf5.H5Error, match=r"^Mismatch in dimension while reading dataset mass\.$"):
        hdf5.read_dataset(GOLDEN / "panic_on_dimension_mismatch.hdf5", "mass", hdf5.MASS)


def test_reference_fixture_structure():
    """The fixtures as the reference's writer lays them out: one root dataset with its
    unit attributes, the output time on the root group."""
    for name, length, factor in (("respect_scale_factor", 0, 5.0), ("panic_on_dimension_mismatch", 1, 1.0)):
        with hdf5.File(GOLDEN / f"{name}.hdf5") as f:
            assert f.keys() == ["mass"] and "mass" in f and "nothing" not in f
            assert set(f.attrs) == {"time"} and f.attrs["time"].dtype == np.float64
            ds = f["mass"]
            assert ds.shape == (1,) and ds.dtype == np.dtype("<f8") and len(ds) == 1
            np.testing.assert_array_equal(ds.read(), [SOLAR_MASS])
            a = ds.attrs
            assert a["scale_factor_si"] == factor and a["scale_factor_si"].dtype == np.float64
            assert (a["scaling_length"], a["scaling_mass"], a["scaling_time"], a["scaling_temperature"]) == \
                (length, 1, 0, 0)
            assert a["scaling_length"].dtype == np.int32 and a["scaling_amount"].dtype == np.int64
            assert hdf5.DefaultUnits().dimension(ds) == hdf5.Dimension(length=length, mass=1)


# ---------------------------------------------------------------------------------------
# the reader on written files

def _write(tmp_path, name="f.hdf5", **kw):
    w = H5Writer(**{k: kw.pop(k) for k in ("user_block", "continuation") if k in kw})
    return w, tmp_path / name


DATA = {
    "f8_rows": np.random.default_rng(1).random((1000, 3)),
    "f4_be": np.random.default_rng(2).random(777).astype(">f4"),
    "i4": np.arange(-500, 500, dtype=np.int32),
    "u8_ids": np.random.default_rng(3).integers(0, 2 ** 63, 300, dtype=np.uint64) * 2 + 1,
    "i8_be": np.arange(100, dtype=">i8") - 50,
    "u1": np.arange(256, dtype=np.uint8),
    "f2": np.linspace(-2, 2, 33).astype(np.float16),
}


@pytest.mark.parametrize("user_block,continuation", [(0, False), (512, True), (2048, False)])
def test_round_trip_contiguous(tmp_path, user_block, continuation):
    w, path = _write(tmp_path, user_block=user_block, continuation=continuation)
    for name, arr in DATA.items():
        w.dataset(f"PartType0/{name}", arr, attrs={"unit": np.float64(2.5), "exp": np.int32(-3)})
    w.group("Header", {"Time": np.float64(0.25), "NumPart_ThisFile": np.array([7, 0, 3], np.uint32),
                       "Name": np.bytes_(b"arepo")})
    w.dataset("Scalar", np.float64(42.0))
    w.write(path)
    with hdf5.File(path) as f:
        assert f.keys() == ["Header", "PartType0", "Scalar"]
        assert f["PartType0"].keys() == sorted(DATA)
        for name, arr in DATA.items():
            ds = f[f"PartType0/{name}"]
            assert ds.shape == arr.shape and ds.dtype == arr.dtype
            out = ds.read()
            assert out.dtype == arr.dtype.newbyteorder("=")
            np.testing.assert_array_equal(out, arr)
            assert ds.attrs == {"unit": 2.5, "exp": -3}
        h = f["Header"].attrs
        assert h["Time"] == 0.25 and h["Name"] == b"arepo"
        np.testing.assert_array_equal(h["NumPart_ThisFile"], [7, 0, 3])
        s = f["Scalar"].read()
        assert s.shape == () and s == 42.0
        with pytest.raises(TypeError):
            len(f["Scalar"])
        assert f["/PartType0/i4"] is f["PartType0"]["i4"]


@pytest.mark.parametrize("filters", [(), ("deflate",), ("shuffle", "deflate"), ("shuffle", "deflate", "fletcher32"),
                                     ("fletcher32",)])
@pytest.mark.parametrize("fanout", [None, 3])
def test_round_trip_chunked(tmp_path, filters, fanout):
    """Chunked datasets with ragged edge chunks in both axes, a one- or two-level chunk
    B-tree, each filter pipeline the reader takes, and row ranges that cut chunks."""
    w, path = _write(tmp_path)
    rows = DATA["f8_rows"]
    w.dataset("rows", rows, layout="chunked", chunks=(64, 2), filters=filters, btree_fanout=fanout)
    w.dataset("ids", DATA["u8_ids"], layout="chunked", chunks=(50,), filters=filters, btree_fanout=fanout)
    w.dataset("be", DATA["f4_be"], layout="chunked", chunks=(100,), filters=filters)
    w.write(path)
    with hdf5.File(path) as f:
        np.testing.assert_array_equal(f["rows"].read(), rows)
        np.testing.assert_array_equal(f["ids"].read(), DATA["u8_ids"])
        np.testing.assert_array_equal(f["be"].read(), DATA["f4_be"])
        for lo, hi in ((0, 1), (63, 65), (100, 333), (960, 1000), (999, 5000), (-10, None), (500, 400)):
            np.testing.assert_array_equal(f["rows"].read(lo, hi), rows[lo:hi])


@pytest.mark.parametrize("members", [1, 40, 300])
def test_groups_of_many_members(tmp_path, members):
    """Groups whose members fill several symbol nodes (8 entries each, as the library
    writes them: a snapshot's PartType0 holds tens of datasets) and, past 256 members,
    a two-level group B-tree."""
    w, path = _write(tmp_path)
    for i in range(members):
        w.dataset(f"PartType0/field_{i:03d}", np.full(3, float(i)))
    w.write(path)
    with hdf5.File(path) as f:
        assert f["PartType0"].keys() == [f"field_{i:03d}" for i in range(members)]
        for i in (0, members // 2, members - 1):
            np.testing.assert_array_equal(f[f"PartType0/field_{i:03d}"].read(), np.full(3, float(i)))


def test_chunk_filter_mask(tmp_path):
    """A chunk stored with a filter skipped (its bit set in the chunk's filter mask) is
    decoded without that filter."""
    w, path = _write(tmp_path)
    arr = np.arange(1000, dtype=np.float64)
    w.dataset("x", arr, layout="chunked", chunks=(128,), filters=("shuffle", "deflate"),
              filter_mask_first_chunk=0b10)
    w.write(path)
    with hdf5.File(path) as f:
        np.testing.assert_array_equal(f["x"].read(), arr)


def test_other_layouts_and_dataspaces(tmp_path):
    w, path = _write(tmp_path)
    w.dataset("compact", np.arange(6, dtype=np.int16).reshape(2, 3), layout="compact")
    w.dataset("v1_layout", DATA["f8_rows"][:10], layout_version=1)
    w.dataset("v2_layout", DATA["i4"], layout_version=2)
    w.dataset("v2_space", DATA["f8_rows"][:5], dataspace_version=2)
    w.dataset("unallocated", np.ones(4), unallocated=True)
    w.dataset("empty", np.zeros((0, 3)))
    w.dataset("empty_chunked", np.zeros((0,)), layout="chunked", chunks=(16,))
    w.write(path)
    with hdf5.File(path) as f:
        np.testing.assert_array_equal(f["compact"].read(), np.arange(6).reshape(2, 3))
        np.testing.assert_array_equal(f["v1_layout"].read(), DATA["f8_rows"][:10])
        np.testing.assert_array_equal(f["v2_layout"].read(), DATA["i4"])
        np.testing.assert_array_equal(f["v2_space"].read(), DATA["f8_rows"][:5])
        np.testing.assert_array_equal(f["unallocated"].read(), np.zeros(4))  # fill value 0
        assert f["empty"].read().shape == (0, 3) and f["empty_chunked"].read().shape == (0,)
        np.testing.assert_array_equal(f["v1_layout"].read(3, 6), DATA["f8_rows"][3:6])


@pytest.mark.parametrize("type_version", [0, 3])
@pytest.mark.parametrize("layout", ["contiguous", "chunked"])
def test_compound_and_array_types(tmp_path, type_version, layout):
    """Vectors stored as one element each: an array type [f64; 3] (trailing axis) and a
    compound {x, y, z} (structured array), as writers of 3-vectors lay them out; a
    compound with an array member and mixed types."""
    rng = np.random.default_rng(9)
    vec = rng.random((50, 3))
    xyz = np.zeros(50, dtype=[("x", "<f8"), ("y", "<f8"), ("z", "<f8")])
    xyz["x"], xyz["y"], xyz["z"] = vec.T
    mixed = np.zeros(20, dtype=[("id", "<u8"), ("pos", "<f4", (3,)), ("flag", "i1")])
    mixed["id"] = np.arange(20) * 7
    mixed["pos"] = rng.random((20, 3))
    mixed["flag"] = np.arange(20) % 3 - 1
    w, path = _write(tmp_path)
    kw = dict(layout=layout, chunks=(16,)) if layout == "chunked" else {}
    w.dataset("vec", vec, dtype=np.dtype(("<f8", (3,))), type_version=type_version, **kw)
    w.dataset("xyz", xyz, type_version=type_version, **kw)
    w.dataset("mixed", mixed, type_version=type_version or 2, **kw)
    w.group("g", {"corner": np.array([1.0, 2.0, 3.0])})
    w.write(path)
    with hdf5.File(path) as f:
        ds = f["vec"]
        assert ds.shape == (50,) and ds.dtype.shape == (3,)
        np.testing.assert_array_equal(ds.read(), vec)
        np.testing.assert_array_equal(ds.read(10, 20), vec[10:20])
        got = f["xyz"].read()
        assert got.dtype.names == ("x", "y", "z")
        np.testing.assert_array_equal(np.stack([got["x"], got["y"], got["z"]], 1), vec)
        got = f["mixed"].read()
        assert got.dtype.names == ("id", "pos", "flag")
        for name in ("id", "pos", "flag"):
            np.testing.assert_array_equal(got[name], mixed[name])


def test_undecoded_attributes_read_as_none(tmp_path):
    """An attribute of a type the reader does not decode (a variable-length string, as
    Arepo's Parameters group may hold) reads as None beside the others; a unit
    attribute of such a type is an error of the unit reader, not of the file."""
    from hdf5_writer import VlenString
    w, path = _write(tmp_path)
    w.group("Parameters", {"InitCondFile": VlenString("ics"), "BoxSize": np.float64(25.0)})
    w.dataset("x", np.arange(3.0), attrs={**_ref_attrs(2.0), "scale_factor_si": VlenString("2")})
    w.write(path)
    with hdf5.File(path) as f:
        assert f["Parameters"].attrs == {"InitCondFile": None, "BoxSize": 25.0}
    with pytest.raises(hdf5.H5Error, match="attribute 'scale_factor_si' of dataset '/x' is not a number"):
        hdf5.read_dataset(path, "x", hdf5.NONE)


def test_rejections(tmp_path):
    w, path = _write(tmp_path)
    w.dataset("x", np.arange(10.0))
    w.dataset("szip", np.arange(10.0), layout="chunked", chunks=(5,), filters=(4,))
    w.write(path)
    good = path.read_bytes()
    with hdf5.File(path) as f:
        with pytest.raises(KeyError):
            f["missing"]
        with pytest.raises(KeyError):
            f["x/below_a_dataset"]
        with pytest.raises(hdf5.H5Error, match="filter 4"):
            f["szip"]

    bad = tmp_path / "bad.hdf5"
    bad.write_bytes(b"not an hdf5 file at all" * 40)
    with pytest.raises(hdf5.H5Error, match="not an HDF5 file"):
        hdf5.File(bad)
    bad.write_bytes(b"")
    with pytest.raises(hdf5.H5Error, match="not an HDF5 file"):
        hdf5.File(bad)

    v2 = bytearray(good)
    v2[8] = 2
    bad.write_bytes(bytes(v2))
    with pytest.raises(hdf5.H5Error, match="superblock version 2"):
        hdf5.File(bad)

    root = int.from_bytes(good[56 + 8:56 + 16], "little")  # the root entry's object header address
    ohdr = bytearray(good)
    ohdr[root:root + 4] = b"OHDR"
    bad.write_bytes(bytes(ohdr))
    with pytest.raises(hdf5.H5Error, match="version 2 object header"):
        hdf5.File(bad)

    bad.write_bytes(good[:root])  # cut before the root group's header
    with pytest.raises(hdf5.H5Error, match="past the end"):
        hdf5.File(bad)


# ---------------------------------------------------------------------------------------
# units and files

def _ref_attrs(factor, length=0, mass=0, time=0, temperature=0):
    return {"scale_factor_si": np.float64(factor), "scaling_length": np.int32(length),
            "scaling_mass": np.int32(mass), "scaling_time": np.int32(time),
            "scaling_temperature": np.int32(temperature)}


def _arepo_attrs(to_cgs, length=0, mass=0, velocity=0, a=0, h=0):
    # Arepo writes the exponents as doubles
    return {"to_cgs": np.float64(to_cgs), "length_scaling": np.float64(length), "mass_scaling": np.float64(mass),
            "velocity_scaling": np.float64(velocity), "a_scaling": np.float64(a), "h_scaling": np.float64(h)}


def test_default_units(tmp_path):
    w, path = _write(tmp_path)
    vals = np.array([1.0, 2.5, -3.0])
    w.dataset("energy", vals, attrs=_ref_attrs(7.0, length=2, time=-2))
    w.dataset("nounits", vals)
    w.write(path)
    out = hdf5.read_dataset(path, "energy", hdf5.ENERGY_PER_MASS)
    np.testing.assert_array_equal(out, vals * 7.0)
    with pytest.raises(hdf5.H5Error, match="Mismatch in dimension"):
        hdf5.read_dataset(path, "energy", hdf5.LENGTH)
    with pytest.raises(hdf5.H5Error, match="No scale factor in dataset"):
        hdf5.read_dataset(path, "nounits", hdf5.NONE)
    np.testing.assert_array_equal(hdf5.read_dataset(path, "nounits", hdf5.NONE, hdf5.IdUnits()), vals)


def test_arepo_units(tmp_path):
    """to_cgs times 0.01^length * 0.001^mass, velocity folded into length and time, a and
    h divided out with the cosmology (src/arepo_postprocess/unit_reader.rs:97-128)."""
    kpc = 3.085678e21  # cm
    w, path = _write(tmp_path)
    x = np.array([1.0, 2.0, 4.0])
    w.dataset("length", x, attrs=_arepo_attrs(kpc, length=1))
    w.dataset("density", x, attrs=_arepo_attrs(6.77e-22, length=-3, mass=1, a=-3, h=2))
    w.dataset("velocity", x, attrs=_arepo_attrs(1e5, velocity=1))
    w.dataset("flag", x, attrs=_arepo_attrs(0.0))
    w.dataset("bad_zero", x, attrs=_arepo_attrs(0.0, mass=1))
    w.dataset("ids", np.arange(3, dtype=np.uint64))
    w.write(path)
    u = hdf5.ArepoUnits()
    np.testing.assert_array_equal(hdf5.read_dataset(path, "length", hdf5.LENGTH, u), x * (0.01 * kpc))
    np.testing.assert_array_equal(hdf5.read_dataset(path, "flag", hdf5.NONE, u), x)  # to_cgs 0: 1
    with pytest.raises(hdf5.H5Error, match="unit scale factor 0"):
        hdf5.read_dataset(path, "bad_zero", hdf5.MASS, u)
    with pytest.raises(hdf5.H5Error, match="no cosmology given"):
        hdf5.read_dataset(path, "density", hdf5.DENSITY, u)
    cosmo = hdf5.Cosmology(a=0.5, h=0.7)
    uc = hdf5.ArepoUnits(cosmo)
    f_rho = (1.0 / (0.5 ** 3 * 0.7 ** -2)) * (0.01 ** -3 * 0.001 ** 1) * 6.77e-22
    np.testing.assert_array_equal(hdf5.read_dataset(path, "density", hdf5.DENSITY, uc), x * f_rho)
    # velocity exponent 1: length 1, time -1
    np.testing.assert_array_equal(hdf5.read_dataset(path, "velocity", hdf5.Dimension(length=1, time=-1), uc),
                                  x * (0.01 * 1e5))
    with pytest.raises(hdf5.H5Error, match="No length scale factor in dataset: '/ids'"):
        hdf5.read_dataset(path, "ids", hdf5.NONE, u)
    ids = hdf5.read_dataset(path, "ids", hdf5.NONE, hdf5.IdUnits())
    assert ids.dtype == np.uint64 and list(ids) == [0, 1, 2]


def test_files_and_directories(tmp_path):
    """A directory reads as its *.hdf5 files in name order, concatenated; a file without
    the dataset contributes no rows (src/io/input/mod.rs:75-97, 219-231)."""
    folder = tmp_path / "snap"
    folder.mkdir()
    parts = [np.arange(5.0), np.arange(5.0, 12.0), None, np.arange(12.0, 13.0)]
    for i, arr in enumerate(parts):
        w = H5Writer()
        if arr is not None:
            w.dataset("PartType0/Masses", arr, attrs=_ref_attrs(1.0, mass=1))
        else:
            w.dataset("PartType1/Masses", np.arange(3.0), attrs=_ref_attrs(1.0, mass=1))
        w.write(folder / f"snap_000.{i}.hdf5")
    (folder / "notes.txt").write_text("not read")
    out = hdf5.read_dataset(folder, "PartType0/Masses", hdf5.MASS)
    np.testing.assert_array_equal(out, np.arange(13.0))
    files = sorted(folder.glob("*.hdf5"))
    np.testing.assert_array_equal(hdf5.read_dataset(files[:2], "PartType0/Masses", hdf5.MASS), np.arange(12.0))
    assert hdf5.input_files(files[1]) == [files[1]]
    assert hdf5.read_dataset(files[2], "PartType0/Masses", hdf5.MASS).shape == (0,)
    with pytest.raises(hdf5.H5Error, match="Failed to open file"):
        hdf5.input_files(tmp_path / "missing")


def test_deflate_bytes_are_zlib(tmp_path):
    """The deflate filter's chunks are zlib streams (RFC 1950): what the writer stores is
    what zlib decodes, so the reader takes files written by the library."""
    w, path = _write(tmp_path)
    arr = np.arange(64, dtype=np.int32)
    w.dataset("x", arr, layout="chunked", chunks=(64,), filters=("deflate",))
    w.write(path)
    raw = path.read_bytes()
    stream = zlib.compress(arr.tobytes(), 6)
    assert raw.find(stream) > 0


def test_random_round_trips(tmp_path_factory):
    """Random datasets through the writer and the reader: shapes of rank 1 to 3, integer
    and float types of both byte orders, contiguous or chunked layouts with random
    chunk shapes and filter pipelines, and random row ranges."""
    hypothesis = pytest.importorskip("hypothesis")
    st = hypothesis.strategies

    dtypes = st.sampled_from(["<f8", ">f8", "<f4", ">f4", "<i4", ">i8", "<u2", "|u1", "<f2"])
    filters = st.sampled_from([(), ("deflate",), ("shuffle", "deflate"), ("shuffle", "deflate", "fletcher32")])

    @hypothesis.settings(max_examples=60, deadline=None)
    @hypothesis.given(shape=st.lists(st.integers(0, 9), min_size=1, max_size=3), dtype=dtypes,
                      chunked=st.booleans(), chunk_seed=st.integers(0, 2 ** 16), filt=filters,
                      fanout=st.sampled_from([None, 2, 5]), rows=st.tuples(st.integers(-12, 12), st.integers(-12, 12)))
    def check(shape, dtype, chunked, chunk_seed, filt, fanout, rows):
        rng = np.random.default_rng(chunk_seed)
        data = (rng.random(shape) * 200 - 100).astype(dtype)
        path = tmp_path_factory.mktemp("rt") / "x.hdf5"
        w = H5Writer()
        if chunked and all(s > 0 for s in shape):
            chunks = tuple(int(rng.integers(1, s + 1)) for s in shape)
            w.dataset("d", data, layout="chunked", chunks=chunks, filters=filt, btree_fanout=fanout)
        else:
            w.dataset("d", data)
        w.write(path)
        with hdf5.File(path) as f:
            np.testing.assert_array_equal(f["d"].read(), data)
            np.testing.assert_array_equal(f["d"].read(*rows), data[rows[0]:rows[1]])

    check()
