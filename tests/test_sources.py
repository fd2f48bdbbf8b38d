"""Point sources from a snapshot's star particles (subsweep_gb300.arepo.read_sources,
bpass_lookup, source_rates; subsweep_gb300.cosmology), on the CPU.

Pinned to the reference's own tests, extracted by tests/golden/gen_reference_kats.py:
the BPASS lookup cases (src/arepo_postprocess/bpass.rs tests) and the cosmological
time differences (src/cosmology.rs tests).  The BPASS table is checked against its
generator's source of truth by the same values at the table's nodes.
"""
import json
import pathlib

import numpy as np
import pytest

from subsweep_gb300 import arepo, bpass_table
from subsweep_gb300.cosmology import YEAR, Cosmology
from hdf5_writer import H5Writer

KATS = json.loads((pathlib.Path(__file__).resolve().parent / "golden" / "reference_kats.json").read_text())


def test_bpass_reference_kats():
    k = KATS["bpass"]
    for case in k["cases"]:
        got = float(arepo.bpass_lookup(case["age_years"] * YEAR, case["metallicity"], arepo.SOLAR_MASS))
        want = case["photons_per_s"]
        assert abs((got - want) / (abs(got) + abs(want))) < k["relative_tolerance"], case


def test_bpass_interpolation():
    ages = np.asarray(bpass_table.AGE_BINS)
    mets = np.asarray(bpass_table.METALLICITY_BINS)
    table = np.asarray(bpass_table.TABLE)
    assert table.shape == (51, 13) and np.all(np.diff(ages) > 0) and np.all(np.diff(mets) > 0)
    # at interior nodes the lookup returns the table entry itself
    for i in (3, 20, 40):
        for j in (2, 6, 10):
            got = arepo.bpass_lookup(ages[i] * YEAR, mets[j], arepo.SOLAR_MASS)
            assert got == table[i, j]
    # linear in age between nodes, linear in the rate per mass in metallicity
    mid_age = 0.5 * (ages[10] + ages[11])
    np.testing.assert_allclose(arepo.bpass_lookup(mid_age * YEAR, mets[4], arepo.SOLAR_MASS),
                               0.5 * (table[10, 4] + table[11, 4]), rtol=1e-12)
    # proportional to the mass; clamped outside the table
    np.testing.assert_allclose(arepo.bpass_lookup(ages[5] * YEAR, mets[3], 3.0 * arepo.SOLAR_MASS),
                               3.0 * table[5, 3], rtol=1e-15)
    young = arepo.bpass_lookup(1.0, 1e-9, arepo.SOLAR_MASS)
    np.testing.assert_allclose(young, arepo.bpass_lookup(ages[0] * 1.00001 * YEAR, mets[0] * 1.00001,
                                                         arepo.SOLAR_MASS), rtol=0)
    vec = arepo.bpass_lookup(np.array([1e6, 1e8, 1e10]) * YEAR, np.array([1e-4, 0.01, 0.02]),
                             np.full(3, arepo.SOLAR_MASS))
    assert vec.shape == (3,) and np.all(np.diff(vec) < 0)  # older populations emit less


def test_cosmology_reference_kats():
    k = KATS["cosmology"]
    c = Cosmology(a=1.0, h=k["h"], omega_0=k["omega_0"], omega_lambda=k["omega_lambda"])
    assert c.time_difference_between_scalefactors(1.0, 1.0) == 0.0
    t = k["time_difference"]
    got = c.time_difference_between_scalefactors(t["a0"], t["a1"])
    assert abs(got - t["gigayears"] * 1e9 * YEAR) < t["tolerance_years"] * YEAR
    grid = k["round_trip_scale_factors"]
    for a0 in grid:
        for a1 in grid:
            dt = c.time_difference_between_scalefactors(a0, a1)
            assert abs(c.scalefactor_after(a0, dt) - a1) < k["round_trip_tolerance"]
    with pytest.raises(NotImplementedError, match="flat"):
        Cosmology(a=1.0, h=0.7, omega_0=0.5, omega_lambda=0.7).time_difference_between_scalefactors(0.5, 1.0)
    with pytest.raises(ValueError, match="non cosmological"):
        Cosmology(a=1.0, h=0.7).time_difference_between_scalefactors(0.5, 1.0)


def _arepo_attrs(to_cgs, length=0, mass=0, velocity=0, a=0, h=0):
    return {"to_cgs": np.float64(to_cgs), "length_scaling": np.float64(length), "mass_scaling": np.float64(mass),
            "velocity_scaling": np.float64(velocity), "a_scaling": np.float64(a), "h_scaling": np.float64(h)}


def test_read_sources_from_star_particles(tmp_path):
    """Stars in Arepo's comoving units; wind particles (formation scale factor <= 0)
    dropped; rates = BPASS(age from the formation scale factor) * escape fraction."""
    rng = np.random.default_rng(3)
    n = 40
    kpc, msun10 = 3.085678e21, 1.989e43
    pos = rng.uniform(0, 1e4, (n, 3))
    met = rng.uniform(1e-4, 0.03, n)
    a_form = rng.uniform(0.05, 0.49, n)
    a_form[[3, 11]] = [0.0, -0.2]  # wind
    mass = rng.uniform(1e-5, 1e-3, n)
    w = H5Writer()
    w.dataset("PartType4/Coordinates", pos, attrs=_arepo_attrs(kpc, length=1, a=1, h=-1))
    w.dataset("PartType4/GFM_Metallicity", met, attrs=_arepo_attrs(0.0))
    w.dataset("PartType4/GFM_StellarFormationTime", a_form, attrs=_arepo_attrs(0.0))
    w.dataset("PartType4/Masses", mass, attrs=_arepo_attrs(msun10, mass=1, h=-1))
    w.write(tmp_path / "snap.hdf5")
    c = Cosmology(a=0.5, h=0.6774, omega_0=0.308983, omega_lambda=0.6911)
    got_pos, got_rates = arepo.read_sources(tmp_path / "snap.hdf5", c, escape_fraction=0.2)
    keep = a_form > 0
    f_len = (1.0 / (0.5 ** -1 * 0.6774 ** 1)) * 0.01 * kpc
    f_mass = (1.0 / (0.6774 ** 1)) * 0.001 * msun10
    np.testing.assert_array_equal(got_pos, pos[keep] * f_len)
    ages = np.array([c.time_difference_between_scalefactors(a, 0.5) for a in a_form[keep]])
    assert np.all(ages > 0)
    np.testing.assert_array_equal(got_rates, arepo.bpass_lookup(ages, met[keep], mass[keep] * f_mass) * 0.2)
    assert got_rates.shape == (n - 2,) and np.all(got_rates > 0)


def test_source_rates_on_nearest_cells():
    rng = np.random.default_rng(8)
    cells = rng.uniform(0, 1, (200, 3))
    src = rng.uniform(0, 1, (50, 3))
    rates = rng.uniform(1e48, 1e50, 50)
    got = arepo.source_rates(cells, src, rates)
    nearest = ((src[:, None, :] - cells[None, :, :]) ** 2).sum(-1).argmin(1)
    want = np.zeros(200)
    for i, r in zip(nearest, rates):  # in source order, as the reference adds them
        want[i] += r
    np.testing.assert_array_equal(got, want)
    assert arepo.source_rates(cells, np.zeros((0, 3)), np.zeros(0)).sum() == 0.0
