"""The oracle against the reference's own known-answer tests (tests/golden/reference_kats.json,
extracted from the reference's test modules by tests/golden/gen_reference_kats.py)."""
import ctypes
import math

import numpy as np
import pytest

from oracle import binding

RATE_FITS = {  # orc_rate_fit selectors, hydrogen_only/mod.rs:175-273
    "case_b_recombination_rate": 0, "case_b_recombination_rate_derivative": 1,
    "collisional_ionization_rate": 2, "collisional_ionization_rate_derivative": 3,
    "collisional_ionization_cooling_rate": 4, "collisional_ionization_cooling_rate_derivative": 5,
    "collisional_excitation_cooling_rate": 6, "collisional_excitation_cooling_rate_derivative": 7,
    "case_b_recombination_cooling_rate": 8, "case_b_recombination_cooling_rate_derivative": 9,
    "bremsstrahlung_cooling_rate": 10, "bremsstrahlung_cooling_rate_derivative": 11,
    "compton_cooling_rate": 12, "compton_cooling_rate_derivative": 13,
}


def test_timestep_level_kat(kats):
    lib = binding.load()
    for case in kats["timestep_level"]:
        got = lib.orc_timestep_level(case["max_num_levels"], case["max_timestep"], case["desired"])
        assert got == case["level"], case


def test_timestep_level_saturating_cast():
    lib = binding.load()
    assert lib.orc_timestep_level(4, 1.0, float("nan")) == 0
    assert lib.orc_timestep_level(4, 1.0, float("inf")) == 0
    assert lib.orc_timestep_level(4, 1.0, 0.0) == 3
    assert lib.orc_timestep_level(4, 1.0, 0.25) == 2   # exact power of two
    assert lib.orc_timestep_level(4, 1.0, 0.2499999) == 3


def test_sweep_order_kat(kats):
    lib = binding.load()
    so = kats["sweep_order"]
    for adv, expected in enumerate(so["orders_after_advances"]):
        out = np.zeros(1 << so["num_levels"], np.int32)
        k = lib.orc_sweep_order_after(so["num_levels"], adv, out.ctypes.data, out.size)
        assert list(out[:k]) == expected
    for adv, expected in enumerate(so["lowest_allowed_after_advances"]):
        assert lib.orc_lowest_allowed_after(so["num_levels"], adv) == expected


def test_rate_fit_derivatives_kat(kats):
    """Port of test_numerical_derivative (hydrogen_only/mod.rs:491-591)."""
    lib = binding.load()
    dt = kats["derivative_test"]
    assert len(dt["pairs"]) == 7
    for fname, dname in dt["pairs"]:
        for t in dt["temperatures"]:
            analytical = lib.orc_rate_fit(RATE_FITS[dname], t, 1.0)
            v1 = lib.orc_rate_fit(RATE_FITS[fname], t, 1.0)
            v2 = lib.orc_rate_fit(RATE_FITS[fname], t + dt["delta"], 1.0)
            numerical = (v2 - v1) / dt["delta"]
            rel = abs(analytical - numerical) / (abs(analytical) + abs(numerical) + 1e-50)
            assert rel < dt["epsilon"], (fname, t, analytical, numerical)


@pytest.mark.parametrize("name", ["fully_ionized_solver", "fully_neutral_solver"])
def test_solver_extremes_kat(kats, name):
    """fully_ionized_solver / fully_neutral_solver (hydrogen_only/mod.rs:948-984): no panic."""
    lib = binding.load()
    e = kats["solver_extremes"][name]
    x = ctypes.c_double(e["ionized_hydrogen_fraction"])
    t = ctypes.c_double(e["temperature_K"])
    density = e["density_g_per_cm3"] * 1e-3 / 1e-6
    length = e["length_kpc"] * 1000 * 3.0857e16
    ts, proc = ctypes.c_double(), ctypes.c_int32()
    lib.orc_solver_perform_timestep(ctypes.byref(x), ctypes.byref(t), density, e["volume_m3"], length,
                                    e["rate_per_s"], e["scale_factor"], 0, 0.0, 0.0,
                                    e["timestep_Myr"] * 1e6 * 3.15576e7, e["safety"], ctypes.byref(ts),
                                    ctypes.byref(proc))
    assert 1e-10 <= x.value <= 1.0 - 1e-10
    assert math.isfinite(t.value) or math.isnan(t.value)


def test_outgoing_rate_threshold():
    lib = binding.load()
    rho = 1e3 * 1.67262192369e-27
    assert lib.orc_outgoing_rate(rho, 0.0, 1.0, 1e-6, 1e-5) == 0.0
    v = lib.orc_outgoing_rate(rho, 0.5, 1e20, 10.0, 1e-5)
    expected = 10.0 * math.exp(-(rho / 1.67262192369e-27 * 0.5) * 2.9580524545305314e-18 * 1e-4 * 1e20)
    assert v == pytest.approx(expected, rel=1e-15)
