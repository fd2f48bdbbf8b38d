"""The reference's free chemistry evolution runs (time_evolution_free,
src/chemistry/hydrogen_only/mod.rs:882-920, `#[ignore]`, CSV output only) on the
oracle's solver: a 1 pc cell, rate = photon flux x (1 pc)^2, 10 kyr steps of
Solver::perform_timestep with safety 0.1 (the harness of mod.rs:646-721), for the
reference's fluxes (0 and 1e5 photons/s/cm^2) over initial fractions, temperatures and
densities of its grid.  The reference writes the states out and asserts nothing; here
the runs are shortened to 20 Myr and the physical end states are checked: every step
converges inside the physical range, optically thin gas under the flux ionizes, dense
gas under it reaches an ionization equilibrium that forgets the initial state, and
dense gas without it recombines and cools.  CPU only."""
import ctypes
import math

import numpy as np
import pytest

from oracle import binding

PARSEC = 3.0857e16          # m
YEAR = 3.15576e7            # s
PROTON_MASS = 1.67262192369e-27
LENGTH, VOLUME = PARSEC, PARSEC ** 3
AREA_CM2 = PARSEC ** 2 * 1e4
STEPS = 2000                # x 10 kyr = 20 Myr

FRACTIONS = (1e-10, 0.5, 1.0)
TEMPERATURES = (1e3, 1.6e4, 1e6)
DENSITIES = (1e-8, 1e-4, 1e0, 1e2)  # hydrogen number density, cm^-3


def evolve(flux: float, n_h: float, x0: float, t0: float):
    lib = binding.load()
    x, t = ctypes.c_double(x0), ctypes.c_double(t0)
    ts, proc = ctypes.c_double(), ctypes.c_int32()
    density = n_h * 1e6 * PROTON_MASS  # kg / m^3
    failures = 0
    for _ in range(STEPS):
        failures += lib.orc_solver_perform_timestep(ctypes.byref(x), ctypes.byref(t), density, VOLUME, LENGTH,
                                                    flux * AREA_CM2, 1.0, 0, 0.0, 0.0, 1e4 * YEAR, 0.1,
                                                    ctypes.byref(ts), ctypes.byref(proc))
        assert 0.0 <= x.value <= 1.0 and math.isfinite(t.value) and t.value > 0.0
    return x.value, t.value, failures


@pytest.fixture(scope="module")
def runs():
    return {(f, n, x0, t0): evolve(f, n, x0, t0)
            for f in (0.0, 1e5) for n in DENSITIES for x0 in FRACTIONS for t0 in TEMPERATURES}


def test_every_step_converges(runs):
    assert all(r[2] == 0 for r in runs.values())


def test_optically_thin_gas_ionizes_under_flux(runs):
    for n in (1e-8, 1e-4):
        for x0 in FRACTIONS:
            for t0 in TEMPERATURES:
                assert runs[(1e5, n, x0, t0)][0] > 0.999, (n, x0, t0)


@pytest.mark.parametrize("n", [1e0, 1e2])
def test_dense_gas_under_flux_forgets_its_initial_state(runs, n):
    ends = np.array([runs[(1e5, n, x0, t0)][:2] for x0 in FRACTIONS for t0 in TEMPERATURES])
    assert 0.0 < ends[:, 0].min() < 0.5
    # initial states 1e3..1e6 K and x 1e-10..1 end within 2 % of each other (the coldest
    # start at 100 cm^-3 is still relaxing thermally at 20 Myr: 1.03 %)
    np.testing.assert_allclose(ends, np.broadcast_to(ends[-1], ends.shape), rtol=0.02)


@pytest.mark.parametrize("n", [1e0, 1e2])
def test_dense_gas_without_flux_recombines_and_cools(runs, n):
    for x0 in FRACTIONS:
        for t0 in (1.6e4, 1e6):
            x, t, _ = runs[(0.0, n, x0, t0)]
            assert x < 0.01 and t < 1e4, (n, x0, t0, x, t)
