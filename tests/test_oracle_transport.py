"""Self-validation of the oracle's transport (no reference golden vectors exist for it):
the analytic attenuation of a 1-D column (examples/sweep_1d.rs setting) and flux
conservation of the push-form corrections."""
import math

import numpy as np
import pytest

from oracle import binding
from subsweep_gb300 import workloads, grid as gridmod
from subsweep_gb300.sweep import SweepParameters, MEGAYEAR, PARSEC, mass_density_from_number_density

SIGMA = 2.9580524545305314e-18 * 1e-4
PROTON_MASS = 1.67262192369e-27


def test_column_attenuation_is_analytic():
    n, s, n_h, S = 40, 1e3 * PARSEC, 5e-5, 1e50
    w = workloads.cartesian_column(n, s, n_h, S)
    w.params.significant_rate_threshold = 0.0
    o = binding.OracleSweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature,
                            w.source, np.array([[1.0, 0.0, 0.0]]))
    o.run_sweeps()
    r = o.rates()
    rho = w.density[0]
    q = math.exp(-(rho / PROTON_MASS * (1.0 - 1e-10)) * SIGMA * s)
    expected_out = S * q ** np.arange(1, n + 1)
    np.testing.assert_allclose(r["outgoing"][:, 0], expected_out, rtol=1e-12)
    np.testing.assert_allclose(r["incoming"][1:, 0], expected_out[:-1], rtol=1e-12)
    assert r["incoming"][0, 0] == 0.0


def test_flux_conservation_periodic_voronoi():
    box = 1.0 * 3.0857e22 / 4
    pts = gridmod.jittered_lattice(8, box, 0.25, 11)
    g = gridmod.voronoi(pts, box, periodic=True, nthreads=1)
    n = g.num_cells
    src = gridmod.place_sources(g, np.array([[box / 2] * 3]), np.array([1e50]))
    params = SweepParameters(directions=16, num_timestep_levels=1, periodic=True, max_timestep=MEGAYEAR)
    dirs = np.array(__import__("subsweep_gb300").directions_from_num(16))
    o = binding.OracleSweep(params, g, np.full(n, float(mass_density_from_number_density(1e-5))),
                            np.full(n, 1e-10), np.full(n, 1e4), src, dirs)
    o.run_sweeps()
    r = o.rates()
    # first step from zero state: every outgoing rate is delivered to a local or periodic
    # neighbour, so per direction sum(incoming) + sum(periodic) == sum(outgoing)
    lhs = r["incoming"].sum(0) + r["periodic"].sum(0)
    rhs = r["outgoing"].sum(0)
    np.testing.assert_allclose(lhs, rhs, rtol=1e-12)
    assert (rhs > 0).all()


def test_periodic_snapshot_vs_immediate_deviation_is_bounded():
    """The reference makes periodic contributions visible in task order (unstable heap);
    the snapshot semantics defer them to the next sweep.  After a few steps both agree
    closely on this small box (the deviation is reported, not pinned)."""
    w = workloads.c1_small_periodic(n_per_side=6, num_directions=16, nthreads=1)
    dirs = __import__("subsweep_gb300").directions_from_num(16)
    outs = []
    for mode in (binding.PERIODIC_SNAPSHOT, binding.PERIODIC_IMMEDIATE):
        o = binding.OracleSweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature,
                                w.source, dirs, periodic_mode=mode)
        for _ in range(3):
            o.run_sweeps()
        outs.append(o.fields())
    dx = np.abs(outs[0]["ionized_hydrogen_fraction"] - outs[1]["ionized_hydrogen_fraction"]).max()
    assert dx < 0.05
