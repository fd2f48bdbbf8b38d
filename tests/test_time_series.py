"""Time-series reductions (compute_time_series_system, src/sweep/time_series.rs:61-155).

CPU: the oracle's restatement against an independent numpy evaluation of the same
formulas from the oracle's own fields and rates.  GPU: sw_get_time_series of the FP64
drop-in against the oracle within 1e-10 relative (only the summation order differs),
the mixed path within 1e-4, and the device reduction against numpy over the library's
own exported fields.
"""
import numpy as np
import pytest

from oracle import binding
from subsweep_gb300 import workloads
from subsweep_gb300.sweep import Sweep

from test_gpu_parity import oracle_dirs

PROTON_MASS = 1.67262192369e-27
SIGMA = 2.9580524545305314e-18 * 1e-4  # m^2
YEAR = 3.15576e7


def reference_series(x, temperature, density, volume, size, cell_rate):
    """The six outputs from per-cell arrays (cell rate = sum over directions of
    incoming + source/D + periodic, photons/s)."""
    mass = density * volume
    nhn = density / PROTON_MASS * (1.0 - x)
    absorbed = 1.0 - np.exp(-nhn * SIGMA * size)
    gamma = ((YEAR * cell_rate) * absorbed / (nhn * volume)) / YEAR
    return {
        "hydrogen_ionization_mass_average": np.sum(mass * x) / np.sum(mass),
        "hydrogen_ionization_volume_average": np.sum(volume * x) / np.sum(volume),
        "temperature_mass_average": np.sum(temperature * mass) / np.sum(mass),
        "temperature_volume_average": np.sum(temperature * volume) / np.sum(volume),
        "photoionization_rate_volume_average": np.sum(gamma * volume) / np.sum(volume),
        "weighted_photoionization_rate_volume_average": np.sum(gamma * x * volume) / np.sum(volume),
    }


def small_workload():
    return workloads.c2_lognormal(n_per_side=8, num_directions=16, num_levels=3, nthreads=2)


def oracle_for(w):
    return binding.OracleSweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
                               oracle_dirs(w.params))


def cell_rates_from(rates, source, num_directions):
    return (rates["incoming"] + (source / num_directions)[:, None] + rates["periodic"]).sum(axis=1)


def test_oracle_time_series_matches_formulas():
    w = small_workload()
    orc = oracle_for(w)
    for _ in range(3):
        orc.run_sweeps()
    f = orc.fields()
    expect = reference_series(f["ionized_hydrogen_fraction"], f["temperature"], w.density, w.grid.volume,
                              w.grid.size, cell_rates_from(orc.rates(), w.source, 16))
    got = orc.time_series()
    assert set(got) == set(binding.TIME_SERIES_NAMES)
    for k, v in expect.items():
        assert got[k] == pytest.approx(v, rel=1e-12), k
    assert 0.0 < got["hydrogen_ionization_volume_average"] < 1.0
    assert got["photoionization_rate_volume_average"] > 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-10), ("mixed", 1e-4)])
def test_gpu_time_series_vs_oracle(precision, rtol):
    w = small_workload()
    gpu = Sweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
                precision=precision)
    orc = oracle_for(w)
    for step in range(3):
        gpu.run_sweeps()
        orc.run_sweeps()
        got, expect = gpu.time_series(), orc.time_series()
        for k in binding.TIME_SERIES_NAMES:
            assert got[k] == pytest.approx(expect[k], rel=rtol), f"step {step} {k}"
    # the device reduction against numpy over the library's own exported state
    f = gpu.fields()
    mine = reference_series(f["ionized_hydrogen_fraction"], f["temperature"], w.density, w.grid.volume,
                            w.grid.size, cell_rates_from(gpu.rates(), w.source, 16))
    got = gpu.time_series()
    for k in binding.TIME_SERIES_NAMES:
        # the mixed path's carried neutral fraction differs from 1 - x in the last bits
        assert got[k] == pytest.approx(mine[k], rel=1e-12 if precision == "fp64" else 1e-6), k
    gpu.close()
