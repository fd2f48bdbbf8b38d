"""The benchmark configurations' generators (subsweep_gb300/workloads.py) at small sizes,
on the CPU: the parameters each configuration states, the source totals, the density
normalisation and the labels the benchmark prints."""
import numpy as np
import pytest

from subsweep_gb300 import workloads
from subsweep_gb300.sweep import MEGAYEAR, mass_density_from_number_density


def _mean_n_h(w):
    return float(np.mean(w.density / mass_density_from_number_density(1.0)))


def test_c4_generator_parameters():
    w = workloads.c4_grf(n_per_side=8, num_sources=20, nthreads=2)
    p = w.params
    assert p.num_timestep_levels == 4 and p.num_directions() == 84 and p.periodic
    assert p.max_timestep == pytest.approx(MEGAYEAR) and p.significant_rate_threshold == 1e-5
    assert w.grid.num_cells == 8 ** 3 and w.steps == 4
    assert float(w.source.sum()) == pytest.approx(1e52, rel=1e-12)
    assert np.count_nonzero(w.source) == 20
    assert _mean_n_h(w) == pytest.approx(2e-4, rel=1e-9)
    # the sources sit on the densest cells, with rates in proportion to their density
    peaks = np.argsort(w.density)[-20:]
    assert set(np.flatnonzero(w.source)) == set(peaks)
    np.testing.assert_allclose(w.source[peaks] / w.density[peaks], w.source[peaks[0]] / w.density[peaks[0]],
                               rtol=1e-12)
    assert w.name == workloads.label("c4", 8)


def test_c5_generator_parameters():
    """C5, the stress configuration: C4's field with ln-sigma 2.0, 4000 sources (all
    cells of a small grid), 6 levels, 20 steps of 1 Myr, threshold 1e-5."""
    w = workloads.c5_grf(n_per_side=8, nthreads=2)
    p = w.params
    assert p.num_timestep_levels == 6 and p.num_directions() == 84 and p.periodic
    assert p.significant_rate_threshold == 1e-5 and w.steps == 20
    assert p.max_timestep * w.steps == pytest.approx(20 * MEGAYEAR)
    assert float(w.source.sum()) == pytest.approx(4e52, rel=1e-12)
    assert _mean_n_h(w) == pytest.approx(2e-4, rel=1e-9)
    assert w.name == workloads.label("c5", 8)
    assert "C5" in w.name and "ln-sigma 2.0" in w.name
    # a wider field than C4's at the same seed and size
    c4 = workloads.c4_grf(n_per_side=8, seed=5, num_sources=20, nthreads=2)
    assert np.std(np.log(w.density)) > np.std(np.log(c4.density))


def test_labels_without_building():
    """The CPU reference arm names the full-size workload from its parameters alone."""
    assert workloads.label("c4") == workloads.label("c4", 256, 84, 4)
    assert workloads.label("c5").startswith("C5 periodic jittered-lattice Voronoi 384^3")
    with pytest.raises(ValueError):
        workloads.label("c6")
