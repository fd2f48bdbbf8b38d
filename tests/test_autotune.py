"""Autotuning of the mixed path's transport kernel.

The first dense sweeps of a handle try each candidate variant (the lockstep kernel with
2 lanes per task at 2 target blocks per SM, with 4 lanes per task at 3, and at 4 with
the next block's slots brought into L1 only) and keep the fastest per task.
Every variant sums in the same order, so a tuned
handle, with or without graph replay after tuning, matches a handle fixed on the
default variant bit for bit.
"""
import numpy as np
import pytest

from subsweep_gb300 import workloads
from subsweep_gb300.sweep import Sweep

pytestmark = pytest.mark.gpu

CANDIDATES = {122, 143, 344}


@pytest.mark.parametrize("use_graphs", [False, True])
def test_autotuned_equals_fixed(use_graphs, monkeypatch):
    monkeypatch.delenv("SUBSWEEP_PULL_VARIANT", raising=False)
    monkeypatch.delenv("SUBSWEEP_AUTOTUNE", raising=False)
    w = workloads.c2_lognormal(n_per_side=12, num_directions=32, num_levels=4, nthreads=2, thick=True)
    mk = lambda tune, graphs: Sweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature,
                                    w.source, precision="mixed", autotune=tune, use_graphs=graphs)
    tuned, fixed = mk(True, use_graphs), mk(False, False)
    # the first steps have 1, 1, 2, 4 and 8 sweeps; tuning needs one dense sweep per
    # candidate and every step opens with one, so it ends within the three warm-up steps
    # a benchmark runs
    steps = 8
    for _ in range(steps):
        assert tuned.run_sweeps() == fixed.run_sweeps()
    ft, ff = tuned.fields(), fixed.fields()
    for k in ft:
        np.testing.assert_array_equal(ft[k], ff[k], err_msg=k)
    st = tuned.stats()
    assert st["pull_variant"] in CANDIDATES
    assert fixed.stats()["pull_variant"] == 143  # the default: 4 lanes per task, 3 blocks per SM
    if use_graphs:
        assert steps - 3 <= st["graph_launches"] < steps  # replay starts once tuning is done
    tuned.close()
    fixed.close()


def _poisson_boxes():
    """Poisson Voronoi boxes: cells with more than 16 upwind faces occur, so the slots
    beyond the registers are exercised."""
    rng = np.random.default_rng(17)
    return workloads.c3_batched(boxes=[workloads.c3_box(rng, 50 + b, 1500, 3000, nthreads=2) for b in range(2)],
                                num_directions=32, num_levels=3)


@pytest.mark.parametrize("variant", [83, 72, 78, 122, 322, 323, 143, 144, 164, 242, 264, 283, 343, 344, 384, 1084, 1143, 1242, 1344,
                                     2242, 2283])
@pytest.mark.parametrize("grid", ["lattice", "poisson"])
def test_variant_equals_default(variant, grid, monkeypatch):
    """Each transport variant (the lockstep kernel at 2, 4, 8 and 16 lanes per task,
    prefetch depths 1 to 3, 2 to 4 target blocks per SM, with and without streaming
    loads, with and without the next block's words loaded one block ahead; the
    level-synchronous wavefront and its fully TMA-staged form) against the
    lockstep kernel with 8 lanes per task at 4 blocks per SM, bit for bit over steps
    with dense and sparse sweeps above level 0."""
    monkeypatch.delenv("SUBSWEEP_AUTOTUNE", raising=False)
    if grid == "lattice":
        w = workloads.c2_lognormal(n_per_side=12, num_directions=32, num_levels=4, nthreads=2, thick=True)
    else:
        w = _poisson_boxes()
    mk = lambda: Sweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
                       precision="mixed", autotune=False)
    monkeypatch.setenv("SUBSWEEP_PULL_VARIANT", "184")
    ref = mk()
    monkeypatch.setenv("SUBSWEEP_PULL_VARIANT", str(variant))
    var = mk()
    for _ in range(6):
        assert var.run_sweeps() == ref.run_sweeps()
        np.testing.assert_array_equal(var.cell_state()["level"], ref.cell_state()["level"])
    fv, fr = var.fields(), ref.fields()
    for k in fr:
        np.testing.assert_array_equal(fv[k], fr[k], err_msg=k)
    assert var.stats()["pull_variant"] == variant
    ref.close()
    var.close()
