"""The mixed path's compact state (no task records or upwind slots, words by task, the
geometry kernel, directions split into task spaces) against the full state.

The geometry kernel classifies each task's faces and sums the upwind words in the
order and with the roundings of the record kernels, so a handle in the compact state
must agree with a full-state handle bit for bit: fields, levels, per-task rates and
dependency counts, over steps with dense and sparse sweeps, on periodic and
non-periodic grids, with one and with several task spaces.  The state is forced on
small grids with SUBSWEEP_COMPACT_STATE=1 (and SUBSWEEP_TASK_SPACES); the library
chooses it by itself for grids of 2^31 tasks or more or whose full state does not fit.
"""
import numpy as np
import pytest

from subsweep_gb300 import grid as gridmod, workloads
from subsweep_gb300.sweep import MEGAYEAR, Sweep, SweepError, SweepParameters, mass_density_from_number_density

pytestmark = pytest.mark.gpu


def _make(w, monkeypatch, compact: bool, spaces: int = 1):
    monkeypatch.delenv("SUBSWEEP_PULL_VARIANT", raising=False)
    if compact:
        monkeypatch.setenv("SUBSWEEP_COMPACT_STATE", "1")
        monkeypatch.setenv("SUBSWEEP_TASK_SPACES", str(spaces))
    else:
        monkeypatch.delenv("SUBSWEEP_COMPACT_STATE", raising=False)
        monkeypatch.delenv("SUBSWEEP_TASK_SPACES", raising=False)
    return Sweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
                 precision="mixed")


def _walled():
    """Poisson Voronoi cells in a walled box of 30 pc cells: boundary faces, no periodic
    ones, cells with many upwind faces."""
    n = 3000
    box = 30 * 3.0857e16 * n ** (1 / 3)
    pts = gridmod.poisson_points(n, box, 23)
    g = gridmod.voronoi(pts, box, periodic=False, nthreads=2)
    src = gridmod.place_sources(g, np.array([[box * 0.3, box * 0.6, box * 0.5]]), np.array([3e49]))
    params = SweepParameters(directions=32, num_timestep_levels=3, periodic=False, max_timestep=0.5 * MEGAYEAR,
                             significant_rate_threshold=1e-5)
    return workloads.Workload("walled", params, g, np.full(g.num_cells, float(mass_density_from_number_density(1e-2))),
                              np.full(g.num_cells, 1e-10), np.full(g.num_cells, 1e4), src, steps=6)


CASES = {
    # periodic jittered lattice, thin cells: the radiation crosses many cells and the
    # periodic faces; four levels give sparse sweeps above level 0
    "c2_periodic": lambda: workloads.c2_lognormal(n_per_side=12, num_directions=32, num_levels=4, nthreads=2),
    "c4_periodic": lambda: workloads.c4_grf(n_per_side=16, num_sources=2, num_directions=84, nthreads=2),
    # a batch of periodic Poisson boxes (block-diagonal grid)
    "c3_boxes": lambda: workloads.c3_batched(
        boxes=[workloads.c3_box(np.random.default_rng(17), 50 + b, 1500, 3000, nthreads=2) for b in range(2)],
        num_directions=32, num_levels=3),
    "walled": _walled,
}


@pytest.mark.parametrize("spaces", [1, 3])
@pytest.mark.parametrize("name", sorted(CASES))
def test_compact_state_equals_full_state(name, spaces, monkeypatch):
    w = CASES[name]()
    full = _make(w, monkeypatch, compact=False)
    comp = _make(w, monkeypatch, compact=True, spaces=spaces)
    st = comp.stats()
    assert st["task_spaces"] == spaces and st["pull_variant"] == 0
    assert full.stats()["task_spaces"] == 0
    for _ in range(6):
        assert comp.run_sweeps() == full.run_sweeps()
        np.testing.assert_array_equal(comp.cell_state()["level"], full.cell_state()["level"])
    ff, fc = full.fields(), comp.fields()
    for k in ff:
        np.testing.assert_array_equal(fc[k], ff[k], err_msg=k)
    rf, rc = full.rates(), comp.rates()
    for k in rf:
        np.testing.assert_array_equal(rc[k], rf[k], err_msg=k)
    for level in range(w.params.num_timestep_levels):
        np.testing.assert_array_equal(comp.dependency_counts(level), full.dependency_counts(level))
    assert comp.stats()["tasks"] == full.stats()["tasks"]
    full.close()
    comp.close()


def test_compact_state_checkpoint(monkeypatch):
    """A checkpoint of a compact-state handle restores into another with the same
    spaces, and a full-state handle refuses it (its words are ordered differently)."""
    w = CASES["c2_periodic"]()
    a = _make(w, monkeypatch, compact=True, spaces=2)
    for _ in range(2):
        a.run_sweeps()
    state = a.save_state()
    times_a = [a.run_sweeps() for _ in range(2)]
    fa = a.fields()
    b = _make(w, monkeypatch, compact=True, spaces=2)
    b.load_state(state)
    assert [b.run_sweeps() for _ in range(2)] == times_a
    fb = b.fields()
    for k in fa:
        np.testing.assert_array_equal(fb[k], fa[k], err_msg=k)
    c = _make(w, monkeypatch, compact=False)
    with pytest.raises(SweepError):
        c.load_state(state)
    for h in (a, b, c):
        h.close()


def test_compact_state_graph_replay(monkeypatch):
    """Steps of a compact-state handle replayed as CUDA graphs (one geometry launch per
    sweep over three task spaces, captured with its barrier reset) equal direct steps."""
    w = CASES["c2_periodic"]()
    monkeypatch.setenv("SUBSWEEP_COMPACT_STATE", "1")
    monkeypatch.setenv("SUBSWEEP_TASK_SPACES", "3")
    mk = lambda graphs: Sweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
                              precision="mixed", use_graphs=graphs)
    direct, replay = mk(False), mk(True)
    for _ in range(6):
        assert replay.run_sweeps() == direct.run_sweeps()
    assert replay.stats()["graph_launches"] > 0
    fd, fr = direct.fields(), replay.fields()
    for k in fd:
        np.testing.assert_array_equal(fr[k], fd[k], err_msg=k)
    direct.close()
    replay.close()
