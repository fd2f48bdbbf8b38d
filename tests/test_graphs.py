"""Steps replayed from a CUDA graph (use_graphs) against direct launches.

The graph holds the same launches with the sweep numbers and the end time read from
the device, so fields, levels, rates and the time series agree bit for bit.  A
dependency cycle still reports SW_ERR_STALLED (the error flag stays set across the
step's sweeps and is read at its end).
"""
import numpy as np
import pytest

from subsweep_gb300 import _native, workloads
from subsweep_gb300.sweep import Sweep, SweepError, SweepParameters

pytestmark = pytest.mark.gpu


def make(w, use_graphs):
    # without autotuning every step is replayed (tuning runs its trial sweeps directly)
    return Sweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
                 precision="mixed", use_graphs=use_graphs, autotune=False)


@pytest.mark.parametrize("name", ["c2", "c3"])
def test_graph_steps_equal_direct_steps(name):
    if name == "c2":
        w = workloads.c2_lognormal(n_per_side=12, num_directions=32, num_levels=4, nthreads=2, thick=True)
    else:
        rng = np.random.default_rng(5)
        boxes = [workloads.c3_box(rng, 40 + b, min_cells=200, max_cells=1500, nthreads=2) for b in range(4)]
        w = workloads.c3_batched(boxes=boxes)
    direct, graph = make(w, False), make(w, True)
    for step in range(6):
        assert graph.run_sweeps() == direct.run_sweeps()
        np.testing.assert_array_equal(graph.cell_state()["level"], direct.cell_state()["level"])
    fd, fg = direct.fields(), graph.fields()
    for k in fd:
        np.testing.assert_array_equal(fg[k], fd[k], err_msg=k)
    rd, rg = direct.rates(), graph.rates()
    for k in rd:
        np.testing.assert_array_equal(rg[k], rd[k], err_msg=k)
    assert graph.time_series() == direct.time_series()
    st = graph.stats()
    assert st["graph_launches"] == 6 and st["tasks"] == direct.stats()["tasks"]
    direct.close()
    graph.close()


def test_fp64_graph_steps_match_direct_steps():
    """The push path replayed from a graph: its FP64 atomics sum in arrival order, so
    graph and direct steps agree to rounding, levels exactly."""
    w = workloads.c2_lognormal(n_per_side=10, num_directions=16, num_levels=3, nthreads=2)
    mk = lambda g: Sweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
                         precision="fp64", use_graphs=g)
    direct, graph = mk(False), mk(True)
    for _ in range(4):
        assert graph.run_sweeps() == direct.run_sweeps()
    np.testing.assert_array_equal(graph.cell_state()["level"], direct.cell_state()["level"])
    fd, fg = direct.fields(), graph.fields()
    for k in ("ionized_hydrogen_fraction", "temperature"):
        np.testing.assert_allclose(fg[k], fd[k], rtol=1e-10, err_msg=k)
    assert graph.stats()["graph_launches"] == 4
    direct.close()
    graph.close()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_graph_step_reports_stall(precision):
    from tests.test_abi import _cyclic_grid
    g = _cyclic_grid()
    n = g.num_cells
    p = SweepParameters(directions=[[0.0, 0.0, 1.0]], num_timestep_levels=1, periodic=False, max_timestep=1.0)
    s = Sweep(p, g, density=np.full(n, 1e-24), ionized_hydrogen_fraction=np.full(n, 1e-10),
              temperature=np.full(n, 1e4), source=np.zeros(n), precision=precision, use_graphs=True)
    with pytest.raises(SweepError) as e:
        s.run_sweeps()
    assert e.value.status == _native.SW_ERR_STALLED
    s.close()
