"""Checkpoint and restart of the evolving state (sw_save_state / sw_load_state).

A handle runs two steps, is checkpointed and runs two more; a second handle created
from the same inputs loads the checkpoint and runs the same two steps.  The mixed path
is deterministic (fixed summation order), so its fields, levels and time series agree
bit for bit; the FP64 drop-in sums corrections with atomics in arrival order, so it
agrees within 1e-10.  A checkpoint is refused by a handle built on another grid.
"""
import numpy as np
import pytest

from subsweep_gb300 import workloads
from subsweep_gb300.sweep import Sweep, SweepError

pytestmark = pytest.mark.gpu


def make(w, precision):
    return Sweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
                 precision=precision)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_restart_continues_identically(precision):
    w = workloads.c2_lognormal(n_per_side=10, num_directions=16, num_levels=3, nthreads=2)
    a = make(w, precision)
    times_a = [a.run_sweeps() for _ in range(2)]
    state = a.save_state()
    times_a += [a.run_sweeps() for _ in range(2)]
    fa, la = a.fields(), a.cell_state()["level"]

    b = make(w, precision)
    b.load_state(state)
    times_b = [b.run_sweeps() for _ in range(2)]
    fb, lb = b.fields(), b.cell_state()["level"]
    assert times_b == times_a[2:]
    np.testing.assert_array_equal(lb, la)
    if precision == "mixed":
        for k in ("ionized_hydrogen_fraction", "temperature", "timestep", "photon_rate"):
            np.testing.assert_array_equal(fb[k], fa[k], err_msg=k)
        assert b.time_series() == a.time_series()
    else:
        for k in ("ionized_hydrogen_fraction", "temperature"):
            np.testing.assert_allclose(fb[k], fa[k], rtol=1e-10, err_msg=k)
    a.close()
    b.close()


def test_checkpoint_refused_by_another_grid():
    w = workloads.c2_lognormal(n_per_side=8, num_directions=16, num_levels=3, nthreads=2)
    other = workloads.c2_lognormal(n_per_side=9, num_directions=16, num_levels=3, nthreads=2)
    a, b = make(w, "mixed"), make(other, "mixed")
    a.run_sweeps()
    with pytest.raises(SweepError):
        b.load_state(a.save_state())
    with pytest.raises(SweepError):
        b.load_state(np.zeros(16, np.uint8))
    a.close()
    b.close()
