"""The allocation-free dependency-count export (sw_get_dependency_counts_noalloc).

It serves callers that cannot allocate device memory themselves or let a library do
it mid-run (a host engine that owns all GPU memory through its own pool, code that
must avoid the synchronisation a cudaMalloc/cudaFree can cause).  It must return
exactly what sw_get_dependency_counts returns, through the C ABI, on consecutive calls
that share its fixed scratch array.  This file sorts last so that a run stopping at
the first failure has already run every other test.
"""

import numpy as np
import pytest

from subsweep_gb300 import _native, workloads
from subsweep_gb300.sweep import Sweep

pytestmark = pytest.mark.gpu


def _noalloc_counts(sweep: Sweep, level: int) -> np.ndarray:
    lib = _native.load_gpu()
    out = np.full((sweep.num_cells, sweep.num_directions), 0xAB, np.uint8)
    st = lib.sw_get_dependency_counts_noalloc(sweep._h, level, out.ctypes.data)
    assert st == _native.SW_OK, lib.sw_last_error(sweep._h).decode()
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_counts_match_allocating_entry_point(precision):
    w = workloads.c2_lognormal(n_per_side=10, num_directions=84, num_levels=4, nthreads=2, thick=True)
    s = Sweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
              precision=precision)
    for _ in range(3):  # spread the cells over several timestep levels
        s.run_sweeps()
    levels = s.cell_state()["level"]
    assert len(np.unique(levels)) > 1
    # two calls in a row: the second reuses (and must first clear) the shared array;
    # level 3 leaves inactive cells whose entries must read zero
    for level in (0, 3):
        np.testing.assert_array_equal(_noalloc_counts(s, level), s.dependency_counts(level))
    s.close()


def test_noalloc_rejects_problems_beyond_its_scratch():
    w = workloads.c1_small_periodic(n_per_side=64, num_directions=84, nthreads=8)
    s = Sweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source)
    lib = _native.load_gpu()
    out = np.zeros((s.num_cells, s.num_directions), np.uint8)
    st = lib.sw_get_dependency_counts_noalloc(s._h, 0, out.ctypes.data)
    assert st == _native.SW_ERR_INVALID_ARG
    assert b"scratch" in lib.sw_last_error(s._h)
    s.close()
