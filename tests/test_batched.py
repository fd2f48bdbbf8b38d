"""C3: independent periodic boxes run as one block-diagonal grid.

A batch must compute, for every box, what the box alone computes.  CPU: the union's
structure, and the oracle on the batch against the oracle on each box (FP64; the
oracle's task heap interleaves boxes, which only reorders additions).  GPU: the mixed
path on the batch against the mixed path on each box, bit for bit in x_HII, T, the
species timestep and the levels.
"""
import numpy as np
import pytest

from oracle import binding
from subsweep_gb300 import grid as gridmod, workloads
from subsweep_gb300.sweep import Sweep, SweepError

from test_gpu_parity import oracle_dirs


def small_boxes(k=3, seed=11):
    rng = np.random.default_rng(seed)
    return [workloads.c3_box(rng, seed * 7 + b, min_cells=200, max_cells=900, nthreads=2) for b in range(k)]


def single(box, batch):
    g, n_h, src = box
    return workloads.c3_batched(boxes=[(g, n_h, src)], num_directions=batch.params.num_directions(),
                                num_levels=batch.params.num_timestep_levels)


def test_concatenate_structure():
    boxes = small_boxes()
    u = gridmod.concatenate([b[0] for b in boxes])
    off = np.cumsum([0] + [b[0].num_cells for b in boxes])
    assert u.num_cells == off[-1] and u.num_faces == sum(b[0].num_faces for b in boxes)
    owner = np.repeat(np.arange(u.num_cells), np.diff(u.row_ptr))
    box_of = np.searchsorted(off, np.arange(u.num_cells), side="right") - 1
    local = u.kind <= 1
    np.testing.assert_array_equal(box_of[u.nbr[local]], box_of[owner[local]])
    for b, (g, _, _) in enumerate(boxes):
        faces = slice(u.row_ptr[off[b]], u.row_ptr[off[b + 1]])
        np.testing.assert_array_equal(u.area[faces], g.area)
        np.testing.assert_array_equal(u.nbr[faces][g.kind <= 1] - off[b], g.nbr[g.kind <= 1])


def oracle_for(w):
    return binding.OracleSweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
                               oracle_dirs(w.params))


def test_oracle_batch_equals_boxes():
    boxes = small_boxes()
    batch = workloads.c3_batched(boxes=boxes, num_directions=16)
    ob = oracle_for(batch)
    singles = [oracle_for(single(b, batch)) for b in boxes]
    for _ in range(3):
        ob.run_sweeps()
        for o in singles:
            o.run_sweeps()
    fb = ob.fields()
    off = np.cumsum([0] + [b[0].num_cells for b in boxes])
    for k, o in enumerate(singles):
        fs = o.fields()
        sl = slice(off[k], off[k + 1])
        for key in ("ionized_hydrogen_fraction", "temperature"):
            np.testing.assert_allclose(fb[key][sl], fs[key], rtol=1e-10, err_msg=f"box {k} {key}")
        np.testing.assert_array_equal(fb["level"][sl], fs["level"])


@pytest.mark.gpu
def test_gpu_batch_equals_boxes_bitwise():
    boxes = small_boxes(k=3, seed=12)
    batch = workloads.c3_batched(boxes=boxes, num_directions=32)

    def make(w):
        return Sweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
                     precision="mixed")

    gb = make(batch)
    gs = [make(single(b, batch)) for b in boxes]
    for _ in range(4):
        tb = gb.run_sweeps()
        for g in gs:
            assert g.run_sweeps() == tb
    fb, lb = gb.fields(), gb.cell_state()["level"]
    off = np.cumsum([0] + [b[0].num_cells for b in boxes])
    for k, g in enumerate(gs):
        fs, ls = g.fields(), g.cell_state()["level"]
        sl = slice(off[k], off[k + 1])
        np.testing.assert_array_equal(lb[sl], ls)
        for key in ("ionized_hydrogen_fraction", "temperature", "timestep"):
            np.testing.assert_array_equal(fb[key][sl], fs[key], err_msg=f"box {k} {key}")
        # a box that skips the step's last sweep alone reports its stored incoming rate,
        # in the batch the rate gathered from its neighbours (another summation order)
        np.testing.assert_allclose(fb["photon_rate"][sl], fs["photon_rate"], rtol=1e-6)
        g.close()
    gb.close()


def test_batch_rejects_neighbour_outside_box():
    """sw_create_batch checks every box's neighbour ids before offsetting them (no CUDA
    call is made for an invalid batch)."""
    boxes = small_boxes(k=2, seed=13)
    g, n_h, src = boxes[1]
    bad = gridmod.Grid(**{**g.__dict__, "nbr": g.nbr.copy()})
    bad.nbr[np.flatnonzero(bad.kind == 0)[0]] = bad.num_cells  # one past the box
    w = workloads.c3_batched(boxes=boxes, num_directions=16)
    dens = w.density[: boxes[0][0].num_cells]
    args = [(boxes[0][0], dens, 1e-10, 1e4, boxes[0][2]), (bad, w.density[boxes[0][0].num_cells:], 1e-10, 1e4, src)]
    with pytest.raises(SweepError) as e:
        Sweep.batch(w.params, args, precision="mixed")
    assert "outside the box" in str(e.value)


@pytest.mark.gpu
def test_create_batch_equals_union():
    boxes = small_boxes(k=3, seed=14)
    w = workloads.c3_batched(boxes=boxes, num_directions=32)
    off = np.cumsum([0] + [b[0].num_cells for b in boxes])
    args = [(b[0], w.density[off[k]:off[k + 1]], 1e-10, 1e4, b[2]) for k, b in enumerate(boxes)]
    a = Sweep.batch(w.params, args, precision="mixed")
    u = Sweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source, precision="mixed")
    assert a.num_cells == u.num_cells
    for _ in range(3):
        assert a.run_sweeps() == u.run_sweeps()
    fa, fu = a.fields(), u.fields()
    for k in fa:
        np.testing.assert_array_equal(fa[k], fu[k], err_msg=k)
    a.close()
    u.close()
