"""The C-ABI library: loads, exports every symbol include/subsweep_gpu.h declares, and
its host-only entry points (defaults, direction tables, argument validation) behave
like the reference.  No compute call needs a GPU here."""
import ctypes
import hashlib
import pathlib
import re
import struct

import numpy as np
import pytest

from subsweep_gb300 import _native, grid as gridmod
from subsweep_gb300.sweep import Sweep, SweepError, SweepParameters

ROOT = pathlib.Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for header in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(sw_\w+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol():
    lib = _native.load_gpu()
    declared = declared_symbols()
    assert declared == set(_native.ABI_SYMBOLS)
    for name in declared:
        assert getattr(lib, name) is not None


def test_default_params_match_reference_defaults():
    """SweepParameters serde defaults (src/sweep/parameters.rs:64-78)."""
    lib = _native.load_gpu()
    p = _native.SwParams()
    assert lib.sw_default_params(ctypes.byref(p)) == 0
    assert p.rotate_directions == 0
    assert p.significant_rate_threshold == 0.0
    assert p.timestep_safety_factor == pytest.approx(0.1)
    assert p.chemistry_timestep_safety_factor == pytest.approx(0.1)
    assert p.check_deadlock == 0 and p.prevent_cooling == 1
    assert p.num_tasks_to_solve_before_send_receive == 10000
    assert p.precision == _native.SW_PRECISION_FP64


@pytest.mark.parametrize("num", [1, 16, 21, 32, 64, 84])
def test_direction_tables_match_reference(kats, num):
    lib = _native.load_gpu()
    out = np.zeros(3 * num)
    assert lib.sw_directions_from_num(num, out.ctypes.data) == 0
    digest = hashlib.sha256(struct.pack("<%dd" % out.size, *out)).hexdigest()
    assert digest == kats["direction_tables"][str(num)]


def test_unknown_direction_count_rejected():
    lib = _native.load_gpu()
    out = np.zeros(3 * 20)
    assert lib.sw_directions_from_num(20, out.ctypes.data) == _native.SW_ERR_INVALID_ARG


def _small():
    g = gridmod.cartesian(3, 3, 3, 1.0, False)
    n = g.num_cells
    return g, dict(density=np.full(n, 1e-24), ionized_hydrogen_fraction=np.full(n, 1e-10),
                   temperature=np.full(n, 1e4), source=np.zeros(n))


def test_rotate_directions_unsupported():
    g, init = _small()
    p = SweepParameters(directions=16, num_timestep_levels=1, periodic=False, max_timestep=1.0,
                        rotate_directions=True)
    with pytest.raises(SweepError) as e:
        Sweep(p, g, **init)
    assert e.value.status == _native.SW_ERR_UNSUPPORTED


def test_bad_direction_count_rejected():
    g, init = _small()
    p = SweepParameters(directions=17, num_timestep_levels=1, periodic=False, max_timestep=1.0)
    with pytest.raises(SweepError) as e:
        Sweep(p, g, **init)
    assert e.value.status == _native.SW_ERR_INVALID_ARG


def test_non_reciprocal_normals_rejected():
    g, init = _small()
    g.normal[1] = [0.0, 0.0, 1.0]  # x+ face of cell 0 (a LOCAL face)
    p = SweepParameters(directions=16, num_timestep_levels=1, periodic=False, max_timestep=1.0)
    with pytest.raises(SweepError) as e:
        Sweep(p, g, **init)
    assert e.value.status == _native.SW_ERR_INVALID_ARG


def test_fully_ionized_initial_state_with_prevent_cooling_rejected():
    """The reference's f64::clamp panics when the x_HII floor exceeds 1 - 1e-10."""
    g, init = _small()
    init["ionized_hydrogen_fraction"] = np.ones(g.num_cells)
    p = SweepParameters(directions=16, num_timestep_levels=1, periodic=False, max_timestep=1.0)
    with pytest.raises(SweepError) as e:
        Sweep(p, g, **init)
    assert e.value.status == _native.SW_ERR_INVALID_ARG


def test_cycle_detected_by_check_deadlock():
    """check_deadlock (deadlock_detection.rs analogue): a 3-cell dependency cycle with
    antisymmetric normals is rejected at creation."""
    g = _cyclic_grid()
    n = g.num_cells
    p = SweepParameters(directions=[[0.0, 0.0, 1.0]], num_timestep_levels=1, periodic=False,
                        max_timestep=1.0, check_deadlock=True)
    with pytest.raises(SweepError) as e:
        Sweep(p, g, density=np.full(n, 1e-24), ionized_hydrogen_fraction=np.full(n, 1e-10),
              temperature=np.full(n, 1e4), source=np.zeros(n))
    assert e.value.status == _native.SW_ERR_STALLED


def _cyclic_grid():
    """Three cells, each face normal tilted so that for d = +z cell 0 -> 1 -> 2 -> 0."""
    tilt = 0.6
    pairs = [(0, 1), (1, 2), (2, 0)]
    faces = {0: [], 1: [], 2: []}
    for a, b in pairs:
        nrm = np.array([0.8, 0.0, tilt])  # a -> b is downwind for +z
        faces[a].append((b, nrm))
        faces[b].append((a, -nrm))
    row, nbr, nrms = [0], [], []
    for c in range(3):
        for b, nrm in faces[c]:
            nbr.append(b)
            nrms.append(nrm)
        row.append(len(nbr))
    e = len(nbr)
    return gridmod.Grid(row_ptr=np.array(row, np.int64), nbr=np.array(nbr, np.int32),
                        kind=np.zeros(e, np.uint8), area=np.ones(e), normal=np.array(nrms),
                        volume=np.ones(3), size=np.ones(3), position=np.zeros((3, 3)),
                        box_size=np.ones(3), periodic=False)


def test_stats_fields_used_by_smoke_and_bench():
    """smoke() and bench.py read these sw_stats fields by name."""
    from subsweep_gb300 import _native
    names = {n for n, _ in _native.SwStats._fields_}
    for k in ("tasks", "chem_cells", "level_sweeps", "step_ms", "transport_kernel_ms", "transport_launches",
              "kernel_launches", "levelled_sweeps", "schedule_levels", "transport_attempts", "chem_attempts",
              "sweep_ms", "chem_ms", "level_ms", "pull_variant", "graph_launches", "task_spaces"):
        assert k in names, k


def _create_sized(num_cells, directions, precision):
    lib = _native.load_gpu()
    p = _native.SwParams()
    assert lib.sw_default_params(ctypes.byref(p)) == 0
    p.num_directions = directions
    p.precision = precision
    g = _native.SwGridCsr()
    g.num_cells = num_cells  # arrays left NULL: never read
    init = _native.SwCellInit()
    h = ctypes.c_void_p()
    st = lib.sw_create(ctypes.byref(p), ctypes.byref(g), ctypes.byref(init), ctypes.byref(h))
    assert not h.value
    return st, lib.sw_last_error(None)


def test_task_id_limits_checked_before_any_allocation():
    """The C5 stress configuration (384^3 cells x 84 directions = 4.76 G tasks) exceeds
    32-bit task ids.  The FP64 path rejects it from the sizes alone; the mixed path
    accepts the sizes (its compact state splits the directions into task spaces) and
    stops at the NULL arrays, before reading one or touching the device; a grid that
    would need more than eight task spaces is rejected."""
    directions = 84
    st, msg = _create_sized(384 ** 3, directions, _native.SW_PRECISION_FP64)
    assert st == _native.SW_ERR_UNSUPPORTED and b"2^32" in msg
    st, msg = _create_sized(384 ** 3, directions, _native.SW_PRECISION_MIXED)
    assert st == _native.SW_ERR_INVALID_ARG and b"NULL" in msg
    st, msg = _create_sized((1 << 30) - 1, directions, _native.SW_PRECISION_MIXED)
    assert st == _native.SW_ERR_UNSUPPORTED and b"task spaces" in msg


def test_no_device_fails_loudly():
    """Without a usable CUDA device a valid handle cannot be created: SW_ERR_CUDA with the
    runtime's message, never a CPU fallback (on a GPU machine there is nothing to test)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    g, init = _small()
    p = SweepParameters(directions=16, num_timestep_levels=1, periodic=False, max_timestep=1.0)
    with pytest.raises(SweepError) as e:
        Sweep(p, g, **init, precision="mixed")
    assert e.value.status == _native.SW_ERR_CUDA
    assert str(e.value)
