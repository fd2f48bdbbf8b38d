"""The runtime's own host logic, without a device: its TimestepState (sweep_host.cpp,
exported as sw_host_* for these checks) against the reference's level-scheduling
known answers (src/sweep/timestep_state.rs:98-137), and the oracle's restatement
against it for every level count."""
import ctypes
import json
import pathlib

import numpy as np
import pytest

from oracle import binding
from subsweep_gb300 import _native

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "reference_kats.json"


@pytest.fixture(scope="module")
def lib():
    lib = _native.load_gpu()
    lib.sw_host_sweep_order.restype = ctypes.c_int32
    lib.sw_host_sweep_order.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32]
    lib.sw_host_lowest_allowed.restype = ctypes.c_int32
    lib.sw_host_lowest_allowed.argtypes = [ctypes.c_int32, ctypes.c_int32]
    return lib


def order(lib, levels, advances):
    out = np.zeros(1 << levels, np.int32)
    k = lib.sw_host_sweep_order(levels, advances, out.ctypes.data, out.size)
    assert 0 < k <= out.size
    return out[:k].tolist()


def test_sweep_order_and_lowest_allowed_kat(lib):
    so = json.loads(GOLDEN.read_text())["sweep_order"]
    for adv, expected in enumerate(so["orders_after_advances"]):
        assert order(lib, so["num_levels"], adv) == expected, adv
    for adv, expected in enumerate(so["lowest_allowed_after_advances"]):
        assert lib.sw_host_lowest_allowed(so["num_levels"], adv) == expected, adv


@pytest.mark.parametrize("levels", [1, 2, 3, 4, 6])
def test_runtime_and_oracle_schedule_agree(lib, levels):
    orc = binding.load()
    for adv in range(levels + 3):
        out = np.zeros(1 << levels, np.int32)
        k = orc.orc_sweep_order_after(levels, adv, out.ctypes.data, out.size)
        assert order(lib, levels, adv) == out[:k].tolist()
        assert lib.sw_host_lowest_allowed(levels, adv) == orc.orc_lowest_allowed_after(levels, adv)
        # every step opens at the lowest allowed level, which every cell's level is floored
        # at: the first sweep of a step covers every cell
        assert order(lib, levels, adv)[0] == lib.sw_host_lowest_allowed(levels, adv)


def test_invalid_arguments(lib):
    out = np.zeros(4, np.int32)
    assert lib.sw_host_sweep_order(0, 0, out.ctypes.data, 4) == -1
    assert lib.sw_host_sweep_order(17, 0, out.ctypes.data, 4) == -1
    assert lib.sw_host_sweep_order(3, -1, out.ctypes.data, 4) == -1
    assert lib.sw_host_sweep_order(3, 0, None, 4) == -1
    assert lib.sw_host_lowest_allowed(0, 0) == -1
    # a short buffer gets the first entries and the full count
    assert lib.sw_host_sweep_order(3, 5, out.ctypes.data, 2) == 4


def _checkpoint(num_cells=10, directions=4, levels=3, np_=32, precision=1, rate_bytes=4, level_fill=1):
    """A checkpoint buffer laid out as sw_save_state writes it: the header, seven
    per-cell double arrays, the per-cell levels, then the per-task sections."""
    import struct
    header = struct.pack("<QIIqqiiIIdiiIIQ", 0x3154504357535553, 2, precision, num_cells, 7 * num_cells,
                         directions, levels, np_, rate_bytes, 0.0, 0, 1, 5, 4, 0)
    nd = np_ * directions
    tail = nd * rate_bytes + (nd * 12 + num_cells * 4 if precision == 1 else 3 * nd * rate_bytes)
    buf = bytearray(header + bytes(7 * 8 * num_cells) + bytes([level_fill]) * num_cells + bytes(tail))
    return buf, len(header) + 7 * 8 * num_cells


def test_checkpoint_validation_rejects_bad_level_before_upload(lib):
    """sw_load_state's host-side validation: a checkpoint whose level section holds a
    level >= num_timestep_levels is refused (it would index the device's per-level
    histograms out of range), as are a bad header and a short buffer."""
    lib.sw_host_check_checkpoint.restype = ctypes.c_int32
    lib.sw_host_check_checkpoint.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    for precision, rate_bytes in ((1, 4), (0, 8)):
        buf, level_off = _checkpoint(precision=precision, rate_bytes=rate_bytes)
        assert lib.sw_host_check_checkpoint(bytes(buf), len(buf)) == 0
        bad = bytearray(buf)
        bad[level_off + 7] = 3  # one cell at level 3 of 3 levels
        assert lib.sw_host_check_checkpoint(bytes(bad), len(bad)) == 3
        bad[level_off + 7] = 255
        assert lib.sw_host_check_checkpoint(bytes(bad), len(bad)) == 3
        assert lib.sw_host_check_checkpoint(bytes(buf), len(buf) - 1) == 2
        assert lib.sw_host_check_checkpoint(bytes(buf[:40]), 40) == 2
        magic = bytearray(buf)
        magic[0] ^= 1
        assert lib.sw_host_check_checkpoint(bytes(magic), len(magic)) == 1
    # a header whose timestep state or counts no handle can have
    buf, _ = _checkpoint(levels=17)
    assert lib.sw_host_check_checkpoint(bytes(buf), len(buf)) == 1
    buf, _ = _checkpoint(num_cells=40, np_=32)
    assert lib.sw_host_check_checkpoint(bytes(buf), len(buf)) == 1


def _schedule(lib, level, np_, n, d, levels, groups):
    lib.sw_host_schedule_order.restype = ctypes.c_int64
    lib.sw_host_schedule_order.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                           ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_int64]
    order = np.zeros(n * d, np.uint32)
    seg = np.zeros(groups * levels + 1, np.uint32)
    k = lib.sw_host_schedule_order(level.ctypes.data, np_, n, d, levels, groups, order.ctypes.data,
                                   seg.ctypes.data, seg.size)
    return k, order, seg[:k + 1] if k >= 0 else seg


@pytest.mark.parametrize("groups", [1, 2, 3, 5])
def test_schedule_order_layout(lib, groups):
    """The positions sw_create lays out: every task (padding cells excluded) once; the
    direction groups one after another, each by level, in task-id order inside a
    segment; every segment one (group, level); the layout is deterministic."""
    rng = np.random.default_rng(groups)
    n, np_, d, levels = 45, 64, 7, 9
    level = rng.integers(0, levels, size=np_ * d).astype(np.uint16)
    k, order, seg = _schedule(lib, level, np_, n, d, levels, groups)
    tasks = np.array([t for t in range(np_ * d) if t % np_ < n], np.uint32)
    assert k >= 1 and seg[0] == 0 and seg[-1] == n * d
    np.testing.assert_array_equal(np.sort(order), tasks)
    bounds = [d * g // groups for g in range(groups + 1)]  # direction groups: [d*g/G, d*(g+1)/G)
    group_of = lambda t: next(g for g in range(groups) if bounds[g] <= t // np_ < bounds[g + 1])
    keys = []
    for s in range(k):
        part = order[seg[s]:seg[s + 1]]
        assert len(part) > 0 and np.all(np.diff(part.astype(np.int64)) > 0)  # task-id order
        gs, ls = {group_of(int(t)) for t in part}, {int(level[t]) for t in part}
        assert len(gs) == 1 and len(ls) == 1  # one (group, level) per segment
        keys.append((gs.pop(), ls.pop()))
    assert keys == sorted(keys) and len(set(keys)) == len(keys)
    k2, order2, seg2 = _schedule(lib, level, np_, n, d, levels, groups)
    assert k2 == k and np.array_equal(order2, order) and np.array_equal(seg2, seg)


def test_schedule_order_rejects_bad_input(lib):
    level = np.zeros(64 * 4, np.uint16)
    assert _schedule(lib, level, 64, 40, 4, 3, 5)[0] == -1  # more groups than directions
    level[3] = 7
    assert _schedule(lib, level, 64, 40, 4, 3, 1)[0] == -1  # a level beyond the count


def test_task_spaces_and_direction_groups(lib, monkeypatch):
    """The compact state's task spaces (fewer than 2^31 tasks each) and the schedule's
    direction groups (one per 40 K tasks of the average Kahn level) at the benchmark
    configurations' sizes."""
    lib.sw_host_task_spaces.restype = ctypes.c_int32
    lib.sw_host_task_spaces.argtypes = [ctypes.c_uint32, ctypes.c_int32]
    lib.sw_host_dir_groups.restype = ctypes.c_int32
    lib.sw_host_dir_groups.argtypes = [ctypes.c_int32, ctypes.c_uint64, ctypes.c_int64]
    np_ = lambda n: (n + 31) // 32 * 32
    assert lib.sw_host_task_spaces(np_(256 ** 3), 84) == 1  # C4: 1.41 G tasks
    assert lib.sw_host_task_spaces(np_(384 ** 3), 84) == 3  # C5: 4.76 G tasks, 28 directions a space
    assert lib.sw_host_task_spaces(np_((1 << 30) - 1), 84) == 0  # beyond eight spaces
    assert lib.sw_host_task_spaces(0, 84) == -1
    monkeypatch.delenv("SUBSWEEP_DIR_GROUPS", raising=False)
    assert lib.sw_host_dir_groups(84, 256 ** 3 * 84, 4927) == 7  # C4 256^3: 286 K tasks per level
    assert lib.sw_host_dir_groups(84, 64 ** 3 * 84, 1200) == 1  # 64^3: 18 K tasks per level
    assert lib.sw_host_dir_groups(84, 10, 5) == 1
    assert lib.sw_host_dir_groups(0, 10, 5) == -1
