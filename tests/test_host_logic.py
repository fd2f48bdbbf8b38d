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
