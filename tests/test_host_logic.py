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
