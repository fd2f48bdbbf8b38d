"""ctypes bindings of the in-tree native libraries (include/subsweep_gpu.h and the
host grid producers).  Loading fails loudly if a library has not been built."""
from __future__ import annotations

import ctypes
import pathlib

from . import build as _build

c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_double = ctypes.c_double
c_void_p = ctypes.c_void_p
P_double = ctypes.POINTER(ctypes.c_double)

SW_OK = 0
SW_ERR_INVALID_ARG = 1
SW_ERR_CUDA = 2
SW_ERR_STALLED = 3
SW_ERR_OOM = 4
SW_ERR_UNSUPPORTED = 5
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "CUDA", 3: "STALLED", 4: "OOM", 5: "UNSUPPORTED"}

SW_PRECISION_FP64 = 0
SW_PRECISION_MIXED = 1

SW_FACE_LOCAL = 0
SW_FACE_LOCAL_PERIODIC = 1
SW_FACE_BOUNDARY = 2

# Every entry point declared in include/subsweep_gpu.h.
ABI_SYMBOLS = (
    "sw_default_params", "sw_directions_from_num", "sw_create", "sw_step", "sw_get_fields",
    "sw_get_cell_state", "sw_set_fields", "sw_get_level_counts", "sw_get_dependency_counts",
    "sw_get_rates", "sw_get_stats", "sw_last_error", "sw_destroy", "sw_get_dependency_counts_noalloc",
    "sw_get_time_series", "sw_checkpoint_size", "sw_save_state", "sw_load_state", "sw_create_batch",
)


class SwParams(ctypes.Structure):
    _fields_ = [
        ("num_directions", c_int32),
        ("explicit_directions", P_double),
        ("num_timestep_levels", c_int32),
        ("periodic", c_int32),
        ("max_timestep", c_double),
        ("rotate_directions", c_int32),
        ("significant_rate_threshold", c_double),
        ("timestep_safety_factor", c_double),
        ("chemistry_timestep_safety_factor", c_double),
        ("check_deadlock", c_int32),
        ("prevent_cooling", c_int32),
        ("num_tasks_to_solve_before_send_receive", c_int64),
        ("scale_factor", c_double),
        ("precision", c_int32),
        ("device", c_int32),
        ("use_graphs", c_int32),
        ("autotune", c_int32),
    ]


class SwGridCsr(ctypes.Structure):
    _fields_ = [
        ("num_cells", c_int64),
        ("row_ptr", c_void_p),
        ("nbr", c_void_p),
        ("kind", c_void_p),
        ("area", c_void_p),
        ("normal", c_void_p),
        ("volume", c_void_p),
        ("size", c_void_p),
    ]


class SwCellInit(ctypes.Structure):
    _fields_ = [
        ("density", c_void_p),
        ("ionized_hydrogen_fraction", c_void_p),
        ("temperature", c_void_p),
        ("source", c_void_p),
    ]


class SwTimeSeries(ctypes.Structure):
    _fields_ = [(name, ctypes.c_double) for name in (
        "hydrogen_ionization_mass_average", "hydrogen_ionization_volume_average",
        "temperature_mass_average", "temperature_volume_average",
        "photoionization_rate_volume_average", "weighted_photoionization_rate_volume_average")]


class SwStats(ctypes.Structure):
    _fields_ = [
        ("steps", c_int64),
        ("level_sweeps", c_int64),
        ("tasks", c_int64),
        ("chem_cells", c_int64),
        ("chem_attempts", c_int64),
        ("chem_failures", c_int64),
        ("sweep_ms", c_double),
        ("chem_ms", c_double),
        ("level_ms", c_double),
        ("simulation_time", c_double),
        ("step_ms", c_double),
        ("transport_kernel_ms", c_double),
        ("transport_launches", c_int64),
        ("kernel_launches", c_int64),
        ("levelled_sweeps", c_int64),
        ("schedule_levels", c_int64),
        ("transport_attempts", c_int64),
        ("upwind_slots", c_int64),
        ("graph_launches", c_int64),
        ("pull_variant", c_int64),
        ("task_spaces", c_int64),
        ("device_bytes", c_int64),
    ]


_gpu = None
_grid = None


def gpu_library_path() -> pathlib.Path:
    return _build.GPU_LIB


def load_gpu() -> ctypes.CDLL:
    """Load libsubsweep_gpu.so (build it first with subsweep_gb300.build.build())."""
    global _gpu
    if _gpu is not None:
        return _gpu
    path = _build.GPU_LIB
    if not path.exists():
        raise RuntimeError(f"{path} is missing: the CUDA sweep library has not been built "
                           "(run `python -c 'import __graft_entry__ as g; g.build()'`)")
    lib = ctypes.CDLL(str(path))
    lib.sw_default_params.argtypes = [ctypes.POINTER(SwParams)]
    lib.sw_directions_from_num.argtypes = [c_int32, c_void_p]
    lib.sw_create.argtypes = [ctypes.POINTER(SwParams), ctypes.POINTER(SwGridCsr),
                              ctypes.POINTER(SwCellInit), ctypes.POINTER(c_void_p)]
    lib.sw_step.argtypes = [c_void_p, P_double]
    lib.sw_get_fields.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
    lib.sw_get_cell_state.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p]
    lib.sw_set_fields.argtypes = [c_void_p, c_void_p, c_void_p]
    lib.sw_get_level_counts.argtypes = [c_void_p, c_void_p]
    lib.sw_get_dependency_counts.argtypes = [c_void_p, c_int32, c_void_p]
    lib.sw_get_rates.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p]
    lib.sw_get_dependency_counts_noalloc.argtypes = [c_void_p, c_int32, c_void_p]
    lib.sw_get_stats.argtypes = [c_void_p, ctypes.POINTER(SwStats)]
    lib.sw_get_time_series.argtypes = [c_void_p, ctypes.POINTER(SwTimeSeries)]
    lib.sw_checkpoint_size.argtypes = [c_void_p, ctypes.POINTER(ctypes.c_size_t)]
    lib.sw_create_batch.argtypes = [ctypes.POINTER(SwParams), c_int32, ctypes.POINTER(SwGridCsr),
                                    ctypes.POINTER(SwCellInit), ctypes.POINTER(c_void_p)]
    lib.sw_save_state.argtypes = [c_void_p, c_void_p, ctypes.c_size_t]
    lib.sw_load_state.argtypes = [c_void_p, c_void_p, ctypes.c_size_t]
    lib.sw_last_error.argtypes = [c_void_p]
    lib.sw_last_error.restype = ctypes.c_char_p
    lib.sw_destroy.argtypes = [c_void_p]
    lib.sw_destroy.restype = None
    # GPU Voronoi producer (csrc/voronoi_gpu.h)
    lib.sw_gpu_grid_voronoi.restype = c_void_p
    lib.sw_gpu_grid_voronoi.argtypes = [c_void_p, c_int64, c_void_p, c_int32, c_int32]
    lib.sw_gpu_grid_status.restype = c_int32
    lib.sw_gpu_grid_status.argtypes = [c_void_p]
    for f in ("sw_gpu_grid_num_faces", "sw_gpu_grid_failed_cells", "sw_gpu_grid_dropped_faces"):
        getattr(lib, f).restype = c_int64
        getattr(lib, f).argtypes = [c_void_p]
    lib.sw_gpu_grid_copy.argtypes = [c_void_p] + [c_void_p] * 7
    lib.sw_gpu_grid_copy.restype = None
    lib.sw_gpu_grid_free.argtypes = [c_void_p]
    lib.sw_gpu_grid_free.restype = None
    for name in ABI_SYMBOLS:
        fn = getattr(lib, name)
        if fn.restype is ctypes.c_int:  # default restype: sw_status
            fn.restype = c_int32
    _gpu = lib
    return lib


def load_grid() -> ctypes.CDLL:
    global _grid
    if _grid is not None:
        return _grid
    path = _build.GRID_LIB
    if not path.exists():
        raise RuntimeError(f"{path} is missing: build the native libraries first")
    lib = ctypes.CDLL(str(path))
    lib.sw_grid_voronoi.restype = c_void_p
    lib.sw_grid_voronoi.argtypes = [c_void_p, c_int64, c_void_p, c_int32, c_int32]
    lib.sw_grid_cartesian.restype = c_void_p
    lib.sw_grid_cartesian.argtypes = [c_int32, c_int32, c_int32, c_double, c_int32]
    for f in ("sw_grid_num_cells", "sw_grid_num_faces", "sw_grid_failed_cells", "sw_grid_dropped_faces"):
        getattr(lib, f).restype = c_int64
        getattr(lib, f).argtypes = [c_void_p]
    lib.sw_grid_copy.argtypes = [c_void_p] + [c_void_p] * 8
    lib.sw_grid_copy.restype = None
    lib.sw_grid_free.argtypes = [c_void_p]
    lib.sw_grid_free.restype = None
    _grid = lib
    return lib
