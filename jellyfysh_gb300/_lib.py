"""ctypes binding of ``libjfgpu.so`` (declared in ``include/jfgpu.h``).

The library is the product's compute path; there is no CPU fallback.  ``load()`` raises ``LibraryMissing`` when the
shared library has not been built and ``NoGpu`` when no CUDA device is visible, so that a caller on a GPU machine
fails loudly instead of silently computing something else.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIBRARY_PATH = os.environ.get("JFGPU_LIBRARY") or os.path.join(HERE, "_build", "libjfgpu.so")

OK = 0
ERROR_NAMES = {0: "ok", 1: "CUDA runtime error", 2: "invalid argument", 3: "device allocation failed",
               4: "table construction failed"}

STATUS_OK, STATUS_VALUE_ERROR, STATUS_ASSERTION, STATUS_ZERO_DIVISION, STATUS_COMPLEX = 0, 1, 2, 3, 4
STATUS_CELL_RANGE, STATUS_EVENT_CAP, STATUS_LIFTING, STATUS_INDEX = 7, 8, 9, 10
STATUS_NAMES = {0: "ok", 1: "ValueError", 2: "AssertionError", 3: "ZeroDivisionError", 4: "complex result",
                7: "cell index out of range", 8: "refinement overflow", 9: "LiftingSchemeError", 10: "IndexError"}
LIFTING_INSIDE_FIRST, LIFTING_OUTSIDE_FIRST, LIFTING_RATIO = 0, 1, 2
DRAW_VALUE, DRAW_UNIT = 0, 1

POT_HARD_SPHERE, POT_LENNARD_JONES, POT_COULOMB = 0, 1, 2
FAR_NONE, FAR_CELL_VETO, FAR_CELL_BOUNDING = 0, 1, 2
MODE_EXACT, MODE_MIXED = 0, 1
EV_PAIR, EV_BOUNDED, EV_HARDCORE, EV_CELL_BOUNDING, EV_CELL_VETO, EV_BOUNDARY, EV_END_OF_CHAIN = range(7)
EV_BOND, EV_COMPOSITE = 8, 9


class LibraryMissing(RuntimeError):
    pass


class NoGpu(RuntimeError):
    pass


class JfgpuError(RuntimeError):
    pass


class CompositeDesc(ctypes.Structure):
    """JfgpuCompositeDesc."""
    _fields_ = [("units", ctypes.c_int32), ("lifting", ctypes.c_int32), ("fourier_cutoff", ctypes.c_int32),
                ("position_cutoff", ctypes.c_int32), ("alpha", ctypes.c_double), ("coulomb_prefactor", ctypes.c_double),
                ("bound_prefactor", ctypes.c_double), ("system_length", ctypes.c_double)]


class WaterDesc(ctypes.Structure):
    """JfgpuWaterDesc."""
    _fields_ = [("molecules", ctypes.c_int32), ("lifting", ctypes.c_int32), ("fourier_cutoff", ctypes.c_int32),
                ("position_cutoff", ctypes.c_int32), ("initial_active", ctypes.c_int32),
                ("initial_direction", ctypes.c_int32), ("mode", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("system_length", ctypes.c_double), ("beta", ctypes.c_double),
                ("chain_time", ctypes.c_double), ("speed", ctypes.c_double), ("oh_r0", ctypes.c_double),
                ("oh_prefactor", ctypes.c_double), ("hh_r0", ctypes.c_double), ("hh_prefactor", ctypes.c_double),
                ("lj_prefactor", ctypes.c_double), ("lj_sigma", ctypes.c_double),
                ("coulomb_prefactor", ctypes.c_double), ("bound_prefactor", ctypes.c_double),
                ("alpha", ctypes.c_double), ("seed", ctypes.c_uint64)]


class ChainDesc(ctypes.Structure):
    _fields_ = [("potential", ctypes.c_int32), ("far", ctypes.c_int32), ("n", ctypes.c_int32),
                ("cells_per_side", ctypes.c_int32), ("neighbor_layers", ctypes.c_int32),
                ("max_occupants", ctypes.c_int32), ("initial_active", ctypes.c_int32),
                ("initial_direction", ctypes.c_int32), ("fourier_cutoff", ctypes.c_int32),
                ("position_cutoff", ctypes.c_int32), ("estimator_points", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("system_length", ctypes.c_double), ("beta", ctypes.c_double),
                ("chain_time", ctypes.c_double), ("speed", ctypes.c_double), ("hs_radius", ctypes.c_double),
                ("lj_prefactor", ctypes.c_double), ("lj_sigma", ctypes.c_double),
                ("coulomb_prefactor", ctypes.c_double), ("bound_prefactor", ctypes.c_double),
                ("ewald_alpha", ctypes.c_double), ("estimator_prefactor", ctypes.c_double),
                ("rng_key", ctypes.c_uint64)]


class ChainState(ctypes.Structure):
    _fields_ = [("time_q", ctypes.c_double), ("time_r", ctypes.c_double), ("eoc_q", ctypes.c_double),
                ("eoc_r", ctypes.c_double), ("events", ctypes.c_int64), ("bound_warnings", ctypes.c_int64),
                ("refine_fallbacks", ctypes.c_int64), ("candidates", ctypes.c_int64), ("refined", ctypes.c_int64),
                ("active", ctypes.c_int32), ("direction", ctypes.c_int32),
                ("eoc_new_active", ctypes.c_int32), ("occ_active", ctypes.c_int32), ("occ_cell", ctypes.c_int32),
                ("n_surplus", ctypes.c_int32), ("status", ctypes.c_int32), ("stopped", ctypes.c_int32),
                ("lift_sum", ctypes.c_double), ("liftings", ctypes.c_int64), ("far_lookups", ctypes.c_int64)]


class Event(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("moved", ctypes.c_int32), ("target", ctypes.c_int32),
                ("new_active", ctypes.c_int32), ("new_direction", ctypes.c_int32), ("accepted", ctypes.c_int32),
                ("time_q", ctypes.c_double), ("time_r", ctypes.c_double), ("x", ctypes.c_double),
                ("y", ctypes.c_double), ("z", ctypes.c_double)]


class WaterCellBuffers(ctypes.Structure):
    """JfgpuWaterCellBuffers."""
    _fields_ = [("roots", ctypes.c_void_p), ("occupancy", ctypes.c_void_p), ("surplus", ctypes.c_void_p),
                ("cell_state", ctypes.c_void_p), ("root_log", ctypes.c_void_p)]


class Buffers(ctypes.Structure):
    _fields_ = [("positions", ctypes.c_void_p), ("positions32", ctypes.c_void_p), ("charges", ctypes.c_void_p),
                ("occupancy", ctypes.c_void_p), ("surplus", ctypes.c_void_p), ("roles", ctypes.c_void_p),
                ("state", ctypes.c_void_p), ("cell_slots", ctypes.c_void_p)]


class Layout(ctypes.Structure):
    _fields_ = [("n_chains", ctypes.c_int64), ("particles", ctypes.c_int64), ("occupancy_slots", ctypes.c_int64),
                ("table_bytes", ctypes.c_int64)]


_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_D = ctypes.c_double
_I32 = ctypes.c_int32

# every symbol of include/jfgpu.h with its argument types
SIGNATURES = {
    "jfgpu_hard_sphere_displacement": (ctypes.c_int, [_D, _P, _P, _I64, _P, _P, _P]),
    "jfgpu_inverse_power_displacement": (ctypes.c_int, [_D, _D, _P, _P, _P, _P, _I64, _P, _P, _P]),
    "jfgpu_inverse_power_derivative": (ctypes.c_int, [_D, _D, _P, _P, _P, _I64, _P, _P, _P]),
    "jfgpu_lennard_jones_displacement": (ctypes.c_int, [_D, _D, _P, _P, _P, _I64, _P, _P, _P]),
    "jfgpu_lennard_jones_derivative": (ctypes.c_int, [_D, _D, _P, _P, _I64, _P, _P, _P]),
    "jfgpu_displaced_even_power_displacement": (ctypes.c_int, [_D, _I32, _D, _P, _P, _P, _I64, _P, _P, _P]),
    "jfgpu_displaced_even_power_derivative": (ctypes.c_int, [_D, _I32, _D, _P, _P, _I64, _P, _P, _P]),
    "jfgpu_coulomb_bound_displacement": (ctypes.c_int, [_D, _D, _P, _P, _P, _P, _I64, _P, _P, _P]),
    "jfgpu_coulomb_bound_derivative": (ctypes.c_int, [_D, _P, _P, _P, _I64, _P, _P, _P]),
    "jfgpu_merged_image_coulomb_derivative": (ctypes.c_int, [_D, _I32, _I32, _D, _D, _P, _P, _P, _I64, _P, _P,
                                                             _P]),
    "jfgpu_merged_image_coulomb_derivative_noalloc": (ctypes.c_int, [_D, _I32, _I32, _D, _D, _P, _P, _P, _I64,
                                                                     _P, _P, _P]),
    "jfgpu_cell_bounding_displacement": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _I64, _P, _P, _P]),
    "jfgpu_lifting": (ctypes.c_int, [_I32, _I32, _P, _P, _P, _I64, _P, _P, _P, _P, _P]),
    "jfgpu_composite_event_time": (ctypes.c_int, [ctypes.POINTER(CompositeDesc), _P, _P, _P, _P, _P, _P, _I64, _P,
                                                  _P, _P]),
    "jfgpu_composite_out_state": (ctypes.c_int, [ctypes.POINTER(CompositeDesc), _I32, _P, _P, _P, _P, _P, _P, _P,
                                                 _P, _I64, _P, _P, _P, _P]),
    "jfgpu_composite_bounded_out_state": (ctypes.c_int, [ctypes.POINTER(CompositeDesc), _I32, _P, _P, _P, _P, _P,
                                                         _P, _P, _P, _P, _I64, _P, _P, _P, _P]),
    "jfgpu_composite_cell_bound_time": (ctypes.c_int, [_P, _P, _I64, _P, _P, _P, _P, _I32, _D, _P, _I64, _P, _P, _P,
                                                       _P]),
    "jfgpu_composite_cell_veto_time": (ctypes.c_int, [_P, _P, _I64, _P, _P, _P, _P, _P, _P, _I64, _P, _P, _P, _P]),
    "jfgpu_walker_table": (ctypes.c_int, [_P, _P, _I64, _P, _P, _P, _P, _P]),
    "jfgpu_walker_sample": (ctypes.c_int, [_P, _P, _P, _I64, _D, _P, _P, _I32, _I64, _P, _P, _P]),
    "jfgpu_water_create": (ctypes.c_int, [ctypes.POINTER(WaterDesc), ctypes.POINTER(ctypes.c_void_p)]),
    "jfgpu_water_destroy": (None, [_P]),
    "jfgpu_water_init": (ctypes.c_int, [_P, _P, _I64, _I64, _P]),
    "jfgpu_water_run": (ctypes.c_int, [_P, _P, _P, _P, _I64, _I64, _I64, _D, _D, _P, _I32, _P]),
    "jfgpu_water_set_cells": (ctypes.c_int, [_P, _I32, _I32, _P, _P, _I32, _I32, _D]),
    "jfgpu_water_cells_init": (ctypes.c_int, [_P, ctypes.POINTER(WaterCellBuffers), _I64, _P]),
    "jfgpu_water_cells_run": (ctypes.c_int, [_P, _P, _P, _P, ctypes.POINTER(WaterCellBuffers), _I64, _I64, _I64,
                                             _D, _D, _P, _I32, _P]),
    "jfgpu_engine_create": (ctypes.c_int, [_P, _I64, _P, ctypes.POINTER(ctypes.c_void_p)]),
    "jfgpu_engine_destroy": (None, [_P]),
    "jfgpu_engine_layout": (ctypes.c_int, [_P, ctypes.POINTER(Layout)]),
    "jfgpu_engine_offsets": (ctypes.c_int, [_P, _P, _P]),
    "jfgpu_engine_bounds": (ctypes.c_int, [_P, _I64, _P, _P, _I64]),
    "jfgpu_chains_init": (ctypes.c_int, [_P, ctypes.POINTER(Buffers), _P]),
    "jfgpu_chains_run": (ctypes.c_int, [_P, ctypes.POINTER(Buffers), _I64, _I64, _I64, _D, _D, _I32, _P, _I64,
                                        _P]),
    "jfgpu_chains_set_block_warps": (ctypes.c_int, [_P, _I32]),
    "jfgpu_chains_set_refine_limit": (ctypes.c_int, [_P, _I32]),
    "jfgpu_chains_set_groups": (ctypes.c_int, [_P, _I32]),
    "jfgpu_chains_set_graphs": (ctypes.c_int, [_P, _I32]),
    "jfgpu_chains_refresh_mirror": (ctypes.c_int, [_P, ctypes.POINTER(Buffers), _I64, _I64, _P]),
    "jfgpu_chains_observe": (ctypes.c_int, [_P, ctypes.POINTER(Buffers), _I64, _I64, _I32, _D, _P, _P, _P]),
    "jfgpu_engine_set_timing": (ctypes.c_int, [_P, _I32]),
    "jfgpu_engine_kernel_times": (ctypes.c_int, [_P, _P, _P, _I32]),
    "jfgpu_engine_launch_count": (ctypes.c_int64, [_P]),
    "jfgpu_random_sequential_addition": (ctypes.c_int, [_I64, _D, _D, ctypes.c_uint64, _I64, _P]),
    "jfgpu_error_string": (ctypes.c_char_p, [ctypes.c_int]),
    "jfgpu_version": (ctypes.c_int, []),
}

_LIB = None


def load_library(path: str = LIBRARY_PATH) -> ctypes.CDLL:
    """Load the shared library and declare every entry point (no GPU needed)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise LibraryMissing("libjfgpu.so is not built (%s); run __graft_entry__.build() or "
                             "python jellyfysh_gb300/build.py" % path)
    handle = ctypes.CDLL(path)
    for name, (restype, argtypes) in SIGNATURES.items():
        fn = getattr(handle, name)
        fn.restype = restype
        fn.argtypes = argtypes
    _LIB = handle
    return handle


def load() -> ctypes.CDLL:
    """Load the library for compute: requires a CUDA device."""
    import torch
    if not torch.cuda.is_available():
        raise NoGpu("jellyfysh_gb300 computes on a CUDA GPU only; no device is visible")
    return load_library()


def check(code: int, what: str = "") -> None:
    if code != OK:
        message = ERROR_NAMES.get(code, "error %d" % code)
        raise JfgpuError("%s failed: %s" % (what or "jfgpu call", message))
