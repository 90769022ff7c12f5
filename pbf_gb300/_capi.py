"""ctypes binding of ``include/pbf.h`` (the C ABI of libpbf_gb300.so).

The library is loaded from the in-tree build directory.  Loading fails
loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpbf_gb300.so")

PBF_OK = 0
PBF_ERR_INVALID_ARGUMENT = 1
PBF_ERR_OUT_OF_MEMORY = 2
PBF_ERR_CUDA = 3
PBF_ERR_DEVICE_FAULT = 4
PBF_ERR_NO_DEVICE = 5
PBF_ERR_UNSUPPORTED = 6

PBF_DEV_NONFINITE = 0x1
PBF_DEV_SORT_TIMEOUT = 0x2
PBF_DEV_RUN_OVER_127 = 0x4
PBF_DEV_INDEX = 0x8

PBF_HOST = 0
PBF_DEVICE = 1

PBF_SWEEP_DIRECT = 0
PBF_SWEEP_MASKED = 1
PBF_SWEEP_COOP = 2
PBF_SWEEP_AUTO = 3

PBF_PASS_MASKED = 0
PBF_PASS_DIRECT = 1
PBF_PASS_COOP = 2
PBF_PASS_DIRECT_COOP = 3
PBF_PASS_MIXED = 4


class Params(C.Structure):
    """pbf_params (include/pbf.h)."""

    _fields_ = [
        ("one_over_rho_0", C.c_float),
        ("epsilon", C.c_float),
        ("gravity", C.c_float),
        ("timestep", C.c_float),
        ("tensile_instability_k", C.c_float),
        ("tensile_instability_scale", C.c_float),
        ("xsph_viscosity_c", C.c_float),
        ("vorticity_epsilon", C.c_float),
        ("h", C.c_float),
        ("num_solver_iterations", C.c_uint32),
        ("vorticity_confinement", C.c_uint32),
        ("external_force", C.c_uint32),
        ("grid", C.c_uint32 * 3),
        ("wall_lo", C.c_float * 3),
        ("wall_hi", C.c_float * 3),
    ]

    def copy(self) -> "Params":
        p = Params()
        C.memmove(C.byref(p), C.byref(self), C.sizeof(Params))
        return p

    def as_dict(self) -> dict:
        d = {}
        for name, _ in self._fields_:
            val = getattr(self, name)
            d[name] = list(val) if hasattr(val, "__len__") else val
        return d


class Tuning(C.Structure):
    """pbf_tuning (include/pbf.h)."""

    _fields_ = [
        ("use_neighbour_lists", C.c_uint32),
        ("list_capacity", C.c_uint32),
        ("skin_h", C.c_float),
        ("block_size", C.c_uint32),
        ("sweep_mode", C.c_uint32),
        ("pair_list_capacity", C.c_uint32),
        ("coop_candidates", C.c_uint32),
        ("auto_period", C.c_uint32),
        ("adjoint_warp_candidates", C.c_uint32),
    ]


class ParamGrads(C.Structure):
    """pbf_param_grads (include/pbf.h)."""

    _fields_ = [
        ("epsilon", C.c_double),
        ("tensile_instability_k", C.c_double),
        ("xsph_viscosity_c", C.c_double),
        ("vorticity_epsilon", C.c_double),
    ]


class Diagnostics(C.Structure):
    _fields_ = [
        ("mean_density_error", C.c_double),
        ("max_density_error", C.c_double),
        ("kinetic_energy", C.c_double),
        ("candidate_pairs", C.c_double),
    ]


# Every entry point of include/pbf.h with its ctypes signature.
_P = C.c_void_p
_F = C.POINTER(C.c_float)
_U32P = C.POINTER(C.c_uint32)
_I32P = C.POINTER(C.c_int32)
SIGNATURES = {
    "pbf_params_default": (C.c_int, [_U32P, C.POINTER(Params)]),
    "pbf_wpoly6": (C.c_double, [C.c_double, C.c_double]),
    "pbf_rest_density_lattice": (C.c_double, [C.c_double, C.c_double]),
    "pbf_scene_block": (C.c_int, [_U32P, C.c_float, _F, C.c_float, C.c_float, C.c_float,
                                  C.c_uint64, _P, _P]),
    "pbf_create": (C.c_int, [C.POINTER(Params), C.c_uint32, C.POINTER(C.c_void_p)]),
    "pbf_create_batch": (C.c_int, [C.POINTER(Params), _U32P, C.c_uint32, C.POINTER(C.c_void_p)]),
    "pbf_num_scenes": (C.c_uint32, [_P]),
    "pbf_scene_range": (C.c_int, [_P, C.c_uint32, _U32P, _U32P]),
    "pbf_set_scene_params": (C.c_int, [_P, C.c_uint32, C.POINTER(Params)]),
    "pbf_get_scene_params": (C.c_int, [_P, C.c_uint32, C.POINTER(Params)]),
    "pbf_num_cells": (C.c_uint32, [_P]),
    "pbf_destroy": (None, [_P]),
    "pbf_set_params": (C.c_int, [_P, C.POINTER(Params)]),
    "pbf_get_params": (C.c_int, [_P, C.POINTER(Params)]),
    "pbf_num_particles": (C.c_uint32, [_P]),
    "pbf_set_stream": (C.c_int, [_P, _P]),
    "pbf_set_state": (C.c_int, [_P, _P, _P, C.c_int]),
    "pbf_get_state": (C.c_int, [_P, _P, _P, C.c_int]),
    "pbf_device_buffers": (C.c_int, [_P, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "pbf_step": (C.c_int, [_P, C.c_uint32]),
    "pbf_synchronize": (C.c_int, [_P]),
    "pbf_set_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
    "pbf_get_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
    "pbf_get_sweep_choice": (C.c_int, [_P, C.POINTER(C.c_uint32)]),
    "pbf_kernels_launched": (C.c_uint64, [_P]),
    "pbf_autotune": (C.c_int, [_P, C.c_uint32, C.POINTER(Tuning)]),
    "pbf_device_status": (C.c_int, [_P, _U32P]),
    "pbf_enable_timing": (C.c_int, [_P, C.c_int]),
    "pbf_get_timing": (C.c_int, [_P, _F]),
    "pbf_get_stage_times": (C.c_int, [_P, C.POINTER(C.c_double), _U32P]),
    "pbf_kernels_per_substep": (C.c_uint32, [_P]),
    "pbf_get_sort": (C.c_int, [_P, _P, _P, _P]),
    "pbf_get_cells": (C.c_int, [_P, _P, _P]),
    "pbf_get_solver": (C.c_int, [_P, _P, _P]),
    "pbf_radix_sort": (C.c_int, [_P, _P, _P, C.c_uint32, C.c_uint32, _P]),
    "pbf_radix_sort_noalloc": (C.c_int, [_P, _P, _P, C.c_uint32, C.c_uint32, _P]),
    "pbf_find_cells": (C.c_int, [_P, C.c_uint32, C.c_uint32, _P, _P, _P]),
    "pbf_compute_diagnostics": (C.c_int, [_P, C.POINTER(Diagnostics)]),
    "pbf_highlight_neighbours": (C.c_int, [_P, _P, C.c_int]),
    "pbf_splat": (C.c_int, [C.c_int, _P, C.c_uint32, _P, C.c_uint32, C.c_uint32, _P, _P]),
    "pbf_save_state": (C.c_int, [_P, C.c_char_p]),
    "pbf_load_state": (C.c_int, [_P, C.c_char_p]),
    "pbf_forward_record": (C.c_int, [_P, C.c_uint32, C.c_uint32]),
    "pbf_backward": (C.c_int, [_P, _P, _P, C.c_int, _P, _P, _P]),
    "pbf_release_record": (C.c_int, [_P]),
    "pbf_status_string": (C.c_char_p, [C.c_int]),
    "pbf_debug_fail_allocation": (None, [C.c_int]),
    "pbf_debug_sort_stall": (None, [C.c_uint32]),
    "pbf_last_error": (C.c_char_p, [_P]),
    "pbf_abi_version": (C.c_int, []),
}

_lib = None


def _bind(path: str) -> C.CDLL:
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def load() -> C.CDLL:
    """Loads libpbf_gb300.so (building nothing); raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -m pbf_gb300.build` "
            "(there is no CPU fallback)")
    _lib = _bind(LIB_PATH)
    return _lib


def load_checked() -> C.CDLL:
    """Loads the bounds-checked build (-DPBF_CHECK,
    pbf_gb300/_build_check/libpbf_gb300_check.so: index checks set
    PBF_DEV_INDEX instead of faulting), a separate library with the same
    entry points; build it with `python -m pbf_gb300.build --check`."""
    from .build import CHECK_LIB
    if not os.path.exists(CHECK_LIB):
        raise RuntimeError(f"{CHECK_LIB} is missing: build it with "
                           "`python -m pbf_gb300.build --check`")
    return _bind(CHECK_LIB)


class PbfError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


def check(status: int, handle=None) -> None:
    if status != PBF_OK:
        lib = load()
        msg = lib.pbf_last_error(handle)
        raise PbfError(status, (msg or b"").decode() or lib.pbf_status_string(status).decode())
