"""ctypes mirror of include/knc.h and the loader of libknc_gpu.so.

The structs here are field-for-field copies of the C structs; the library is
the CUDA build in ``app-kilonova_gb300/_build``. There is no CPU fallback: if
the library is missing, :func:`load` raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # app-kilonova_gb300/
LIB_PATH = PKG_ROOT / "_build" / "libknc_gpu.so"

# status codes
KNC_OK = 0
KNC_ERR_INVALID_ARGUMENT = 1
KNC_ERR_CONFIG = 2
KNC_ERR_CUDA = 3
KNC_ERR_NO_BLOCK = 4
KNC_ERR_HYDRO = 5
KNC_ERR_UNSUPPORTED = 6
KNC_ERR_OUT_OF_MEMORY = 7
KNC_ERR_TIMEOUT = 8

# hydro error kinds
KNC_HYDRO_NONE = 0
KNC_HYDRO_NEGATIVE_DENSITY = 1
KNC_HYDRO_NEGATIVE_PRESSURE = 2
KNC_HYDRO_NEGATIVE_ENERGY_DENSITY = 3
KNC_HYDRO_ROOT_FINDER_FAILED = 4

KNC_SYSTEM_RELATIVISTIC = 0
KNC_SYSTEM_NEWTONIAN = 1
KNC_RIEMANN_HLLE = 0
KNC_RIEMANN_HLLC = 1
KNC_PRECISION_FP64 = 0
KNC_PRECISION_MIXED = 1
KNC_GUESS_PLAIN = 0
KNC_GUESS_MLP = 1

KNC_MODEL_WIND = 0
KNC_MODEL_JET = 1
KNC_MODEL_SPHERE = 2
KNC_MODEL_HOST = 3
KNC_MODEL_JET_IN_CLOUD = 4
KNC_MODEL_KINETIC_BOMB = 5
KNC_MODEL_JET_IN_STAR = 6

KNC_KERNEL_GHOST = 0
KNC_KERNEL_C2P = 1
KNC_KERNEL_UPDATE = 2
KNC_KERNEL_FUSED = 3
KNC_UPDATE_TILE = 0
KNC_UPDATE_TILE_TMA = 1
KNC_UPDATE_STRIP = 2
KNC_RECOVERY_INLINE = 0
KNC_RECOVERY_DEFERRED = 1
KNC_KERNEL_KINDS = 4

KNC_MLP_HIDDEN = 64
KNC_MLP_OFF_W1 = 0
KNC_MLP_OFF_B1 = 192
KNC_MLP_OFF_W2 = 256
KNC_MLP_OFF_B2 = 4352
KNC_MLP_OFF_W3 = 4416
KNC_MLP_OFF_B3 = 4480
KNC_MLP_OFF_XMEAN = 4481
KNC_MLP_OFF_XSCALE = 4484
KNC_MLP_NUM_PARAMS = 4487
KNC_NOALLOC_MAX_ZONES = 131072

HYDRO_ERROR_NAMES = {
    KNC_HYDRO_NONE: "None",
    KNC_HYDRO_NEGATIVE_DENSITY: "NegativeDensity",
    KNC_HYDRO_NEGATIVE_PRESSURE: "NegativePressure",
    KNC_HYDRO_NEGATIVE_ENERGY_DENSITY: "NegativeEnergyDensity",
    KNC_HYDRO_ROOT_FINDER_FAILED: "RootFinderFailed",
}


class HydroParams(C.Structure):
    _fields_ = [
        ("system", C.c_int32),
        ("runge_kutta_order", C.c_int32),
        ("riemann_solver", C.c_int32),
        ("adaptive_time_step", C.c_int32),
        ("gamma_law_index", C.c_double),
        ("plm_theta", C.c_double),
        ("cfl_number", C.c_double),
    ]


class MeshParams(C.Structure):
    _fields_ = [
        ("reference_radius", C.c_double),
        ("inner_radius", C.c_double),
        ("outer_radius", C.c_double),
        ("inner_excision_speed", C.c_double),
        ("outer_excision_speed", C.c_double),
        ("excision_delay", C.c_double),
        ("num_radial_zones", C.c_int64),
        ("num_polar_zones", C.c_int64),
        ("block_size", C.c_int64),
        ("has_num_radial_zones", C.c_int32),
        ("has_excision_delay", C.c_int32),
    ]


class ModelParams(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("reserved", C.c_int32),
        ("seed", C.c_uint64),
        ("p", C.c_double * 16),
    ]


class Error(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("block", C.c_int32),
        ("i", C.c_int32),
        ("j", C.c_int32),
        ("r", C.c_double),
        ("theta", C.c_double),
        ("value", C.c_double),
        ("message", C.c_char * 256),
    ]


class Tuning(C.Structure):
    _fields_ = [("tile_rows", C.c_int32), ("fused", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("update_form", C.c_int32), ("recovery_form", C.c_int32)]


class MlpTrainParams(C.Structure):
    _fields_ = [
        ("steps", C.c_int64),
        ("batch", C.c_int32),
        ("reserved", C.c_int32),
        ("lr", C.c_float),
        ("beta1", C.c_float),
        ("beta2", C.c_float),
        ("eps", C.c_float),
        ("seed", C.c_uint64),
    ]


PRIMITIVE_AT_FN = C.CFUNCTYPE(None, C.c_double, C.c_double, C.c_double,
                              C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p)

_P = C.c_void_p
_DP = C.POINTER(C.c_double)
_FP = C.POINTER(C.c_float)
_I32P = C.POINTER(C.c_int32)
_I64P = C.POINTER(C.c_int64)

# name -> (restype, argtypes); every entry point declared in include/knc.h
SIGNATURES = {
    "knc_create": (C.c_int, [C.POINTER(HydroParams), C.POINTER(MeshParams), C.POINTER(_P)]),
    "knc_destroy": (None, [_P]),
    "knc_status_string": (C.c_char_p, [C.c_int]),
    "knc_last_error": (C.c_int, [_P, C.POINTER(Error)]),
    "knc_set_model": (C.c_int, [_P, C.POINTER(ModelParams)]),
    "knc_set_host_model": (C.c_int, [_P, PRIMITIVE_AT_FN, _P]),
    "knc_init_from_model": (C.c_int, [_P, C.c_double]),
    "knc_add_block": (C.c_int, [_P, C.c_int32, _DP, _DP]),
    "knc_remove_block": (C.c_int, [_P, C.c_int32]),
    "knc_get_block": (C.c_int, [_P, C.c_int32, _DP, _DP]),
    "knc_num_blocks": (C.c_int, [_P, _I32P]),
    "knc_block_indexes": (C.c_int, [_P, _I32P, C.c_int32]),
    "knc_block_shape": (C.c_int, [_P, _I64P, _I64P]),
    "knc_set_block_shapes": (C.c_int, [_P, C.c_int32, C.c_int32, _I32P, _I32P]),
    "knc_block_shape_of": (C.c_int, [_P, C.c_int32, _I64P, _I64P]),
    "knc_set_state": (C.c_int, [_P, _DP, _DP]),
    "knc_get_state": (C.c_int, [_P, _DP, _DP]),
    "knc_set_time": (C.c_int, [_P, C.c_double, C.c_int64, C.c_int64]),
    "knc_get_time": (C.c_int, [_P, _DP, _I64P, _I64P]),
    "knc_time_step": (C.c_int, [_P, _DP]),
    "knc_advance": (C.c_int, [_P, C.c_int32]),
    "knc_set_precision": (C.c_int, [_P, C.c_int32]),
    "knc_set_c2p_guess": (C.c_int, [_P, C.c_int32, _FP, C.c_size_t]),
    "knc_set_batched": (C.c_int, [_P, C.c_int32]),
    "knc_set_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
    "knc_advance_dt": (C.c_int, [_P, C.c_int32, C.c_double]),
    "knc_advance_host": (C.c_int, [_P, _DP, _DP, _DP, _DP, C.c_int32]),
    "knc_zone_updates": (C.c_int, [_P, _I64P]),
    "knc_get_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
    "knc_autotune": (C.c_int, [_P, C.c_int32, C.POINTER(Tuning), _DP]),
    "knc_set_mixed_w_split": (C.c_int, [_P, C.c_double]),
    "knc_set_wait_test": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "knc_selftest_copy_wait": (C.c_int, [C.c_int32, C.POINTER(C.c_int32)]),
    "knc_synchronize": (C.c_int, [_P]),
    "knc_c2p_stats": (C.c_int, [_P, _I64P, _I64P, _I64P, _I64P]),
    "knc_reset_c2p_stats": (C.c_int, [_P]),
    "knc_launch_count": (C.c_int, [_P, _I64P]),
    "knc_set_profiling": (C.c_int, [_P, C.c_int32]),
    "knc_kernel_times": (C.c_int, [_P, _DP, _I64P]),
    "knc_mark": (C.c_int, [_P, C.c_int32]),
    "knc_elapsed_ms": (C.c_int, [_P, C.c_int32, C.c_int32, _DP]),
    "knc_get_primitives": (C.c_int, [_P, C.c_int32, _DP]),
    "knc_get_products": (C.c_int, [_P, C.c_int32, _DP, _DP, _DP, _DP]),
    "knc_set_device": (C.c_int, [C.c_int32]),
    "knc_device_count": (C.c_int, [C.POINTER(C.c_int32)]),
    "knc_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    "knc_host_free": (C.c_int, [C.c_void_p]),
    "knc_mlp_num_params": (C.c_size_t, []),
    "knc_sample_pairs": (C.c_int, [_P, C.c_int32, _DP, C.c_int64, _I64P]),
    "knc_generate_pairs": (C.c_int, [C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.c_uint64, C.c_int64, _DP]),
    "knc_mlp_train": (C.c_int, [_DP, C.c_int64, _FP, C.POINTER(MlpTrainParams), _FP]),
    "knc_mlp_forward_backward": (C.c_int, [_FP, _FP, _FP, C.c_int32, _FP, _FP, _FP]),
    "knc_mlp_features": (None, [_DP, _FP]),
    "knc_measure_fp64_peak": (C.c_int, [_DP]),
    "knc_test_conversions": (C.c_int, [_DP, C.c_int64, _DP]),
    "knc_recover_primitives_noalloc": (C.c_int, [C.POINTER(HydroParams), C.POINTER(MeshParams), C.c_int32,
                                                 _P, _P, _P, _P, C.POINTER(Error)]),
}


class KncError(RuntimeError):
    """A non-zero status from the library, with the decoded hydro error."""

    def __init__(self, status: int, message: str, error: dict | None = None):
        super().__init__(message)
        self.status = status
        self.error = error or {}


_lib = None


def load(path: str | os.PathLike | None = None):
    """Load libknc_gpu.so (built by ``build.py``); raise if it is absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(
            f"{p} not found: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(p), mode=C.RTLD_GLOBAL)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def dptr(a):
    """Pointer to the data of a C-contiguous float64 numpy array."""
    return a.ctypes.data_as(_DP)


def fptr(a):
    return a.ctypes.data_as(_FP)
