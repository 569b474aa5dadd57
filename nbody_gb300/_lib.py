"""ctypes binding of libnbody_gb300.so (include/nbody_gb300.h).

The library is the product: this module loads it from the package directory
and raises if it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libnbody_gb300.so"

# enum values of include/nbody_gb300.h
NBG_OK = 0
STATUS_NAMES = {0: "ok", 1: "invalid argument", 2: "foreign buffer", 3: "size mismatch",
                4: "out of memory", 5: "cuda error", 6: "unsupported",
                7: "not initialized", 8: "device timeout", 9: "device error",
                10: "exceeds a fixed capacity"}
ALGO = {"direct": 0, "bh": 1}
PRECISION = {"fp64": 0, "mixed": 1}
LAYOUT = {"heap": 1, "heap_stackless": 2}
TRAVERSE = {"cycle": 0, "nested_tree": 1}
K_DIRECT, K_TREE_BUILD, K_BH_WALK, K_VECOPS, K_ENS_STEP, K_JUDGE = 0, 1, 2, 3, 4, 5
JUDGE_STATS = 11  # NBG_JUDGE_STATS

# Every symbol the header declares: checked by the CPU test suite.
EXPORTS = [
    "nbg_params_default", "nbg_status_string", "nbg_abi_version", "nbg_engine_create",
    "nbg_engine_destroy", "nbg_type_name", "nbg_last_error", "nbg_init", "nbg_get_data",
    "nbg_problem_size", "nbg_get_y", "nbg_fcompute", "nbg_clamp", "nbg_create_buffer",
    "nbg_free_buffer", "nbg_buffer_size", "nbg_buffer_device_ptr", "nbg_read_buffer",
    "nbg_write_buffer", "nbg_copy_buffer", "nbg_fill_buffer", "nbg_fmadd_inplace",
    "nbg_fmadd", "nbg_fmaddn_inplace", "nbg_fmaddn_corr", "nbg_fmaddn", "nbg_fmaxabs",
    "nbg_synchronize", "nbg_stream", "nbg_host_alloc", "nbg_host_free",
    "nbg_profile_enable", "nbg_profile_query", "nbg_launch_count",
    "nbg_measure_fp32_peak", "nbg_tune_set", "nbg_tune_get", "nbg_direct_mixed_noalloc",
    "nbg_bh_counters", "nbg_learn_param_count", "nbg_learn_set_weights",
    "nbg_learn_get_weights", "nbg_learn_init_weights", "nbg_learn_generate",
    "nbg_learn_sample_count", "nbg_learn_read_samples", "nbg_learn_clear_samples",
    "nbg_learn_train", "nbg_learn_loss_grad", "nbg_tree_leaves", "nbg_learn_predict", "nbg_learn_predict_tc", "nbg_learn_tc_accumulators", "nbg_statistics",
    "nbg_ensemble_params_default", "nbg_ensemble_create", "nbg_ensemble_destroy",
    "nbg_ensemble_last_error", "nbg_ensemble_init", "nbg_ensemble_step",
    "nbg_ensemble_synchronize", "nbg_ensemble_status", "nbg_ensemble_get_state",
    "nbg_ensemble_fcompute", "nbg_ensemble_statistics", "nbg_ensemble_tune_set",
    "nbg_ensemble_launch_count", "nbg_ensemble_profile", "nbg_autotune",
    "nbg_ensemble_autotune", "nbg_stream_open", "nbg_stream_set_header", "nbg_stream_write",
    "nbg_stream_write_host", "nbg_stream_flush", "nbg_stream_close", "nbg_stream_last_error",
    "nbg_bh_stack_peak", "nbg_bh_fallback_groups", "nbg_learn_judge_stats",
    "nbg_learn_band_rows",
]


class Params(C.Structure):
    """struct nbg_params."""
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("device", C.c_int32),
        ("algo", C.c_int32),
        ("precision", C.c_int32),
        ("softening", C.c_double),
        ("distance_to_node_radius_ratio", C.c_double),
        ("tree_build_rate", C.c_uint64),
        ("tree_layout", C.c_int32),
        ("traverse_type", C.c_int32),
        ("learned", C.c_int32),
        ("block_size", C.c_int32),
        ("learned_tight_ratio", C.c_double),
    ]


class EnsembleParams(C.Structure):
    """struct nbg_ensemble_params."""
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("device", C.c_int32),
        ("softening", C.c_double),
        ("tolerance", C.c_double),
        ("dt_initial", C.c_double),
        ("dt_min", C.c_double),
        ("dt_max", C.c_double),
        ("use_graph", C.c_int32),
    ]


class NbgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


_lib = None


def _proto(lib, name, restype, *argtypes):
    fn = getattr(lib, name)
    fn.restype = restype
    fn.argtypes = list(argtypes)


def load() -> C.CDLL:
    """Load libnbody_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} not found: build it with "
                          "`python -m nbody_gb300.build` (there is no CPU fallback)")
    lib = C.CDLL(str(LIB_PATH))
    vp, i32, u64, sz, dbl = C.c_void_p, C.c_int, C.c_uint64, C.c_size_t, C.c_double
    dp = C.POINTER(C.c_double)
    _proto(lib, "nbg_params_default", None, C.POINTER(Params))
    _proto(lib, "nbg_status_string", C.c_char_p, i32)
    _proto(lib, "nbg_abi_version", i32)
    _proto(lib, "nbg_engine_create", i32, C.POINTER(Params), C.POINTER(vp))
    _proto(lib, "nbg_engine_destroy", None, vp)
    _proto(lib, "nbg_type_name", C.c_char_p, vp)
    _proto(lib, "nbg_last_error", C.c_char_p, vp)
    _proto(lib, "nbg_init", i32, vp, sz, vp, vp, vp)
    _proto(lib, "nbg_get_data", i32, vp, vp, vp)
    _proto(lib, "nbg_problem_size", sz, vp)
    _proto(lib, "nbg_get_y", vp, vp)
    _proto(lib, "nbg_fcompute", i32, vp, dbl, u64, vp, vp)
    _proto(lib, "nbg_clamp", i32, vp, vp, dbl)
    _proto(lib, "nbg_create_buffer", i32, vp, sz, C.POINTER(vp))
    _proto(lib, "nbg_free_buffer", i32, vp, vp)
    _proto(lib, "nbg_buffer_size", sz, vp)
    _proto(lib, "nbg_buffer_device_ptr", vp, vp)
    _proto(lib, "nbg_read_buffer", i32, vp, vp, vp)
    _proto(lib, "nbg_write_buffer", i32, vp, vp, vp)
    _proto(lib, "nbg_copy_buffer", i32, vp, vp, vp)
    _proto(lib, "nbg_fill_buffer", i32, vp, vp, dbl)
    _proto(lib, "nbg_fmadd_inplace", i32, vp, vp, vp, dbl)
    _proto(lib, "nbg_fmadd", i32, vp, vp, vp, vp, dbl)
    _proto(lib, "nbg_fmaddn_inplace", i32, vp, vp, C.POINTER(vp), sz, dp, sz)
    _proto(lib, "nbg_fmaddn_corr", i32, vp, vp, vp, C.POINTER(vp), sz, dp, sz)
    _proto(lib, "nbg_fmaddn", i32, vp, vp, vp, C.POINTER(vp), sz, dp, sz)
    _proto(lib, "nbg_fmaxabs", i32, vp, vp, dp)
    _proto(lib, "nbg_synchronize", i32, vp)
    _proto(lib, "nbg_stream", vp, vp)
    _proto(lib, "nbg_host_alloc", i32, sz, C.POINTER(vp))
    _proto(lib, "nbg_host_free", None, vp)
    _proto(lib, "nbg_profile_enable", i32, vp, i32)
    _proto(lib, "nbg_profile_query", i32, vp, i32, dp, C.POINTER(u64))
    _proto(lib, "nbg_launch_count", u64, vp)
    _proto(lib, "nbg_measure_fp32_peak", i32, vp, dp)
    _proto(lib, "nbg_tune_set", i32, vp, C.c_char_p, C.c_int64)
    _proto(lib, "nbg_tune_get", i32, vp, C.c_char_p, C.POINTER(C.c_int64))
    _proto(lib, "nbg_direct_mixed_noalloc", i32, vp, vp, vp, sz, dbl, vp)
    _proto(lib, "nbg_bh_counters", i32, vp, C.POINTER(u64), C.POINTER(u64))
    _proto(lib, "nbg_bh_stack_peak", i32, vp, C.POINTER(u64), C.POINTER(u64))
    _proto(lib, "nbg_bh_fallback_groups", i32, vp, C.POINTER(u64))
    fp = C.POINTER(C.c_float)
    ip = C.POINTER(C.c_int)
    _proto(lib, "nbg_learn_param_count", sz)
    _proto(lib, "nbg_learn_set_weights", i32, vp, fp, sz)
    _proto(lib, "nbg_learn_get_weights", i32, vp, fp, sz)
    _proto(lib, "nbg_learn_init_weights", i32, vp, u64)
    _proto(lib, "nbg_learn_generate", i32, vp, sz, u64, i32, C.POINTER(sz))
    _proto(lib, "nbg_learn_sample_count", sz, vp)
    _proto(lib, "nbg_learn_read_samples", i32, vp, sz, sz, fp, fp, ip)
    _proto(lib, "nbg_learn_clear_samples", i32, vp)
    _proto(lib, "nbg_learn_train", i32, vp, i32, sz, dbl, u64, dbl, dp, dp)
    _proto(lib, "nbg_learn_loss_grad", i32, vp, fp, fp, sz, dp, fp)
    _proto(lib, "nbg_tree_leaves", i32, vp, ip)
    _proto(lib, "nbg_learn_predict", i32, vp, fp, sz, fp)
    _proto(lib, "nbg_learn_predict_tc", i32, vp, fp, sz, fp)
    _proto(lib, "nbg_learn_tc_accumulators", i32, vp, fp, sz, fp)
    _proto(lib, "nbg_learn_judge_stats", i32, vp, dp, sz)
    _proto(lib, "nbg_learn_band_rows", i32, vp, C.POINTER(u64))
    _proto(lib, "nbg_statistics", i32, vp, vp, dp)
    u32p = C.POINTER(C.c_uint32)
    _proto(lib, "nbg_ensemble_params_default", None, C.POINTER(EnsembleParams))
    _proto(lib, "nbg_ensemble_create", i32, C.POINTER(EnsembleParams), C.POINTER(vp))
    _proto(lib, "nbg_ensemble_destroy", None, vp)
    _proto(lib, "nbg_ensemble_last_error", C.c_char_p, vp)
    _proto(lib, "nbg_ensemble_init", i32, vp, sz, u32p, vp, vp, vp)
    _proto(lib, "nbg_ensemble_step", i32, vp, i32)
    _proto(lib, "nbg_ensemble_synchronize", i32, vp)
    _proto(lib, "nbg_ensemble_status", i32, vp, dp, dp, u32p, u32p)
    _proto(lib, "nbg_ensemble_get_state", i32, vp, vp, vp)
    _proto(lib, "nbg_ensemble_fcompute", i32, vp, dp)
    _proto(lib, "nbg_ensemble_statistics", i32, vp, dp)
    _proto(lib, "nbg_ensemble_tune_set", i32, vp, C.c_char_p, C.c_int64)
    _proto(lib, "nbg_ensemble_launch_count", u64, vp)
    _proto(lib, "nbg_ensemble_profile", i32, vp, i32, dp, C.POINTER(u64))
    _proto(lib, "nbg_autotune", i32, vp, i32, C.c_char_p, sz)
    _proto(lib, "nbg_ensemble_autotune", i32, vp, i32, C.c_char_p, sz)
    _proto(lib, "nbg_stream_open", i32, vp, C.c_char_p, C.c_int64, i32, C.POINTER(vp))
    _proto(lib, "nbg_stream_set_header", i32, vp, sz, u64, vp, vp)
    _proto(lib, "nbg_stream_write", i32, vp, vp, u64, dbl)
    _proto(lib, "nbg_stream_write_host", i32, vp, vp, vp, u64, dbl)
    _proto(lib, "nbg_stream_flush", i32, vp)
    _proto(lib, "nbg_stream_close", i32, vp)
    _proto(lib, "nbg_stream_last_error", C.c_char_p, vp)
    _lib = lib
    return lib
