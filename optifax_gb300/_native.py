"""ctypes binding of the C ABI in include/optifax.h (liboptifax.so).

The library is the only compute path: if it is missing or no CUDA device is
present, the functions here raise.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

HEUN, RK23 = 0, 1
VARIANT_BATCH_XTAL, VARIANT_BATCH_OP, VARIANT_NO_BC, VARIANT_HARD_BC, VARIANT_ODE23, VARIANT_NEE = range(6)
PULSE_NAN, PULSE_ATTEMPT_LIMIT = 0x1, 0x2

EXPORTS = ["optifax_create", "optifax_destroy", "optifax_status_string", "optifax_last_error",
           "optifax_opo_mex_batch", "optifax_propagate", "optifax_opo_run", "optifax_propagate_noalloc",
           "optifax_propagate_fp64", "optifax_propagate_f32x2", "optifax_gemm_bf16", "optifax_tc_error",
           "optifax_fno_param_count", "optifax_fno_create", "optifax_fno_destroy", "optifax_fno_set_params",
           "optifax_fno_get_params", "optifax_fno_forward", "optifax_fno_backward", "optifax_fno_adam",
           "optifax_ff_encode", "optifax_ff_step",
           "optifax_ff_encode_env", "optifax_ff_decode_env", "optifax_setup_work_bytes", "optifax_setup_pulses",
           "optifax_gnlse", "optifax_fno_set_grads", "optifax_propagate_graph", "optifax_graph_launch",
           "optifax_graph_kernels", "optifax_graph_destroy"]

_lib = None


class OptifaxPulse(ctypes.Structure):
    _fields_ = [("n_points", ctypes.c_int32), ("n_steps", ctypes.c_int32),
                ("E_in", ctypes.c_void_p), ("A_out", ctypes.c_void_p),
                ("alpha", ctypes.c_void_p), ("beta", ctypes.c_void_p), ("G", ctypes.c_void_p),
                ("Ap", ctypes.c_void_p), ("stepmods", ctypes.c_void_p),
                ("trace", ctypes.c_void_p), ("forced", ctypes.c_void_p),
                ("trace_cap", ctypes.c_int32), ("n_forced", ctypes.c_int32),
                ("w0", ctypes.c_float), ("h", ctypes.c_float),
                ("bdiffw0", ctypes.c_double), ("dt", ctypes.c_double),
                ("max_err", ctypes.c_float), ("min_err", ctypes.c_float), ("sel", ctypes.c_float),
                ("stepmods_limit", ctypes.c_int32), ("cta_points", ctypes.c_int32)]


class OptifaxPulseStats(ctypes.Structure):
    _fields_ = [("attempts", ctypes.c_int32), ("accepted", ctypes.c_int32),
                ("rejected", ctypes.c_int32), ("status", ctypes.c_int32),
                ("z_steps", ctypes.c_int64), ("k_final", ctypes.c_float),
                ("stepmod_final", ctypes.c_float), ("n_chunks", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 3)]


STATS_BYTES = ctypes.sizeof(OptifaxPulseStats)


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load liboptifax.so (building it in-tree first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"optifax CUDA library not built: {path}")
        _build.build()
    lib = ctypes.CDLL(path)
    vp, i32, f32, f64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_float, ctypes.c_double
    lib.optifax_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int]
    lib.optifax_create.restype = ctypes.c_int
    lib.optifax_destroy.argtypes = [vp]
    lib.optifax_destroy.restype = ctypes.c_int
    lib.optifax_status_string.argtypes = [ctypes.c_int]
    lib.optifax_status_string.restype = ctypes.c_char_p
    lib.optifax_last_error.argtypes = [vp]
    lib.optifax_last_error.restype = ctypes.c_char_p
    lib.optifax_opo_mex_batch.argtypes = [vp, vp, vp, vp, f32, f64, f32, i32, f64, vp, f32, f32, f32,
                                          vp, vp, i32, i32, i32, i32, vp, vp, vp, vp]
    lib.optifax_opo_mex_batch.restype = ctypes.c_int
    lib.optifax_propagate.argtypes = [vp, ctypes.POINTER(OptifaxPulse), i32, i32, i32, i32, vp, vp]
    lib.optifax_propagate.restype = ctypes.c_int
    lib.optifax_propagate_graph.argtypes = [vp, ctypes.POINTER(OptifaxPulse), i32, i32, i32, i32, vp,
                                            ctypes.POINTER(vp)]
    lib.optifax_propagate_graph.restype = ctypes.c_int
    lib.optifax_graph_launch.argtypes = [vp, vp]
    lib.optifax_graph_launch.restype = ctypes.c_int
    lib.optifax_graph_kernels.argtypes = [vp]
    lib.optifax_graph_kernels.restype = ctypes.c_int
    lib.optifax_graph_destroy.argtypes = [vp]
    lib.optifax_graph_destroy.restype = ctypes.c_int
    lib.optifax_propagate_noalloc.argtypes = [ctypes.POINTER(OptifaxPulse), i32, vp, vp]
    lib.optifax_propagate_noalloc.restype = ctypes.c_int
    lib.optifax_propagate_fp64.argtypes = [i32, i32, i32, vp, vp, vp, vp, vp, i32, f64, f64, f64, f64,
                                           f64, f64, f64, i32, vp, i32, vp, vp]
    lib.optifax_propagate_fp64.restype = ctypes.c_int
    lib.optifax_propagate_f32x2.argtypes = lib.optifax_propagate_fp64.argtypes
    lib.optifax_propagate_f32x2.restype = ctypes.c_int
    i64 = ctypes.c_int64
    lib.optifax_gemm_bf16.argtypes = [vp, i64, i64, vp, i64, i64, vp, i64, i32, i32, i32, i32, i32, vp]
    lib.optifax_gemm_bf16.restype = ctypes.c_int
    lib.optifax_tc_error.argtypes = [ctypes.POINTER(i32), i32]
    lib.optifax_tc_error.restype = ctypes.c_int
    lib.optifax_fno_param_count.argtypes = []
    lib.optifax_fno_param_count.restype = ctypes.c_int64
    lib.optifax_fno_create.argtypes = [ctypes.POINTER(vp), i32, i32, i32]
    lib.optifax_fno_create.restype = ctypes.c_int
    lib.optifax_fno_destroy.argtypes = [vp]
    lib.optifax_fno_destroy.restype = ctypes.c_int
    lib.optifax_fno_set_params.argtypes = [vp, vp, vp]
    lib.optifax_fno_set_params.restype = ctypes.c_int
    lib.optifax_fno_get_params.argtypes = [vp, vp, vp]
    lib.optifax_fno_get_params.restype = ctypes.c_int
    lib.optifax_fno_forward.argtypes = [vp, vp, vp, i32, vp]
    lib.optifax_fno_forward.restype = ctypes.c_int
    lib.optifax_fno_backward.argtypes = [vp, vp, vp, vp, i32, vp, vp, vp]
    lib.optifax_fno_backward.restype = ctypes.c_int
    lib.optifax_fno_set_grads.argtypes = [vp, vp, vp]
    lib.optifax_fno_set_grads.restype = ctypes.c_int
    lib.optifax_fno_adam.argtypes = [vp, f32, f32, f32, f32, f32, i32, vp]
    lib.optifax_fno_adam.restype = ctypes.c_int
    lib.optifax_ff_encode.argtypes = [vp, i64, i32, i32, i32, i32, i32, f32, vp, vp, i32, vp, vp]
    lib.optifax_ff_encode.restype = ctypes.c_int
    lib.optifax_ff_step.argtypes = [vp, vp, vp, vp, vp, vp, vp, i32, i32, i32, i32, f32, vp, vp, vp, vp]
    lib.optifax_ff_step.restype = ctypes.c_int
    lib.optifax_ff_encode_env.argtypes = [vp, i64, i32, i32, i32, ctypes.POINTER(i32), f32, vp, vp, i32, vp, vp]
    lib.optifax_ff_encode_env.restype = ctypes.c_int
    lib.optifax_ff_decode_env.argtypes = [vp, vp, i32, i32, ctypes.POINTER(i32), f32, vp, vp]
    lib.optifax_ff_decode_env.restype = ctypes.c_int
    lib.optifax_setup_work_bytes.argtypes = [i32]
    lib.optifax_setup_work_bytes.restype = ctypes.c_int64
    lib.optifax_setup_pulses.argtypes = [ctypes.POINTER(OptifaxSetup), i32, vp, i64, vp]
    lib.optifax_setup_pulses.restype = ctypes.c_int
    lib.optifax_gnlse.argtypes = [vp, ctypes.POINTER(OptifaxGnlsePulse), i32, vp]
    lib.optifax_gnlse.restype = ctypes.c_int
    _lib = lib
    return lib


class OptifaxSetup(ctypes.Structure):
    _fields_ = [("n_points", ctypes.c_int32), ("n_steps", ctypes.c_int32),
                ("window", ctypes.c_double), ("dt", ctypes.c_double), ("lambda_ref", ctypes.c_double),
                ("length", ctypes.c_double), ("step_size", ctypes.c_double), ("celsius", ctypes.c_double),
                ("g_scale", ctypes.c_double), ("walls", ctypes.c_void_p), ("n_walls", ctypes.c_int32),
                ("seed", ctypes.c_int32), ("pump_lambda", ctypes.c_double), ("pump_t_rms", ctypes.c_double),
                ("pump_energy", ctypes.c_double), ("waist", ctypes.c_double), ("n_medium", ctypes.c_double),
                ("lambda_lo_nm", ctypes.c_double), ("lambda_hi_nm", ctypes.c_double),
                ("alpha", ctypes.c_void_p), ("beta", ctypes.c_void_p), ("G", ctypes.c_void_p),
                ("E", ctypes.c_void_p)]


class OptifaxGnlseStats(ctypes.Structure):
    _fields_ = [("attempts", ctypes.c_int32), ("accepted", ctypes.c_int32), ("status", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class OptifaxGnlsePulse(ctypes.Structure):
    _fields_ = [("n_points", ctypes.c_int32), ("n_saves", ctypes.c_int32),
                ("A", ctypes.c_void_p), ("B", ctypes.c_void_p), ("W", ctypes.c_void_p), ("RW", ctypes.c_void_p),
                ("gamma", ctypes.c_double), ("fr", ctypes.c_double), ("dT", ctypes.c_double),
                ("alpha", ctypes.c_double), ("length", ctypes.c_double), ("rtol", ctypes.c_double),
                ("atol", ctypes.c_double), ("AT_out", ctypes.c_void_p), ("AW_out", ctypes.c_void_p),
                ("trace", ctypes.c_void_p), ("trace_cap", ctypes.c_int32), ("max_attempts", ctypes.c_int32),
                ("stats", ctypes.c_void_p)]


class OptifaxError(RuntimeError):
    pass


def check(rc: int, handle=None, what: str = "optifax"):
    if rc != 0:
        lib = load()
        detail = lib.optifax_last_error(handle).decode() if handle else ""
        raise OptifaxError(f"{what}: {lib.optifax_status_string(rc).decode()} ({rc}) {detail}")


class Context:
    """Owns an optifax_handle (twiddle tables, descriptor staging) on one device."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        check(self.lib.optifax_create(ctypes.byref(h), int(device)), None, "optifax_create")
        self.handle = h
        self.device = device

    def close(self):
        if getattr(self, "handle", None):
            self.lib.optifax_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
