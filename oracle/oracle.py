"""ctypes binding of the FP64 CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py (cpu_baseline leg and the
``--impl reference`` arm) import this module.  The product path in
optifax_gb300/ never does.  Parity status: pinned to the reference's own CUDA kernels for the
MEX schedules (oracle/ref_mex.py, tests/test_reference_kernels_gpu.py); the
NEE_CPU.m schedule is unpinned (see oracle.c header).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboptifax_oracle.so")
_lib = None

HEUN_MEX, RK23_MEX, HEUN_NEE = 0, 1, 2
TIME_SHIFTED, TIME_UNSHIFTED, TIME_NEE = 0, 1, 2
ABC_SOFT, ABC_NONE, ABC_HARD = 0, 1, 2
CHUNKS_CEIL, CHUNKS_TRUNC = 0, 1


class _Params(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int), ("time_mode", ctypes.c_int), ("abc_mode", ctypes.c_int),
                ("chunk_mode", ctypes.c_int), ("g_per_pulse", ctypes.c_int),
                ("stepmods_limit", ctypes.c_int), ("shared_schedule", ctypes.c_int),
                ("N", ctypes.c_int), ("B", ctypes.c_int), ("S", ctypes.c_int),
                ("w0", ctypes.c_double), ("bdiffw0", ctypes.c_double), ("h", ctypes.c_double),
                ("dt", ctypes.c_double), ("maxErr", ctypes.c_double), ("minErr", ctypes.c_double),
                ("sel", ctypes.c_double)]


class _Stats(ctypes.Structure):
    _fields_ = [("attempts", ctypes.c_int), ("accepted", ctypes.c_int), ("rejected", ctypes.c_int),
                ("nchunks", ctypes.c_int), ("z_steps", ctypes.c_longlong),
                ("k_final", ctypes.c_double), ("stepmod_final", ctypes.c_double),
                ("pct_max_last", ctypes.c_double), ("status", ctypes.c_int), ("pad", ctypes.c_int)]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    srcs = ("oracle.c", "oracle.h", "gnlse_oracle.c", "gnlse_oracle.h", "oracle_fft.h", "Makefile")
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(os.path.join(_HERE, f)) for f in srcs):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB_PATH)
        _lib.ofx_oracle_run.restype = ctypes.c_int
        _lib.ofx_oracle_fft.restype = ctypes.c_int
    return _lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def _iptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if a is not None else None


@dataclass
class OracleResult:
    A: np.ndarray            # complex128 (B, N): fftshifted time field
    Ap: np.ndarray           # complex128 flat, reference layout
    stepmods: np.ndarray     # float64 (S,) or (B, S)
    trace: list              # per schedule: int array (n_attempts, 3)
    stats: list              # per schedule: dict


def run(E, alpha, G, beta, *, w0, bdiffw0, h, n_steps, dt, max_err, min_err, sel,
        method=HEUN_MEX, time_mode=TIME_SHIFTED, abc_mode=ABC_SOFT, chunk_mode=CHUNKS_CEIL,
        g_per_pulse=False, stepmods_limit=None, shared_schedule=True,
        Ap=None, ap_chunks=None, stepmods=None, trace_cap=0, forced=None, nthreads=0):
    """Run the oracle.  E: complex (B, N) fftshifted time fields."""
    E = np.ascontiguousarray(np.atleast_2d(E), dtype=np.complex128)
    B, N = E.shape
    S = int(n_steps)
    p = _Params(method=method, time_mode=time_mode, abc_mode=abc_mode, chunk_mode=chunk_mode,
                g_per_pulse=int(bool(g_per_pulse)),
                stepmods_limit=int(stepmods_limit if stepmods_limit is not None else -(-N // 128) * 128),
                shared_schedule=int(bool(shared_schedule)), N=N, B=B, S=S,
                w0=float(w0), bdiffw0=float(bdiffw0), h=float(h), dt=float(dt),
                maxErr=float(max_err), minErr=float(min_err), sel=float(sel))
    alpha = np.ascontiguousarray(alpha, dtype=np.float64)
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    G = np.ascontiguousarray(G, dtype=np.float64).ravel()
    A = np.zeros_like(E)
    if ap_chunks is None:
        ap_chunks = int(S / sel) + (1 if int(S / sel) * sel < S else 0)
    if Ap is None:
        Ap = np.zeros(B * ap_chunks * N, dtype=np.complex128)
    Ap = np.ascontiguousarray(Ap, dtype=np.complex128).ravel().copy()
    nsched = 1 if shared_schedule else B
    if stepmods is None:
        stepmods = np.zeros(S * nsched, dtype=np.float64)
    stepmods = np.ascontiguousarray(stepmods, dtype=np.float64).ravel().copy()
    trace = np.zeros(max(trace_cap, 1) * 3 * nsched, dtype=np.int32)
    nat = np.zeros(nsched, dtype=np.int32)
    stats = (_Stats * nsched)()
    fz = None
    nf = 0
    if forced is not None:
        fz = np.ascontiguousarray(forced, dtype=np.int32).ravel()
        nf = fz.size // nsched
    rc = lib().ofx_oracle_run(ctypes.byref(p), _dptr(E.view(np.float64)), _dptr(alpha), _dptr(G),
                              _dptr(beta), _dptr(A.view(np.float64)), _dptr(Ap.view(np.float64)),
                              ctypes.c_longlong(Ap.size), _dptr(stepmods),
                              _iptr(trace) if trace_cap > 0 else None, ctypes.c_int(trace_cap),
                              _iptr(nat), _iptr(fz), ctypes.c_int(nf), stats, ctypes.c_int(nthreads))
    if rc != 0:
        raise RuntimeError(f"oracle failed rc={rc}")
    tr = []
    for s in range(nsched):
        n = min(int(nat[s]), trace_cap)
        tr.append(trace[s * 3 * max(trace_cap, 1): s * 3 * max(trace_cap, 1) + 3 * n].reshape(n, 3).copy())
    st = [{f: getattr(stats[s], f) for f, _ in _Stats._fields_} for s in range(nsched)]
    return OracleResult(A=A, Ap=Ap, stepmods=stepmods if shared_schedule else stepmods.reshape(B, S),
                        trace=tr, stats=st)


def fft(x, inverse=False):
    x = np.ascontiguousarray(x, dtype=np.complex128)
    out = np.empty_like(x)
    rc = lib().ofx_oracle_fft(_dptr(x.view(np.float64)), _dptr(out.view(np.float64)),
                              ctypes.c_int(x.size), ctypes.c_int(int(inverse)))
    if rc:
        raise ValueError("size must be a power of two")
    return out
