"""ctypes binding of ref_mex.cpp: the reference's own CUDA kernels on the GPU
(TEST INFRASTRUCTURE ONLY; tests/ and bench.py load it, the product never does).

The kernels come from the MEX files OPO_CUDA_{BATCH_XTAL,BATCH_OP,NO_BC,HARD_BC}.cu
and ode23/OPO_CUDA_ODE23.cu compiled unmodified into oracle/_ref/*.cubin
(oracle/Makefile, target ``ref``, built where the reference source is present and
shipped as files); ref_mex.cpp drives them with cuFFT as the MEX drivers
OPO_TEST_CUDA do.  ``run`` / ``run_ode23`` take the MEX's inputs in its units (FP32
arrays, FP64 bdiffw0 and dt) and return its three outputs plus the per-attempt
decision trace.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(_HERE, "_ref", "opo_cuda_batch_xtal.cubin")
CUBIN_ODE23 = os.path.join(_HERE, "_ref", "opo_cuda_ode23.cubin")
# Heun MEX variants, numbered as optifax_gb300's OPTIFAX_VARIANT_*: BATCH_XTAL,
# BATCH_OP, NO_BC, HARD_BC
HEUN_CUBINS = [os.path.join(_HERE, "_ref", f"opo_cuda_{v}.cubin")
               for v in ("batch_xtal", "batch_op", "no_bc", "hard_bc")]
_LIB_PATH = os.path.join(_HERE, "_build", "libref_mex.so")
_lib = None


def reference_kernel_sources():
    """The reference's MEX source directory (toolbox/lib/MEXlib/src), or None where
    the reference is absent (the GPU host: the cubins travel as built files).  The
    checkout is found through OPTIFAX_REFERENCE, else at its location in the
    build container."""
    root = os.environ.get("OPTIFAX_REFERENCE", "/root/reference")
    src = os.path.join(root, "toolbox", "lib", "MEXlib", "src")
    return src if os.path.isdir(src) else None


def build() -> None:
    """Build the harness (and, where the reference source exists, the cubins)."""
    cmd = ["make", "-s", "-C", _HERE, "ref"]
    src = reference_kernel_sources()
    if src:
        cmd.append("REF_SRC=" + src)
    subprocess.run(cmd, check=True)


def available(cubin: str = CUBIN):
    """(True, "") when the compiled reference kernels are present, else (False, why)."""
    if not os.path.exists(cubin):
        return False, (f"oracle/_ref/{os.path.basename(cubin)} absent "
                       "(built only where the reference source is)")
    return True, ""


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB_PATH)
        _lib.refmex_run.restype = ctypes.c_int
        _lib.refmex_run_ode23.restype = ctypes.c_int
        _lib.refmex_last_error.restype = ctypes.c_char_p
    return _lib


def n_chunks(n_steps: int, sel: float, variant: int = 0) -> int:
    """Chunk count as the MEX driver computes it: FP32 and rounded up for BATCH_XTAL
    and BATCH_OP (:403-407), integer and truncated for NO_BC and HARD_BC."""
    if variant >= 2:
        return int(n_steps) // int(sel)
    s = np.float32(n_steps)
    sel = np.float32(sel)
    n = int(np.float32(s / sel))
    if np.float32(n) * sel < s:
        n += 1
    return n


@dataclass
class RefResult:
    A: np.ndarray          # complex64 (B, N): output 0 (A0)
    Ap: np.ndarray         # complex64 (B, nchunks, N): output 1
    stepmods: np.ndarray   # float32 (S,): output 2
    trace: np.ndarray      # int32 (attempts, 3): k, stepmod, flags|8 accepted|own flags<<4
    attempts: int
    seconds: float         # device wall time of the pass


def run(E, alpha, G, beta, *, w0, bdiffw0, h, n_steps, dt, max_err, min_err, sel,
        Ap=None, stepmods=None, trace_cap=200000, forced=None, variant=0) -> RefResult:
    """One Heun MEX pass through the reference's kernels of `variant` (0 BATCH_XTAL,
    1 BATCH_OP, 2 NO_BC, 3 HARD_BC)."""
    E = np.ascontiguousarray(np.atleast_2d(E), dtype=np.complex64)
    B, N = E.shape
    S = int(n_steps)
    nch = max(n_chunks(S, sel, variant), 1)
    alpha = np.ascontiguousarray(alpha, dtype=np.float32)
    beta = np.ascontiguousarray(beta, dtype=np.float32)
    G = np.ascontiguousarray(G, dtype=np.float32).ravel()
    if variant == 0:
        if G.size == S:
            G = np.tile(G, B)      # one G row per pulse (XTAL layout, KN_kernel :222)
        if G.size != S * B:
            raise ValueError("G must hold S or S*B values")
    elif G.size != S:
        raise ValueError("G must hold S values (one poling shared by the batch)")
    Ap = np.zeros((B, nch, N), np.complex64) if Ap is None else np.ascontiguousarray(Ap, np.complex64).copy()
    sm = np.zeros(S, np.float32) if stepmods is None else np.ascontiguousarray(stepmods, np.float32).copy()
    A = np.zeros((B, N), np.complex64)
    trace = np.zeros(max(trace_cap, 1) * 3, np.int32)
    nat = ctypes.c_int(0)
    secs = ctypes.c_double(0.0)
    fz = None if forced is None else np.ascontiguousarray(forced, np.int32).ravel()
    fptr = ctypes.POINTER(ctypes.c_float)
    iptr = ctypes.POINTER(ctypes.c_int)
    rc = lib().refmex_run(
        HEUN_CUBINS[variant].encode(), ctypes.c_int(variant), E.view(np.float32).ctypes.data_as(fptr),
        ctypes.c_int(N), ctypes.c_int(B),
        alpha.ctypes.data_as(fptr), G.ctypes.data_as(fptr), beta.ctypes.data_as(fptr),
        ctypes.c_float(w0), ctypes.c_double(bdiffw0), ctypes.c_float(h), ctypes.c_int(S),
        ctypes.c_double(dt), ctypes.c_float(max_err), ctypes.c_float(min_err), ctypes.c_float(sel),
        Ap.view(np.float32).ctypes.data_as(fptr), ctypes.c_longlong(Ap.size * 2),
        sm.ctypes.data_as(fptr), A.view(np.float32).ctypes.data_as(fptr),
        trace.ctypes.data_as(iptr), ctypes.c_int(trace_cap), ctypes.byref(nat),
        None if fz is None else fz.ctypes.data_as(iptr), ctypes.c_int(0 if fz is None else fz.size),
        ctypes.byref(secs))
    if rc != 0:
        raise RuntimeError("reference kernels: " + lib().refmex_last_error().decode())
    n = min(nat.value, trace_cap)
    return RefResult(A=A, Ap=Ap, stepmods=sm, trace=trace[:3 * n].reshape(n, 3).copy(),
                     attempts=nat.value, seconds=secs.value)


def run_ode23(E, alpha, G, beta, *, w0, bdiffw0, h, n_steps, dt, max_err, min_err, sel,
              Ap=None, stepmods=None, trace_cap=200000, forced=None) -> RefResult:
    """One pulse through the reference's ODE23 (RK23) kernels and driver."""
    E = np.ascontiguousarray(np.atleast_2d(E), dtype=np.complex64)
    if E.shape[0] != 1:
        raise ValueError("ODE23 reference kernels: one pulse per call")
    N = E.shape[1]
    S = int(n_steps)
    sel_i = int(sel)
    nch = S // sel_i
    alpha = np.ascontiguousarray(alpha, dtype=np.float32)
    beta = np.ascontiguousarray(beta, dtype=np.float32)
    G = np.ascontiguousarray(G, dtype=np.float32).ravel()[:S].copy()
    Ap = np.zeros((1, max(nch, 1), N), np.complex64) if Ap is None else np.ascontiguousarray(Ap, np.complex64).copy()
    sm = np.zeros(S, np.float32) if stepmods is None else np.ascontiguousarray(stepmods, np.float32).copy()
    A = np.zeros((1, N), np.complex64)
    trace = np.zeros(max(trace_cap, 1) * 3, np.int32)
    nat = ctypes.c_int(0)
    secs = ctypes.c_double(0.0)
    fz = None if forced is None else np.ascontiguousarray(forced, np.int32).ravel()
    fptr = ctypes.POINTER(ctypes.c_float)
    iptr = ctypes.POINTER(ctypes.c_int)
    rc = lib().refmex_run_ode23(
        CUBIN_ODE23.encode(), E.view(np.float32).ctypes.data_as(fptr), ctypes.c_int(N),
        alpha.ctypes.data_as(fptr), G.ctypes.data_as(fptr), beta.ctypes.data_as(fptr),
        ctypes.c_float(w0), ctypes.c_double(bdiffw0), ctypes.c_float(h), ctypes.c_int(S),
        ctypes.c_double(dt), ctypes.c_float(max_err), ctypes.c_float(min_err), ctypes.c_int(sel_i),
        Ap.view(np.float32).ctypes.data_as(fptr), ctypes.c_longlong(Ap.size * 2),
        sm.ctypes.data_as(fptr), A.view(np.float32).ctypes.data_as(fptr),
        trace.ctypes.data_as(iptr), ctypes.c_int(trace_cap), ctypes.byref(nat),
        None if fz is None else fz.ctypes.data_as(iptr), ctypes.c_int(0 if fz is None else fz.size),
        ctypes.byref(secs))
    if rc != 0:
        raise RuntimeError("reference ODE23 kernels: " + lib().refmex_last_error().decode())
    n = min(nat.value, trace_cap)
    return RefResult(A=A, Ap=Ap, stepmods=sm, trace=trace[:3 * n].reshape(n, 3).copy(),
                     attempts=nat.value, seconds=secs.value)
