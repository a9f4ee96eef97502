"""TEST INFRASTRUCTURE ONLY: FP64 restatement of the chi(3) fibre GNLSE solver
(toolbox/lib/internal/main/gnlsefib.m) -- the oracle for optifax_gb300's GPU
kernel in csrc/ofx_gnlse.cu.  Only tests/ and bench.py's cpu_baseline leg import
it.  propagate_c binds the C restatement of the same scheme (oracle/gnlse_oracle.c),
which runs independent pulses in parallel.

The equation, grids and operators follow gnlsefib.m:22-66: the interaction-picture
spectral field AW obeys dAW/dz = i gamma W ifft(AT ((1 - fR) |AT|^2 + RS)) e^{-Lz},
AT = fft(AW e^{Lz}), RS = dT fR fft(ifft(|AT|^2) RW), L = i sum_m beta_m V^m/m! - alpha/2,
W = V + w0 with gamma/w0 when a shock frequency is given, RW = n ifft(fftshift(hR)),
in MATLAB's fft/ifft conventions (fft: exp(-i ...), ifft: exp(+i ...) / n).

gnlsefib.m integrates with MATLAB's ode45 (RelTol 1e-5, AbsTol 1e-12, NormControl
on, gnlsefib.m:77-80), a closed third-party binary.  This oracle and the GPU kernel
instead share one published scheme: the Dormand-Prince 5(4) pair (FSAL) with the
same tolerances and NormControl error norm, err = ||h sum e_i k_i||_2 /
max(||y||_2, ||y_new||_2, AbsTol/RelTol), accept when err <= RelTol, the standard
controller h *= min(5, max(0.1, 0.8 (RelTol/err)^(1/5))) (no growth after a
rejection), steps at most a tenth of the fibre and clamped to land on the save
points (so no dense-output interpolation).  Positions are integers in a unit of
flength / 2^40, so the GPU and the oracle evaluate at identical z; the oracle can
replay the GPU's (step, accept) sequence so that the comparison is arithmetic only.
Parity with MATLAB's own ode45 is not claimed (unpinned): both integrate the same
ODE to the same tolerance.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np

Z_BITS = 40                      # z in units of flength / 2^40

# Dormand-Prince 5(4) tableau (Dormand & Prince 1980)
DP_C = [0.0, 1 / 5, 3 / 10, 4 / 5, 8 / 9, 1.0, 1.0]
DP_A = [[],
        [1 / 5],
        [3 / 40, 9 / 40],
        [44 / 45, -56 / 15, 32 / 9],
        [19372 / 6561, -25360 / 2187, 64448 / 6561, -212 / 729],
        [9017 / 3168, -355 / 33, 46732 / 5247, 49 / 176, -5103 / 18656],
        [35 / 384, 0.0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84]]
DP_E = [71 / 57600, 0.0, -71 / 16695, 71 / 1920, -17253 / 339200, 22 / 525, -1 / 40]


@dataclass
class GnlseOps:
    """The operators of gnlsefib.m:22-50 in FFT order."""
    n: int
    dT: float
    B: np.ndarray        # real dispersion sum_m beta_m V^m / m! (rad/m), FFT order
    alpha: float         # field loss coefficient: L = iB - alpha/2
    W: np.ndarray        # V + w0 (shock) or 1, FFT order
    gamma: float         # gamma / w0 with shock, else gamma
    RW: np.ndarray       # n ifft(fftshift(hR)), complex, FFT order
    fr: float
    raman: bool


def gnlse_ops(T, w0, gamma, betas, loss, fr, RT) -> GnlseOps:
    """gnlsefib.m:22-50."""
    T = np.asarray(T, dtype=np.float64)
    n = T.size
    dT = float(T[1] - T[0])
    V = 2 * np.pi * np.arange(-n // 2, n // 2, dtype=np.float64) / (n * dT)
    alpha = math.log(10.0 ** (loss / 10.0))
    B = np.zeros(n)
    for i, b in enumerate(betas):
        B += b / math.factorial(i + 2) * V ** (i + 2)
    if abs(w0) > np.finfo(float).eps:
        g = gamma / w0
        W = V + w0
    else:
        g = gamma
        W = np.ones(n)
    RT = np.atleast_1d(np.asarray(RT, dtype=np.float64))
    raman = RT.size > 1 and abs(fr) >= np.finfo(float).eps
    RW = n * np.fft.ifft(np.fft.fftshift(RT)) if raman else np.zeros(n, complex)
    return GnlseOps(n=n, dT=dT, B=np.fft.fftshift(B), alpha=alpha, W=np.fft.fftshift(W), gamma=g,
                    RW=RW, fr=float(fr), raman=raman)


def raman_response(T, tau1=12.2e-15, tau2=32.0e-15):
    """hR(t) of fused silica (Waveguide.m:34-42): (t1^2 + t2^2)/(t1 t2^2) e^{-t/t2} sin(t/t1), t >= 0."""
    T = np.asarray(T, dtype=np.float64)
    h = (tau1 ** 2 + tau2 ** 2) / (tau1 * tau2 ** 2) * np.exp(-T / tau2) * np.sin(T / tau1)
    h[T < 0] = 0.0
    return h


def _lz(ops: GnlseOps, z: float) -> np.ndarray:
    return np.exp(-0.5 * ops.alpha * z) * np.exp(1j * ops.B * z)


def rhs(ops: GnlseOps, z: float, AW: np.ndarray) -> np.ndarray:
    """gnlsefib.m:54-66."""
    e = _lz(ops, z)
    AT = np.fft.fft(AW * e)
    IT = np.abs(AT) ** 2
    if not ops.raman:
        M = np.fft.ifft(AT * IT)
    else:
        RS = ops.dT * ops.fr * np.fft.fft(np.fft.ifft(IT) * ops.RW)
        M = np.fft.ifft(AT * ((1 - ops.fr) * IT + RS))
    return 1j * ops.gamma * ops.W * M / e


@dataclass
class GnlseResult:
    Z: np.ndarray        # (nsaves,) positions
    AT: np.ndarray       # (nsaves, n) time-domain field, natural time order
    AW: np.ndarray       # (nsaves, n) spectral field, fftshifted and scaled by dT n (gnlsefib.m:82-89)
    steps: list          # (h_count, accepted) per attempt
    attempts: int
    accepted: int


def propagate(ops: GnlseOps, A, flength, nsaves, rtol=1e-5, atol=1e-12, forced=None) -> GnlseResult:
    """Integrate from z = 0 to flength, saving at linspace(0, flength, nsaves).
    forced: optional sequence of (h_count, accepted) replacing the step control."""
    n = ops.n
    unit = flength / 2 ** Z_BITS
    total = 1 << Z_BITS
    # save points i total / (nsaves - 1), rounded half up in integers (as the GPU kernel)
    saves = [(i * total + (nsaves - 1) // 2) // (nsaves - 1) for i in range(nsaves)]
    hmax = total // 10
    thr = atol / rtol
    y = np.fft.ifft(np.asarray(A, dtype=np.complex128))
    zc = 0
    out_aw = np.zeros((nsaves, n), complex)
    out_at = np.zeros((nsaves, n), complex)

    def save(i, zc_, y_):
        aw = y_ * _lz(ops, zc_ * unit)
        out_at[i] = np.fft.fft(aw)
        out_aw[i] = np.fft.fftshift(aw) * ops.dT * n

    save(0, 0, y)
    f = rhs(ops, 0.0, y)
    ny = np.linalg.norm(y)
    nf = np.linalg.norm(f)
    # initial step: the error-per-step estimate 0.8 rtol^(1/5) max(||y||, thr) / ||f||
    h = hmax if nf == 0.0 else min(hmax, max(1, int((0.8 * rtol ** 0.2) * max(ny, thr) / nf / unit)))
    steps = []
    att = acc = 0
    fi = 0
    for si in range(1, len(saves)):
        target = saves[si]
        while zc < target:
            hc = min(h, target - zc)
            if forced is not None:
                if fi >= len(forced):
                    raise RuntimeError("forced schedule exhausted")
                hc = int(forced[fi][0])
            hz = hc * unit
            k = [f]
            for s in range(1, 7):
                ys = y + hz * sum(DP_A[s][j] * k[j] for j in range(s) if DP_A[s][j] != 0.0)
                zs = (zc + int(round(DP_C[s] * hc))) * unit
                k.append(rhs(ops, zs, ys))
            ynew = y + hz * sum(DP_A[6][j] * k[j] for j in range(6) if DP_A[6][j] != 0.0)
            errv = hz * sum(DP_E[j] * k[j] for j in range(7) if DP_E[j] != 0.0)
            nyn = np.linalg.norm(ynew)
            err = np.linalg.norm(errv) / max(ny, nyn, thr)
            ok = err <= rtol
            if forced is not None:
                ok = bool(forced[fi][1])
                fi += 1
            steps.append((hc, int(ok)))
            att += 1
            fac = 5.0 if err == 0.0 else 0.8 * (rtol / err) ** 0.2
            if ok:
                acc += 1
                zc += hc
                y, f, ny = ynew, k[6], nyn
                h = min(hmax, max(1, int(hc * min(5.0, fac))))
            else:
                h = max(1, int(hc * max(0.1, min(1.0, fac))))
        save(si, zc, y)
    Z = np.array([s * unit for s in saves])
    return GnlseResult(Z=Z, AT=out_at, AW=out_aw, steps=steps, attempts=att, accepted=acc)


class _CParams(ctypes.Structure):
    """ofx_gnlse_params (oracle/gnlse_oracle.h)."""
    _fields_ = [("n", ctypes.c_int), ("n_saves", ctypes.c_int), ("gamma", ctypes.c_double),
                ("fr", ctypes.c_double), ("dT", ctypes.c_double), ("alpha", ctypes.c_double),
                ("length", ctypes.c_double), ("rtol", ctypes.c_double), ("atol", ctypes.c_double)]


def propagate_c(ops: GnlseOps, A, flength, nsaves, rtol=1e-5, atol=1e-12, forced=None, nthreads=0,
                trace_cap=200000):
    """The C restatement (oracle/gnlse_oracle.c) of propagate() for a batch of fields
    A (B x n, or n) in parallel; forced: per pulse a sequence of (h_count, accepted),
    or one sequence for a single pulse.  Returns one GnlseResult per pulse."""
    from . import oracle as orc
    lib = orc.lib()
    A = np.ascontiguousarray(np.atleast_2d(np.asarray(A, dtype=np.complex128)))
    nb, n = A.shape
    if n != ops.n:
        raise ValueError("fields must have the operators' grid size")
    p = _CParams(n=n, n_saves=int(nsaves), gamma=ops.gamma, fr=ops.fr if ops.raman else 0.0, dT=ops.dT,
                 alpha=ops.alpha, length=float(flength), rtol=float(rtol), atol=float(atol))
    B = np.ascontiguousarray(ops.B, dtype=np.float64)
    W = np.ascontiguousarray(ops.W, dtype=np.float64)
    RW = np.ascontiguousarray(ops.RW, dtype=np.complex128) if ops.raman else None
    AT = np.zeros((nb, nsaves, n), dtype=np.complex128)
    AW = np.zeros((nb, nsaves, n), dtype=np.complex128)
    trace = np.zeros((nb, max(trace_cap, 1), 2), dtype=np.int64)
    n_forced = 0
    fz = None
    if forced is not None:
        fl = [forced] if nb == 1 and len(forced) and np.ndim(forced[0]) == 1 else list(forced)
        n_forced = max(len(f) for f in fl)
        fz = np.zeros((nb, max(n_forced, 1), 2), dtype=np.int64)
        for b, f in enumerate(fl):
            fz[b, :len(f)] = np.asarray(f, dtype=np.int64).reshape(-1, 2)
    att = np.zeros(nb, dtype=np.int32)
    acc = np.zeros(nb, dtype=np.int32)
    dp = lambda a: a.ctypes.data_as(ctypes.c_void_p) if a is not None else None
    fn = lib.ofx_gnlse_oracle_run
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(_CParams), ctypes.c_int] + [ctypes.c_void_p] * 7 + \
        [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    rc = fn(ctypes.byref(p), nb, dp(A), dp(B), dp(W), dp(RW), dp(AT), dp(AW), dp(trace), trace_cap,
            dp(fz), n_forced, dp(att), dp(acc), int(nthreads))
    if rc != 0:
        raise RuntimeError(f"ofx_gnlse_oracle_run failed ({rc})")
    total = 1 << Z_BITS
    Z = np.array([((i * total + (nsaves - 1) // 2) // (nsaves - 1)) * (flength / total) for i in range(nsaves)])
    out = []
    for b in range(nb):
        k = min(int(att[b]), trace_cap)
        steps = [(int(h), int(a)) for h, a in trace[b, :k]]
        out.append(GnlseResult(Z=Z, AT=AT[b], AW=AW[b], steps=steps, attempts=int(att[b]), accepted=int(acc[b])))
    return out
