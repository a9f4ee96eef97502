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
on, outputs at linspace(0, flength, nsaves); gnlsefib.m:70-80).  ode45 itself is a
closed binary; its algorithm is published (Shampine & Reichelt, "The MATLAB ODE
Suite", SIAM J. Sci. Comput. 18(1), 1997) and restated here, shared by this oracle,
the C restatement and the GPU kernel:
  * the Dormand-Prince 5(4) pair (FSAL), NormControl error norm
    err = ||h sum e_i k_i||_2 / max(||y||_2, ||y_new||_2, AbsTol/RelTol), accepted
    when err <= RelTol;
  * initial step: h = min(hmax, span), reduced to 1/rh when h rh > 1, with
    rh = (||f0|| / max(||y0||, threshold)) / (0.8 RelTol^(1/5));
  * hmax = span / 10 (MaxStep's default); before each step the step is stretched
    to the end of the span when 1.1 h >= the remaining length;
  * after a failed step: the first failure of the step scales h by
    max(0.1, 0.8 (RelTol/err)^(1/5)), later ones halve it;
  * after an accepted step with no failure: h /= 1.25 (err/RelTol)^(1/5) when that
    divisor exceeds 0.2, else h *= 5; after a step that failed first, h is kept;
  * the steps do not stop at the save points: a save point inside an accepted step
    is output from a separate Dormand-Prince step of exactly that length from the
    step's start (5th order; MATLAB interpolates with its 4th-order continuous
    extension instead, so saved values inside a step differ from MATLAB's by the
    order of the local error, while the step sequence is ode45's).
Positions are integers in a unit of flength / 2^40 (hmin = 1 unit), so the GPU and
the oracle evaluate at identical z; the oracle can replay the GPU's (step, accept)
sequence so that the comparison is arithmetic only.  Parity with MATLAB's own ode45
output is not claimed (no MATLAB): the step-control rules are restated from the
publication, not compared with a MATLAB run.
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


def _dp_step(ops: GnlseOps, y, f, zc, hc, unit, last_stage=6):
    """Stages of one Dormand-Prince step of hc units from (zc, y) with k1 = f: returns
    (the 5th-order value, [k1..k7] or [k1..k6] when last_stage == 5)."""
    hz = hc * unit
    k = [f]
    for s in range(1, last_stage + 1):
        ys = y + hz * sum(DP_A[s][j] * k[j] for j in range(s) if DP_A[s][j] != 0.0)
        zs = (zc + int(round(DP_C[s] * hc))) * unit
        k.append(rhs(ops, zs, ys))
    ynew = y + hz * sum(DP_A[6][j] * k[j] for j in range(6) if DP_A[6][j] != 0.0)
    return ynew, k


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
    si = 1
    f = rhs(ops, 0.0, y)
    ny = np.linalg.norm(y)
    nf = np.linalg.norm(f)
    # initial step (ode45, NormControl): min(hmax, span), 1/rh when h rh > 1
    h = hmax
    rh = (nf / max(ny, thr)) / (0.8 * rtol ** 0.2)
    if h * unit * rh > 1.0:
        h = max(1, int(1.0 / rh / unit))
    steps = []
    att = acc = 0
    fi = 0
    while zc < total:
        h = min(hmax, max(1, h))
        hc = h
        if 1.1 * hc >= total - zc:
            hc = total - zc                      # stretch to the end of the span
        nofailed = True
        while True:
            if forced is not None:
                if fi >= len(forced):
                    raise RuntimeError("forced schedule exhausted")
                hc = int(forced[fi][0])
            ynew, k = _dp_step(ops, y, f, zc, hc, unit)
            errv = (hc * unit) * sum(DP_E[j] * k[j] for j in range(7) if DP_E[j] != 0.0)
            nyn = np.linalg.norm(ynew)
            err = np.linalg.norm(errv) / max(ny, nyn, thr)
            ok = err <= rtol
            if forced is not None:
                ok = bool(forced[fi][1])
                fi += 1
            steps.append((hc, int(ok)))
            att += 1
            if ok:
                break
            if nofailed:
                nofailed = False
                fac = 0.1 if not np.isfinite(err) else max(0.1, 0.8 * (rtol / err) ** 0.2)
                hc = max(1, int(hc * fac))
            else:
                hc = max(1, hc // 2)
        acc += 1
        # save points inside the step: a separate step of exactly that length from zc
        while si < nsaves and saves[si] < zc + hc:
            ys, _ = _dp_step(ops, y, f, zc, saves[si] - zc, unit, last_stage=5)
            save(si, saves[si], ys)
            si += 1
        zc += hc
        y, f, ny = ynew, k[6], nyn
        if si < nsaves and saves[si] == zc:
            save(si, zc, y)
            si += 1
        if nofailed:
            temp = 1.25 * (err / rtol) ** 0.2
            h = int(hc / temp) if temp > 0.2 else 5 * hc
        else:
            h = hc
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
