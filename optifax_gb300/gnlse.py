"""chi(3) fibre propagation: the generalised nonlinear Schroedinger equation on the GPU.

Equivalent of OptiFax's gnlsefib (toolbox/lib/internal/main/gnlsefib.m:1-89, called
by gnlsefibsim.m:30 with the fibre's gamma0, betas, Raman fraction and response):
``gnlsefib(T, A, w0, gamma, betas, loss, fr, RT, flength, nsaves)`` returns
``Z, AT, AW, W`` with the reference's meaning (AT: time-domain field at each save,
AW: fftshifted spectral field x dT n, W: absolute angular-frequency grid).  The
operators (gnlsefib.m:22-50) are set up here in FP64; the propagation itself runs in
the sm_103a kernel behind ``optifax_gnlse`` (csrc/ofx_gnlse.cu): an adaptive
Dormand-Prince 5(4) pair with the tolerances the reference gives ode45 (RelTol
1e-5, AbsTol 1e-12, NormControl) under ode45's published step control (initial
step, first-failure scaling then halving, growth only after a step without
failure, steps of at most a tenth of the fibre stretched to its end); save points
inside a step are output by a separate step of exactly that length.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _native as nat
from .solver import context, _stream_ptr, on_stream

GNLSE_POINTS = (512, 1024, 2048, 4096)


def raman_response(T, tau1: float = 12.2e-15, tau2: float = 32.0e-15) -> np.ndarray:
    """hR(t) of fused silica (Waveguide.m:34-42, OpticalFibre.m:25-27):
    (t1^2 + t2^2)/(t1 t2^2) e^{-t/t2} sin(t/t1) for t >= 0, else 0."""
    T = np.asarray(T, dtype=np.float64)
    h = (tau1 ** 2 + tau2 ** 2) / (tau1 * tau2 ** 2) * np.exp(-T / tau2) * np.sin(T / tau1)
    h[T < 0] = 0.0
    return h


@dataclass
class FibreOperators:
    """gnlsefib.m:22-50 in FFT order: L = iB - alpha/2, W, gamma (/ w0 with shock), RW."""
    n: int
    dT: float
    V: np.ndarray            # angular-frequency offsets, centred order
    B: np.ndarray            # sum_m beta_m V^m / m!, FFT order (rad/m)
    alpha: float             # log(10^(loss/10)): field loss enters as -alpha/2
    W: np.ndarray            # FFT order
    gamma: float
    RW: Optional[np.ndarray]  # FFT order, None without Raman
    fr: float


def fibre_operators(T, w0: float, gamma: float, betas: Sequence[float], loss: float, fr: float,
                    RT) -> FibreOperators:
    T = np.asarray(T, dtype=np.float64)
    n = T.size
    dT = float(T[1] - T[0])
    V = 2 * np.pi * np.arange(-n // 2, n // 2, dtype=np.float64) / (n * dT)
    alpha = math.log(10.0 ** (loss / 10.0))
    B = np.zeros(n)
    for i, b in enumerate(betas):
        B += b / math.factorial(i + 2) * V ** (i + 2)
    if abs(w0) > np.finfo(float).eps:
        g, W = gamma / w0, V + w0
    else:
        g, W = gamma, np.ones(n)
    RT = np.atleast_1d(np.asarray(RT, dtype=np.float64))
    raman = RT.size > 1 and abs(fr) >= np.finfo(float).eps
    RW = n * np.fft.ifft(np.fft.fftshift(RT)) if raman else None
    return FibreOperators(n=n, dT=dT, V=V, B=np.fft.fftshift(B), alpha=alpha, W=np.fft.fftshift(W),
                          gamma=g, RW=RW, fr=float(fr) if raman else 0.0)


@dataclass
class GnlseRun:
    Z: np.ndarray                 # (nsaves,) save positions [m]
    AT: torch.Tensor              # (B, nsaves, n) complex64 on the device
    AW: torch.Tensor              # (B, nsaves, n) complex64 on the device
    W: np.ndarray                 # absolute angular frequencies V + w0 (centred)
    stats: List[dict]
    trace: Optional[torch.Tensor]  # (B, trace_cap, 2) int64: step (length/2^40 units), accepted


@on_stream
def propagate(ops: FibreOperators, A, flength: float, nsaves: int, *, w0: float = 0.0, rtol: float = 1e-5,
              atol: float = 1e-12, device: int = 0, trace_cap: int = 0, max_attempts: int = 0,
              stream=None) -> GnlseRun:
    """Propagate a batch of input fields A (B x n, or n) through one fibre."""
    n = ops.n
    if n not in GNLSE_POINTS:
        raise nat.OptifaxError(f"gnlse: n_points must be one of {GNLSE_POINTS}")
    dev = torch.device(f"cuda:{device}")
    A = torch.as_tensor(np.ascontiguousarray(np.atleast_2d(A), dtype=np.complex64)).to(dev) \
        if not isinstance(A, torch.Tensor) else torch.atleast_2d(A).to(dev, torch.complex64).contiguous()
    if A.dim() != 2 or A.shape[1] != n:
        raise nat.OptifaxError(f"gnlse: input fields must have {n} points (the operators' grid)")
    if nsaves < 2:
        raise nat.OptifaxError("gnlse: nsaves must be at least 2 (z = 0 and z = flength)")
    nb = A.shape[0]
    B_d = torch.from_numpy(np.ascontiguousarray(ops.B)).to(dev)
    W_d = torch.from_numpy(np.ascontiguousarray(ops.W, dtype=np.float32)).to(dev)
    RW_d = None if ops.RW is None else torch.from_numpy(np.ascontiguousarray(ops.RW, dtype=np.complex64)).to(dev)
    AT = torch.empty((nb, nsaves, n), dtype=torch.complex64, device=dev)
    AW = torch.empty((nb, nsaves, n), dtype=torch.complex64, device=dev)
    stats = torch.zeros((nb, 4), dtype=torch.int32, device=dev)
    trace = torch.zeros((nb, max(trace_cap, 1), 2), dtype=torch.int64, device=dev) if trace_cap > 0 else None
    arr = (nat.OptifaxGnlsePulse * nb)()
    for b in range(nb):
        p = arr[b]
        p.n_points, p.n_saves = n, nsaves
        p.A = A[b].data_ptr()
        p.B, p.W = B_d.data_ptr(), W_d.data_ptr()
        p.RW = RW_d.data_ptr() if RW_d is not None else None
        p.gamma, p.fr, p.dT, p.alpha = ops.gamma, ops.fr, ops.dT, ops.alpha
        p.length, p.rtol, p.atol = float(flength), float(rtol), float(atol)
        p.AT_out, p.AW_out = AT[b].data_ptr(), AW[b].data_ptr()
        p.trace = trace[b].data_ptr() if trace is not None else None
        p.trace_cap = trace_cap if trace is not None else 0
        p.max_attempts = int(max_attempts)
        p.stats = stats[b].data_ptr()
    ctx = context(device)
    nat.check(ctx.lib.optifax_gnlse(ctx.handle, arr, nb, _stream_ptr(stream)), ctx.handle, "optifax_gnlse")
    st = stats.cpu().numpy()
    return GnlseRun(Z=np.linspace(0.0, flength, nsaves), AT=AT, AW=AW, W=ops.V + w0,
                    stats=[{"attempts": int(s[0]), "accepted": int(s[1]), "status": int(s[2])} for s in st],
                    trace=trace)


def gnlsefib(T, A, w0, gamma, betas, loss, fr, RT, flength, nsaves, **kw):
    """[Z, AT, AW, W] = gnlsefib(T, A, w0, gamma, betas, loss, fr, RT, flength, nsaves)
    (gnlsefib.m:1-2) for one field; AT and AW are (nsaves, n) device tensors."""
    ops = fibre_operators(T, w0, gamma, betas, loss, fr, RT)
    r = propagate(ops, A, flength, nsaves, w0=w0, **kw)
    return r.Z, r.AT[0], r.AW[0], r.W
