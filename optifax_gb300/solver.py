"""Host-side mirror of OptiFax's crystal-pass solver interface.

``opo_mex_batch`` takes the same 14 arguments and returns the same 3 results
as the reference's ``obj.Solver`` call (toolbox/lib/classes/OpticalSim.m:237-252),
i.e. the MEX gateway OPO_mex_BATCH.cpp:19-141.  Arrays are CUDA tensors
(PyTorch is used for device memory only); the computation is the
optifax C ABI in liboptifax.so.  Memory layouts follow the MATLAB column-
major arrays: an N x B MATLAB array is a (B, N) contiguous tensor here.

``propagate`` is the batched per-pulse entry (optifax_propagate): every pulse
has its own grid size, crystal, tolerances and adaptive step schedule.
"""
from __future__ import annotations

import ctypes
import dataclasses
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _native as nat
from ._native import (HEUN, RK23, VARIANT_BATCH_XTAL, VARIANT_BATCH_OP, VARIANT_NO_BC,
                      VARIANT_HARD_BC, VARIANT_ODE23, Context, check)

_contexts = {}


def context(device: int = 0) -> Context:
    if device not in _contexts:
        _contexts[device] = Context(device)
    return _contexts[device]


def _stream_ptr(stream) -> int:
    if stream is None:
        stream = torch.cuda.current_stream()
    return int(stream.cuda_stream)


def _cuda(t, dtype):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("solver arrays must be CUDA tensors")
    if t.dtype != dtype:
        raise TypeError(f"expected {dtype}, got {t.dtype}")
    return t.contiguous()


def n_chunks(n_steps: int, sel: float, variant: int = VARIANT_BATCH_XTAL) -> int:
    """Chunk count of the reference driver (ceil for BATCH_XTAL/BATCH_OP, :406-410)."""
    f32 = np.float32
    nc = int(f32(n_steps) / f32(sel))
    if variant in (VARIANT_BATCH_XTAL, VARIANT_BATCH_OP) and f32(nc) * f32(sel) < f32(n_steps):
        nc += 1
    return nc


def opo_mex_batch(Et, xT_h, G33, w0, bdiffw0, h, nSteps, dt, hBarg, maxErr, minErr, sel,
                  ApFT, stepMods, *, variant: int = VARIANT_BATCH_XTAL, stream=None):
    """[Et, ApFT, stepMods] = Solver(Et, T_step, G33, w0, bdiffw0, h, nSteps, dt, hB,
    maxErr, minErr, sel, ApFT, stepMods).

    Et: (B, N) complex64; xT_h, hBarg: (N,) float32; G33: (S,) or (B, S) float32;
    ApFT: (B, chunks, N) complex64; stepMods: (S,) float32.  Scalars as in the
    reference (w0, h, maxErr, minErr, sel single; bdiffw0, dt double).
    """
    Et = _cuda(Et, torch.complex64)
    if Et.dim() == 1:
        Et = Et.unsqueeze(0)
    B, N = Et.shape
    dev = Et.device.index or 0
    ctx = context(dev)
    xT_h = _cuda(xT_h, torch.float32)
    hBarg = _cuda(hBarg, torch.float32)
    G33 = _cuda(G33, torch.float32)
    ApFT = _cuda(ApFT, torch.complex64)
    stepMods = _cuda(stepMods, torch.float32)
    if hBarg.numel() != N or xT_h.numel() != N:
        raise ValueError("T_step and hB must have N = size(Et, 1) elements")
    S = int(nSteps)
    chunks = ApFT.numel() // (N * B)
    A_out = torch.empty_like(Et)
    Ap_out = torch.empty_like(ApFT)
    sm_out = torch.empty_like(stepMods)
    rc = ctx.lib.optifax_opo_mex_batch(
        ctx.handle, Et.data_ptr(), xT_h.data_ptr(), G33.data_ptr(),
        float(w0), float(bdiffw0), float(h), S, float(dt), hBarg.data_ptr(),
        float(maxErr), float(minErr), float(sel), ApFT.data_ptr(), stepMods.data_ptr(),
        N, B, chunks, int(variant), A_out.data_ptr(), Ap_out.data_ptr(), sm_out.data_ptr(),
        _stream_ptr(stream))
    check(rc, ctx.handle, "optifax_opo_mex_batch")
    return A_out, Ap_out, sm_out


@dataclasses.dataclass
class PulseSpec:
    """One crystal pass (device tensors).  Mirrors optifax_pulse in include/optifax.h."""

    E: torch.Tensor               # (N,) complex64, fftshifted time
    alpha: torch.Tensor           # (N,) float32
    beta: torch.Tensor            # (N,) float32
    G: torch.Tensor               # (S,) float32
    w0: float
    bdiffw0: float
    h: float
    dt: float
    max_err: float
    min_err: float
    sel: float
    n_steps: int
    out: Optional[torch.Tensor] = None
    Ap: Optional[torch.Tensor] = None          # (chunks, N) complex64
    stepmods: Optional[torch.Tensor] = None    # (S,) float32
    trace_cap: int = 0
    forced: Optional[torch.Tensor] = None      # (n,) int32
    trace: Optional[torch.Tensor] = None       # filled: (trace_cap, 3) int32


def propagate(pulses: Sequence[PulseSpec], *, method: int = HEUN, variant: int = VARIANT_BATCH_XTAL,
              cta_points: int = 0, stream=None, want_stats: bool = True):
    """Run every pulse's crystal pass in one call; returns (outputs, stats array or None)."""
    if not pulses:
        raise ValueError("no pulses")
    dev = pulses[0].E.device.index or 0
    ctx = context(dev)
    arr = (nat.OptifaxPulse * len(pulses))()
    keep = []
    for i, p in enumerate(pulses):
        E = _cuda(p.E, torch.complex64)
        N = E.numel()
        if p.out is None:
            p.out = torch.empty_like(E)
        if p.trace_cap > 0 and p.trace is None:
            p.trace = torch.zeros((p.trace_cap, 3), dtype=torch.int32, device=E.device)
        al = _cuda(p.alpha, torch.float32)
        be = _cuda(p.beta, torch.float32)
        G = _cuda(p.G, torch.float32)
        keep += [E, al, be, G]
        d = arr[i]
        d.n_points = N
        d.n_steps = int(p.n_steps)
        d.E_in = E.data_ptr()
        d.A_out = p.out.data_ptr()
        d.alpha, d.beta, d.G = al.data_ptr(), be.data_ptr(), G.data_ptr()
        d.Ap = p.Ap.data_ptr() if p.Ap is not None else None
        d.stepmods = p.stepmods.data_ptr() if p.stepmods is not None else None
        d.trace = p.trace.data_ptr() if p.trace is not None else None
        d.trace_cap = int(p.trace_cap)
        if p.forced is not None:
            f = _cuda(p.forced, torch.int32)
            keep.append(f)
            d.forced, d.n_forced = f.data_ptr(), f.numel()
        d.w0, d.h = float(p.w0), float(p.h)
        d.bdiffw0, d.dt = float(p.bdiffw0), float(p.dt)
        d.max_err, d.min_err, d.sel = float(p.max_err), float(p.min_err), float(p.sel)
        d.stepmods_limit = 0
    stats = None
    if want_stats:
        stats = torch.zeros((len(pulses), nat.STATS_BYTES // 4), dtype=torch.int32, device=pulses[0].E.device)
    rc = ctx.lib.optifax_propagate(ctx.handle, arr, len(pulses), int(method), int(variant),
                                   int(cta_points), stats.data_ptr() if stats is not None else None,
                                   _stream_ptr(stream))
    check(rc, ctx.handle, "optifax_propagate")
    return [p.out for p in pulses], stats


def decode_stats(stats: torch.Tensor) -> List[dict]:
    """Decode the (n, 12) int32 stats tensor into optifax_pulse_stats dicts."""
    raw = stats.cpu().numpy()
    out = []
    for row in raw:
        b = row.tobytes()
        s = nat.OptifaxPulseStats.from_buffer_copy(b)
        out.append({f: getattr(s, f) for f, _ in nat.OptifaxPulseStats._fields_ if f != "reserved"})
    return out
