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
import functools
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _native as nat
from ._native import (HEUN, RK23, VARIANT_BATCH_XTAL, VARIANT_BATCH_OP, VARIANT_NO_BC,
                      VARIANT_HARD_BC, VARIANT_ODE23, VARIANT_NEE, Context, check)

_contexts = {}


def context(device: int = 0) -> Context:
    if device not in _contexts:
        _contexts[device] = Context(device)
    return _contexts[device]


def _stream_ptr(stream) -> int:
    if stream is None:
        stream = torch.cuda.current_stream()
    return int(stream.cuda_stream)


def on_stream(fn):
    """Run a wrapper taking ``stream=`` wholly on that stream: input preparation
    (contiguous copies, zeroed records), the library call and any read-back.  The
    given stream first waits for the current stream, where the caller made the
    inputs; temporaries are then allocated on the given stream, so the caching
    allocator cannot hand them out while the call still reads them.  Outputs are
    ready on the given stream (synchronise it before using them elsewhere).
    stream=None, or the current stream, runs the wrapper unchanged."""
    @functools.wraps(fn)
    def wrapper(*args, stream=None, **kw):
        if stream is None or stream == torch.cuda.current_stream(stream.device):
            return fn(*args, stream=stream, **kw)
        stream.wait_stream(torch.cuda.current_stream(stream.device))
        with torch.cuda.stream(stream):
            return fn(*args, stream=stream, **kw)
    return wrapper


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


@on_stream
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
    cta_points: int = 0                        # points per CTA (0: the call's choice / autotuned)


@on_stream
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
        d.cta_points = int(p.cta_points or _tuned_cta_points(N, cta_points))
    stats = None
    if want_stats:
        stats = torch.zeros((len(pulses), nat.STATS_BYTES // 4), dtype=torch.int32, device=pulses[0].E.device)
    rc = ctx.lib.optifax_propagate(ctx.handle, arr, len(pulses), int(method), int(variant),
                                   int(cta_points), stats.data_ptr() if stats is not None else None,
                                   _stream_ptr(stream))
    check(rc, ctx.handle, "optifax_propagate")
    return [p.out for p in pulses], stats


class PropagateGraph:
    """A batch recorded once by optifax_propagate_graph and replayed by launch():
    the specs' tensors (inputs read, outputs and stats rewritten on every replay)
    stay bound to the graph, which keeps references to them."""

    def __init__(self, ctx, handle, outputs, stats, keep, kernels):
        self.ctx, self.handle, self.outputs, self.stats, self._keep = ctx, handle, outputs, stats, keep
        self.kernels = kernels

    def launch(self, stream=None):
        rc = self.ctx.lib.optifax_graph_launch(self.handle, _stream_ptr(stream))
        check(rc, None, "optifax_graph_launch")

    def close(self):
        if self.handle:
            self.ctx.lib.optifax_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


def propagate_graph(pulses: Sequence[PulseSpec], *, method: int = HEUN, variant: int = VARIANT_BATCH_XTAL,
                    cta_points: int = 0) -> PropagateGraph:
    """Record the batch of ``propagate`` once into a CUDA graph (one persistent grid per
    cluster shape) and return it; ``graph.launch(stream)`` replays it."""
    if not pulses:
        raise ValueError("no pulses")
    dev = pulses[0].E.device.index or 0
    ctx = context(dev)
    arr = (nat.OptifaxPulse * len(pulses))()
    keep = []
    for i, p in enumerate(pulses):
        E = _cuda(p.E, torch.complex64)
        if p.out is None:
            p.out = torch.empty_like(E)
        al, be, G = _cuda(p.alpha, torch.float32), _cuda(p.beta, torch.float32), _cuda(p.G, torch.float32)
        keep += [E, al, be, G, p.out]
        d = arr[i]
        d.n_points, d.n_steps = E.numel(), int(p.n_steps)
        d.E_in, d.A_out = E.data_ptr(), p.out.data_ptr()
        d.alpha, d.beta, d.G = al.data_ptr(), be.data_ptr(), G.data_ptr()
        d.w0, d.h = float(p.w0), float(p.h)
        d.bdiffw0, d.dt = float(p.bdiffw0), float(p.dt)
        d.max_err, d.min_err, d.sel = float(p.max_err), float(p.min_err), float(p.sel)
        d.stepmods_limit = 0
        d.cta_points = int(p.cta_points or _tuned_cta_points(E.numel(), cta_points))
    stats = torch.zeros((len(pulses), nat.STATS_BYTES // 4), dtype=torch.int32, device=pulses[0].E.device)
    torch.cuda.synchronize(pulses[0].E.device)
    g = ctypes.c_void_p()
    rc = ctx.lib.optifax_propagate_graph(ctx.handle, arr, len(pulses), int(method), int(variant), int(cta_points),
                                         stats.data_ptr(), ctypes.byref(g))
    check(rc, ctx.handle, "optifax_propagate_graph")
    return PropagateGraph(ctx, g, [p.out for p in pulses], stats, keep, ctx.lib.optifax_graph_kernels(g))


def _propagate_wide(entry, E, alpha, beta, G, *, w0, bdiffw0, h, dt, n_steps, max_err, min_err, sel,
                    variant, trace_cap, stream):
    E = _cuda(E, torch.complex128)
    squeeze = E.dim() == 1
    if squeeze:
        E = E.unsqueeze(0)
    B, N = E.shape
    al, be, G = _cuda(alpha, torch.float64), _cuda(beta, torch.float64), _cuda(G, torch.float64)
    S = int(n_steps)
    if al.numel() != N or be.numel() != N or G.numel() not in (S, S * B):
        raise ValueError("alpha/beta must have N elements and G S or B*S")
    g_per_pulse = int(G.numel() == S * B and B > 1)
    out = torch.empty_like(E)
    lib = nat.load()
    st = nat.OptifaxPulseStats()
    tr = (ctypes.c_int32 * (3 * trace_cap))() if trace_cap > 0 else None
    if stream is None:
        stream = torch.cuda.current_stream(E.device)
    rc = getattr(lib, entry)(N, B, S, E.data_ptr(), out.data_ptr(), al.data_ptr(), be.data_ptr(),
                             G.data_ptr(), g_per_pulse, float(w0), float(bdiffw0), float(h), float(dt),
                             float(max_err), float(min_err), float(sel), int(variant),
                             ctypes.cast(tr, ctypes.c_void_p) if tr is not None else None,
                             int(trace_cap), ctypes.byref(st), int(stream.cuda_stream))
    check(rc, None, entry)
    stats = {f: getattr(st, f) for f, _ in nat.OptifaxPulseStats._fields_ if f != "reserved"}
    trace = None
    if tr is not None:
        n = min(stats["attempts"], trace_cap)
        trace = np.frombuffer(tr, dtype=np.int32).reshape(-1, 3)[:n].copy()
    return (out[0] if squeeze else out), stats, trace


@on_stream
def propagate_fp64(E, alpha, beta, G, *, w0, bdiffw0, h, dt, n_steps, max_err, min_err, sel,
                   variant: int = VARIANT_BATCH_XTAL, trace_cap: int = 0, stream=None):
    """The plain full-FP64 crystal pass (optifax_propagate_fp64).

    E: (B, N) or (N,) complex128 CUDA tensor; alpha, beta: (N,) float64; G: (S,)
    or (B, S) float64.  Returns (A_out complex128 like E, stats dict, trace
    ndarray (attempts, 3) or None).  All pulses share one schedule.
    """
    return _propagate_wide("optifax_propagate_fp64", E, alpha, beta, G, w0=w0, bdiffw0=bdiffw0, h=h, dt=dt,
                           n_steps=n_steps, max_err=max_err, min_err=min_err, sel=sel, variant=variant,
                           trace_cap=trace_cap, stream=stream)


@on_stream
def propagate_f32x2(E, alpha, beta, G, *, w0, bdiffw0, h, dt, n_steps, max_err, min_err, sel,
                    variant: int = VARIANT_BATCH_XTAL, trace_cap: int = 0, stream=None):
    """The float-float crystal pass (optifax_propagate_f32x2): arguments and
    results as propagate_fp64, field and transforms in float-float."""
    return _propagate_wide("optifax_propagate_f32x2", E, alpha, beta, G, w0=w0, bdiffw0=bdiffw0, h=h, dt=dt,
                           n_steps=n_steps, max_err=max_err, min_err=min_err, sel=sel, variant=variant,
                           trace_cap=trace_cap, stream=stream)


# ---------------------------------------------------------------------------
# Autotuner: points per CTA (and so cluster size) per grid size
# ---------------------------------------------------------------------------
_TUNED = {}


def _tuned_cta_points(n_points: int, call_choice: int) -> int:
    if call_choice:
        return 0
    return _TUNED.get(n_points, 0)


def autotune(n_points_list=(4096, 8192, 16384, 32768, 65536), crystal_length=0.1e-3, replicas=None,
             device: int = 0, verbose: bool = False) -> dict:
    """Pick cta_points for each grid size by timing short crystal passes.

    For each N every compiled cta_points in [max(512, N/16), min(4096, N)] is
    timed on `replicas` identical pulses (default: enough to fill the GPU) and
    the fastest per pulse-attempt is kept for later propagate() calls.
    """
    import time
    from . import physics as ph
    dev = torch.device(f"cuda:{device}")
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    out = {}
    for N in n_points_list:
        win = ph.SimWindow(1040e-9, N, N * 6e-12 / 2 ** 13)
        si = ph.solver_inputs(ph.Crystal(crystal_length, 30e-6), win)
        e = np.fft.fftshift(ph.sech_pump(win, 1040e-9, min(200e-15, win.temporal_range / 12), 2.0))
        best = None
        for M in (4096, 2048, 1024, 512):
            if M > N or N // M > 16:
                continue
            reps = replicas or max(1, sms // (N // M))
            mk = lambda: PulseSpec(E=torch.from_numpy(e.astype(np.complex64)).to(dev),
                                   alpha=torch.from_numpy(si.alpha).to(dev), beta=torch.from_numpy(si.beta).to(dev),
                                   G=torch.from_numpy(si.G).to(dev), w0=si.w0, bdiffw0=si.bdiffw0, h=si.h,
                                   dt=si.dt, max_err=si.max_err, min_err=si.min_err, sel=si.sel,
                                   n_steps=si.n_steps, cta_points=M)
            specs = [mk() for _ in range(reps)]
            try:
                propagate(specs)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                _, st = propagate(specs)
                torch.cuda.synchronize()
                el = time.perf_counter() - t0
            except Exception:
                continue
            att = sum(s_["attempts"] for s_ in decode_stats(st))
            per = el / max(att, 1)
            if verbose:
                print(f"autotune N={N} cta_points={M}: {per * 1e6:.3f} us per pulse-attempt")
            if best is None or per < best[1]:
                best = (M, per)
        if best:
            out[N] = best[0]
            _TUNED[N] = best[0]
    return out


def decode_stats(stats: torch.Tensor) -> List[dict]:
    """Decode the (n, 12) int32 stats tensor into optifax_pulse_stats dicts."""
    raw = stats.cpu().numpy()
    out = []
    for row in raw:
        b = row.tobytes()
        s = nat.OptifaxPulseStats.from_buffer_copy(b)
        out.append({f: getattr(s, f) for f, _ in nat.OptifaxPulseStats._fields_ if f != "reserved"})
    return out
