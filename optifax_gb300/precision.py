"""Precision study: one long chirped-crystal pass in FP32 (FP64 phase), in
float-float and in full FP64.

The workload is a 2^16-point sech^2 pump (100 fs, 3 W, 1040 nm) through a 20 mm
MgO:PPLN crystal with a linearly chirped grating, period 28 -> 32 um
(chirpedgrating.m with a = 1, tol 0.1 um), 2*10^5 solver steps of 0.1 um.  The
FP32 propagator (optifax_propagate) runs it with its own adaptive schedule and
again replaying the FP64 run's accept/reject decisions; the float-float pass
(optifax_propagate_f32x2) runs it with its own schedule from the FP64 input; the
plain FP64 solver (optifax_propagate_fp64) is the FP64 reference at this size.
Each result reports the relative L2 field error, the relative pulse-energy
error and the power-weighted RMS spectral phase error against the FP64 result.
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np
import torch

from . import physics as ph
from . import solver as sv

DT = 6e-12 / 2 ** 13


@dataclasses.dataclass
class PrecisionCase:
    n_points: int = 2 ** 16
    length: float = 20e-3
    p1: float = 28e-6
    p2: float = 32e-6
    tau: float = 100e-15
    power: float = 3.0
    seed: int = 4


def build(case: PrecisionCase):
    """(window, solver inputs, fftshifted in-crystal field complex128)."""
    win = ph.SimWindow(1040e-9, case.n_points, case.n_points * DT)
    xt = ph.Crystal(case.length, ("chirpedgrating", case.p1, case.p2, 1.0, 0.1e-6))
    si = ph.solver_inputs(xt, win)
    pump = ph.sech_pump(win, 1040e-9, case.tau, case.power)
    noise = ph.photon_noise(win, case.seed, mask=ph.window_transmission(win))
    e = np.fft.fftshift(pump + noise)
    e = np.fft.ifft(np.fft.fft(e) * np.sqrt(1.0 / si.n_index))
    return win, si, e


def metrics(a: np.ndarray, ref: np.ndarray, floor: float = 1e-3) -> dict:
    """Field, energy and spectral-phase error of `a` against `ref` (same layout).

    The spectral phase error is the RMS of the wrapped phase difference per FFT
    bin, weighted by the reference's spectral power over bins holding more than
    `floor` of the peak bin power.
    """
    a = np.asarray(a, dtype=np.complex128)
    ref = np.asarray(ref, dtype=np.complex128)
    fa, fr = np.fft.fft(a), np.fft.fft(ref)
    pw = np.abs(fr) ** 2
    m = pw > floor * pw.max()
    dphi = np.angle(fa[m] * np.conj(fr[m]))
    return {"rel_l2": float(np.linalg.norm(a - ref) / np.linalg.norm(ref)),
            "energy_rel": float(abs(np.sum(np.abs(a) ** 2) - np.sum(np.abs(ref) ** 2)) / np.sum(np.abs(ref) ** 2)),
            "spectral_phase_rms_rad": float(np.sqrt(np.sum(pw[m] * dphi ** 2) / np.sum(pw[m]))),
            "bins": int(m.sum())}


def _fp32_spec(si, e, dev, forced=None, trace_cap=0):
    return sv.PulseSpec(E=torch.from_numpy(e.astype(np.complex64)).to(dev),
                        alpha=torch.from_numpy(si.alpha).to(dev), beta=torch.from_numpy(si.beta).to(dev),
                        G=torch.from_numpy(si.G).to(dev), w0=si.w0, bdiffw0=si.bdiffw0, h=si.h, dt=si.dt,
                        max_err=si.max_err, min_err=si.min_err, sel=si.sel, n_steps=si.n_steps,
                        trace_cap=trace_cap,
                        forced=None if forced is None else torch.from_numpy(forced.astype(np.int32)).to(dev))


def run_fp64(si, e, dev, trace_cap=1 << 22, entry="propagate_fp64"):
    """The FP64 pass (or, with entry="propagate_f32x2", the float-float pass);
    returns (field, stats, trace or None, seconds)."""
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    A, st, tr = getattr(sv, entry)(
        torch.from_numpy(np.ascontiguousarray(e, dtype=np.complex128)).to(dev),
        torch.from_numpy(si.alpha.astype(np.float64)).to(dev), torch.from_numpy(si.beta.astype(np.float64)).to(dev),
        torch.from_numpy(si.G.astype(np.float64)).to(dev), w0=si.w0, bdiffw0=si.bdiffw0, h=si.h, dt=si.dt,
        n_steps=si.n_steps, max_err=si.max_err, min_err=si.min_err, sel=si.sel, trace_cap=trace_cap)
    torch.cuda.synchronize(dev)
    return A.cpu().numpy(), st, tr, time.perf_counter() - t0


def run_fp32(si, e, dev, forced=None, trace_cap=0):
    spec = _fp32_spec(si, e, dev, forced, trace_cap)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    outs, stats = sv.propagate([spec])
    torch.cuda.synchronize(dev)
    el = time.perf_counter() - t0
    return outs[0].cpu().numpy(), sv.decode_stats(stats)[0], spec, el


def study(case: PrecisionCase = PrecisionCase(), device: int = 0) -> dict:
    """Run the three passes and return the report (errors against the FP64 run)."""
    dev = torch.device(f"cuda:{device}")
    win, si, e = build(case)
    a64, st64, tr64, t64 = run_fp64(si, e, dev)
    a32, st32, _, t32 = run_fp32(si, e, dev)
    forced = tr64[:, 2] & 3
    a32r, st32r, _, t32r = run_fp32(si, e, dev, forced=forced)
    # the FP64 pass started from the FP32-rounded input: separates the error of
    # storing the input field in FP32 from the rounding during the pass
    e32 = e.astype(np.complex64).astype(np.complex128)
    a64q, st64q, _, _ = run_fp64(si, e32, dev, trace_cap=0)
    a2, st2, tr2, t2 = run_fp64(si, e, dev, entry="propagate_f32x2")
    same = tr2 is not None and tr2.shape == tr64.shape and bool(np.array_equal(tr2[:, :2], tr64[:, :2]))
    return {"case": dataclasses.asdict(case), "n_steps": si.n_steps,
            "fp64": {"attempts": st64["attempts"], "rejected": st64["rejected"], "seconds": t64,
                     "status": st64["status"]},
            "fp32": {"attempts": st32["attempts"], "rejected": st32["rejected"], "seconds": t32,
                     "status": st32["status"], **metrics(a32, a64)},
            "f32x2": {"attempts": st2["attempts"], "rejected": st2["rejected"], "seconds": t2,
                      "status": st2["status"], "schedule_identical": same, **metrics(a2, a64)},
            "fp32_replayed": {"attempts": st32r["attempts"], "seconds": t32r, "status": st32r["status"],
                              **metrics(a32r, a64)},
            "fp64_from_fp32_input": {"attempts": st64q["attempts"], **metrics(a64q, a64)},
            "fp32_vs_fp64_from_fp32_input": metrics(a32r, a64q),
            "input_energy_ratio_out_in": float(np.sum(np.abs(a64) ** 2) / np.sum(np.abs(e) ** 2))}
