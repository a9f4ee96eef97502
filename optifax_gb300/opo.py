"""Synchronously pumped OPO round trips on the GPU (OpticalSim.run equivalent).

Reference per trip (toolbox/lib/classes/OpticalSim.m:230-288):
  pump add (OpticalPulse.add, OpticalPulse.m:518-527) and refraction into the
  crystal (refract, :190-197); crystal pass (obj.Solver); refraction to air;
  optics before the output coupler (propagate, :137-161); output coupling
  (outputcouple, :163-172, regime "R": intracavity sqrt(R), output sqrt(T));
  delay (applyGD, :256-261).
Every one of those is a per-mode product on the spectrum of the fftshifted
field, so with X the crystal-output spectrum the next crystal input is
    Y = X * feedback + pump,   feedback = r_out sqrt(T_filter) sqrt(R_oc) exp(-i Delay dw) r_in,
                               pump     = r_in FFT(pump field in air),
which the kernel applies at the end of each pass (one launch for all trips).
r_in = sqrt(n_air / n_xtal) per mode and r_out = 1 / r_in.
"""
from __future__ import annotations

import ctypes
import dataclasses
from typing import Optional

import numpy as np
import torch

from . import _native as nat
from . import physics as ph
from .solver import context, _stream_ptr, on_stream

TALLY_OUTPUT, TALLY_OUTPUT_SIGNAL, TALLY_INTRACAVITY, TALLY_PUMP_BAND = range(4)
ESD_OUTPUT, ESD_XTAL_OUT = range(2)


class OptifaxOpo(ctypes.Structure):
    _fields_ = [("pass_", nat.OptifaxPulse), ("feedback", ctypes.c_void_p), ("pump", ctypes.c_void_p),
                ("tally_w", ctypes.c_void_p), ("trips", ctypes.c_void_p),
                ("n_trips", ctypes.c_int32), ("n_tally", ctypes.c_int32),
                ("steady_trips", ctypes.c_int32), ("steady_tally", ctypes.c_int32),
                ("steady_tol", ctypes.c_float), ("reserved", ctypes.c_int32), ("history", ctypes.c_void_p),
                ("esd_w", ctypes.c_void_p), ("esd", ctypes.c_void_p), ("n_esd", ctypes.c_int32),
                ("reserved2", ctypes.c_int32), ("stepmods_trips", ctypes.c_void_p)]


TRIP_RECORD_BYTES = 48


@dataclasses.dataclass
class CavitySpec:
    """A singly resonant SPOPO: crystal, signal-band filter, output coupler, delay."""

    n_points: int = 2 ** 14
    window: float = 12e-12
    crystal_length: float = 5e-3
    period: object = 30e-6
    d_eff: float = 14e-12
    pump_power: float = 2.0
    pump_tau: float = 200e-15
    pump_wavelength: float = 1040e-9
    f_rep: float = 100e6
    waist: float = 15e-6
    oc_output: float = 0.10                  # output-coupler transmission (regime "R")
    signal_band_nm: tuple = (1350.0, 1800.0)  # fed-back band
    filter_edge_nm: float = 10.0
    delay: float = 0.0                       # [s] cavity-length detuning
    error_bounds: tuple = (2.5e-3, 5e-2)
    seed: int = 1
    n_air: float = 1.0
    step_size: float = 1e-7                  # solver step h [m] (NonlinearCrystal.m:12)


@dataclasses.dataclass
class CavityArrays:
    win: ph.SimWindow
    si: ph.SolverInputs
    E0: np.ndarray            # first crystal input (fftshifted time), complex128
    feedback: np.ndarray      # natural FFT order, complex128
    pump: np.ndarray          # natural FFT order, complex128
    tally_w: np.ndarray       # (4, N) float64
    unit: float               # J per |X|^2 in air
    esd_w: np.ndarray = None  # (2, N): pJ/THz per |X|^2 of the output-coupled and crystal-output pulses


def build_cavity(spec: CavitySpec) -> CavityArrays:
    win = ph.SimWindow(spec.pump_wavelength, spec.n_points, spec.window)
    xt = ph.Crystal(spec.crystal_length, spec.period, d_eff=spec.d_eff, step_size=spec.step_size)
    si = ph.solver_inputs(xt, win, error_bounds=spec.error_bounds)
    n_x = si.n_index                                   # natural FFT order
    r_in = np.sqrt(spec.n_air / n_x)
    lam = np.fft.ifftshift(win.wavelengths)
    lam_nm = lam * 1e9
    lo, hi = spec.signal_band_nm
    t_filter = np.where(lam > 0, ph.smoothed_top_hat(lam_nm, lo, hi, spec.filter_edge_nm), 0.0)
    dw = np.fft.ifftshift(win.rel_omegas)
    delay = np.exp(-1j * spec.delay * dw)
    feedback = np.sqrt(t_filter) * np.sqrt(1.0 - spec.oc_output) * delay      # r_out r_in = 1
    pump_t = ph.sech_pump(win, spec.pump_wavelength, spec.pump_tau, spec.pump_power,
                          f_rep=spec.f_rep, waist=spec.waist, n_medium=spec.n_air)
    pump_k = r_in * np.fft.fft(np.fft.fftshift(pump_t))
    noise_t = ph.photon_noise(win, spec.seed, waist=spec.waist, n_medium=spec.n_air,
                              mask=ph.window_transmission(win))
    E0 = np.fft.ifft(r_in * np.fft.fft(np.fft.fftshift(noise_t)) + pump_k)
    n = spec.n_points
    unit = (ph.C0 * spec.n_air * ph.EPS0 / 2.0) * np.pi * spec.waist ** 2 * win.dt / n
    r_out2 = 1.0 / r_in ** 2
    sig = ((lam_nm > lo) & (lam_nm < hi)).astype(np.float64)
    pband = ((lam_nm > 1000.0) & (lam_nm < 1080.0)).astype(np.float64)
    tally_w = np.stack([unit * r_out2 * t_filter * spec.oc_output,
                        unit * r_out2 * t_filter * spec.oc_output * sig,
                        unit * r_out2,
                        unit * r_out2 * pband])
    # energy spectral densities in pJ/THz (OpticalPulse.ESD_pJ_THz: I2pow / dNu * 1e24)
    df = 1.0 / (n * win.dt)
    esd_w = np.stack([tally_w[0], tally_w[2]]) / df * 1e24
    return CavityArrays(win=win, si=si, E0=E0, feedback=feedback, pump=pump_k, tally_w=tally_w, unit=unit,
                        esd_w=esd_w)


@dataclasses.dataclass
class OpoResult:
    field: torch.Tensor          # crystal input of the next trip (fftshifted time), complex64
    trips: np.ndarray            # structured per-trip records
    trips_done: int
    stats: dict
    trips_dev: Optional[torch.Tensor] = None
    stats_dev: Optional[torch.Tensor] = None
    history: Optional[torch.Tensor] = None   # (n_trips, N) crystal-output spectra when requested
    esd: Optional[torch.Tensor] = None       # (2, N) trip sums of the ESDs (pJ/THz), natural FFT order
    step_size_modifiers: Optional[torch.Tensor] = None   # (n_trips, S) per-trip stepmods records

    def decode(self):
        """Copy the device records to the host (after the stream has finished)."""
        from .solver import decode_stats
        st = decode_stats(self.stats_dev)[0]
        done = int(self.stats_dev[0, 9].item())
        rec = np.frombuffer(self.trips_dev.cpu().numpy().tobytes(), dtype=_TRIP_DTYPE)
        return rec[:done].copy(), done, st


_TRIP_DTYPE = np.dtype([("attempts", "<i4"), ("accepted", "<i4"), ("rejected", "<i4"),
                        ("status", "<i4"), ("tally", "<f8", (4,))])


class OpticalSim:
    """Device-resident SPOPO (mirrors OpticalSim(src, cav, simWin, errorBounds, stepSize).run)."""

    def __init__(self, spec: CavitySpec, device: int = 0, variant: int = nat.VARIANT_BATCH_XTAL,
                 cta_points: int = 0):
        self.spec = spec
        self.arrays = build_cavity(spec)
        self.dev = torch.device(f"cuda:{device}")
        a = self.arrays
        si = a.si
        t = lambda x, dt: torch.from_numpy(np.ascontiguousarray(x).astype(dt)).to(self.dev)
        self.alpha = t(si.alpha, np.float32)
        self.beta = t(si.beta, np.float32)
        self.G = t(si.G, np.float32)
        self.feedback = t(a.feedback, np.complex64)
        self.pump = t(a.pump, np.complex64)
        self.tally_w = t(a.tally_w, np.float32)
        self.esd_w = t(a.esd_w, np.float32)
        self.field = t(a.E0, np.complex64)
        self.variant = variant
        self.cta_points = cta_points
        self.ctx = context(device)
        self.trip_number = 0

    def _descriptor(self, n_trips, steady_tol, steady_trips, steady_tally, history, esd=False, steps=False):
        si = self.arrays.si
        N = self.field.numel()
        out = torch.empty_like(self.field)
        trips = torch.zeros((n_trips, TRIP_RECORD_BYTES // 4), dtype=torch.int32, device=self.dev)
        cv = OptifaxOpo()
        d = cv.pass_
        d.n_points, d.n_steps = N, si.n_steps
        d.E_in, d.A_out = self.field.data_ptr(), out.data_ptr()
        d.alpha, d.beta, d.G = self.alpha.data_ptr(), self.beta.data_ptr(), self.G.data_ptr()
        d.w0, d.h, d.bdiffw0, d.dt = si.w0, si.h, si.bdiffw0, si.dt
        d.max_err, d.min_err, d.sel = si.max_err, si.min_err, si.sel
        cv.feedback, cv.pump, cv.tally_w = self.feedback.data_ptr(), self.pump.data_ptr(), self.tally_w.data_ptr()
        cv.trips = trips.data_ptr()
        cv.n_trips, cv.n_tally = int(n_trips), 4
        cv.steady_trips, cv.steady_tally, cv.steady_tol = int(steady_trips), int(steady_tally), float(steady_tol)
        hist = torch.zeros((n_trips, N), dtype=torch.complex64, device=self.dev) if history else None
        cv.history = hist.data_ptr() if hist is not None else None
        esd_acc = torch.zeros((2, N), dtype=torch.float32, device=self.dev) if esd else None
        if esd_acc is not None:
            cv.esd_w, cv.esd, cv.n_esd = self.esd_w.data_ptr(), esd_acc.data_ptr(), 2
        smt = torch.zeros((n_trips, si.n_steps), dtype=torch.float32, device=self.dev) if steps else None
        cv.stepmods_trips = smt.data_ptr() if smt is not None else None
        return cv, out, trips, hist, esd_acc, smt

    def run(self, n_trips: int, *, steady_tol: float = 0.0, steady_trips: int = 0,
            steady_tally: int = TALLY_OUTPUT_SIGNAL, stream=None, host_out: bool = True,
            history: bool = False, esd: bool = False, step_records: bool = False) -> OpoResult:
        """Run n_trips round trips in one launch.  history=True also returns every
        trip's crystal-output spectrum X (n_trips, N) in ``result.history``; esd=True
        the trip sums of the output-coupled and crystal-output ESDs (``result.esd``,
        see ``esd_averages``); step_records=True each trip's stepmods record
        (``result.step_size_modifiers``, OpticalSim.StepSizeModifiers)."""
        return run_many([self], n_trips, steady_tol=steady_tol, steady_trips=steady_trips,
                        steady_tally=steady_tally, stream=stream, host_out=host_out, history=history,
                        esd=esd, step_records=step_records)[0]

    def esd_averages(self, res: OpoResult) -> dict:
        """OpticalSim.averageSimPulses (OpticalSim.m:303-315) from a run's ESD sums:
        the output ESD averaged over the trips, the crystal-output ESD below the pump
        limit (lambda_pump + 5 linewidths, "pump depletion") and above twice that limit
        ("idler"), all in pJ/THz per FFT bin, with the wavelengths (natural FFT order)."""
        if res.esd is None:
            raise ValueError("run with esd=True")
        n = max(res.trips_done, 1)
        e = res.esd.double().cpu().numpy() / n
        lam_nm = np.fft.ifftshift(self.arrays.win.wavelengths) * 1e9
        lw = ph.default_linewidth(self.spec.pump_wavelength, self.spec.pump_tau)
        pump_lim = (self.spec.pump_wavelength + 5 * lw) * 1e9
        xt = e[ESD_XTAL_OUT]
        return {"wavelength_nm": lam_nm, "out": e[ESD_OUTPUT],
                "pump_depletion": np.where(lam_nm > pump_lim, 0.0, xt),
                "idler": np.where(lam_nm < 2 * pump_lim, 0.0, xt)}


@on_stream
def run_many(sims, n_trips: int, *, steady_tol: float = 0.0, steady_trips: int = 0,
             steady_tally: int = TALLY_OUTPUT_SIGNAL, stream=None, host_out: bool = True,
             history: bool = False, esd: bool = False, step_records: bool = False):
    """Run several independent cavities (same device) for n_trips each in one launch."""
    if not sims:
        raise ValueError("no cavities")
    dev = sims[0].dev
    arr = (OptifaxOpo * len(sims))()
    outs = []
    for i, sim in enumerate(sims):
        if sim.dev != dev or sim.variant != sims[0].variant:
            raise ValueError("cavities of one launch share the device and the variant")
        cv, out, trips, hist, esd_acc, smt = sim._descriptor(n_trips, steady_tol, steady_trips, steady_tally,
                                                             history, esd, step_records)
        arr[i] = cv
        outs.append((out, trips, hist, esd_acc, smt))
    stats = torch.zeros((len(sims), nat.STATS_BYTES // 4), dtype=torch.int32, device=dev)
    ctx = sims[0].ctx
    lib = ctx.lib
    lib.optifax_opo_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(OptifaxOpo), ctypes.c_int32,
                                    ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    rc = lib.optifax_opo_run(ctx.handle, arr, len(sims), int(sims[0].variant), int(sims[0].cta_points),
                             stats.data_ptr(), _stream_ptr(stream))
    nat.check(rc, ctx.handle, "optifax_opo_run")
    results = []
    for i, (sim, (out, trips, hist, esd_acc, smt)) in enumerate(zip(sims, outs)):
        sim.field = out
        res = OpoResult(field=out, trips=None, trips_done=-1, stats={}, trips_dev=trips,
                        stats_dev=stats[i:i + 1])
        res.history = hist
        res.esd = esd_acc
        res.step_size_modifiers = smt
        if host_out:
            res.trips, res.trips_done, res.stats = res.decode()
            sim.trip_number += res.trips_done
        results.append(res)
    return results
