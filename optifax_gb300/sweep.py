"""Batched crystal-pass sweeps with uneven grids and crystals: 256 instances, N 2^12..2^16, 0.5-10 mm crystals.

Every instance has its own grid size, crystal length, poling period, pump
power and pulse width, and its own adaptive step schedule; all run in one
optifax_propagate call (one grid per cluster shape, launched concurrently).
The reference cannot batch these (one cuFFT plan and one shared step per MEX
call, OPO_CUDA_BATCH_XTAL.cu:418-419,450-466), so it would run them one by one.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
from typing import List

import numpy as np
import torch

from . import _native as nat
from . import physics as ph
from . import solver as sv

DT = 6e-12 / 2 ** 13            # fixed sample spacing: window = N dt


@dataclasses.dataclass
class Instance:
    n_points: int
    length: float
    period: float
    power: float
    tau: float
    seed: int


def uneven_sweep_instances(n: int = 256, seed: int = 2, n_range=(12, 16), length_range=(0.5e-3, 10e-3),
                      period_range=(28e-6, 32e-6), power_range=(0.5, 3.0), tau_range=(100e-15, 300e-15)):
    """Instances drawn with a seeded generator: N uniform over 2^12..2^16 and the
    other parameters uniform over their ranges."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        out.append(Instance(n_points=int(2 ** rng.integers(n_range[0], n_range[1] + 1)),
                            length=float(rng.uniform(*length_range)),
                            period=float(rng.uniform(*period_range)),
                            power=float(rng.uniform(*power_range)),
                            tau=float(rng.uniform(*tau_range)),
                            seed=seed * 100000 + i))
    return out


def build_inputs(inst: Instance):
    """Solver inputs and the in-crystal field (fftshifted, complex128) of one instance."""
    win = ph.SimWindow(1040e-9, inst.n_points, inst.n_points * DT)
    si = ph.solver_inputs(ph.Crystal(inst.length, inst.period), win)
    pump = ph.sech_pump(win, 1040e-9, inst.tau, inst.power)
    noise = ph.photon_noise(win, inst.seed, mask=ph.window_transmission(win))
    e = np.fft.fftshift(pump + noise)
    e = np.fft.ifft(np.fft.fft(e) * np.sqrt(1.0 / si.n_index))
    return win, si, e


def to_specs(inputs, device: int = 0, trace_cap: int = 0) -> List[sv.PulseSpec]:
    dev = torch.device(f"cuda:{device}")
    specs = []
    for win, si, e in inputs:
        specs.append(sv.PulseSpec(
            E=torch.from_numpy(e.astype(np.complex64)).to(dev),
            alpha=torch.from_numpy(si.alpha).to(dev), beta=torch.from_numpy(si.beta).to(dev),
            G=torch.from_numpy(si.G).to(dev), w0=si.w0, bdiffw0=si.bdiffw0, h=si.h, dt=si.dt,
            max_err=si.max_err, min_err=si.min_err, sel=si.sel, n_steps=si.n_steps, trace_cap=trace_cap))
    return specs


def build_specs_device(insts: List[Instance], device: int = 0, trace_cap: int = 0, stream=None) -> List[sv.PulseSpec]:
    """The instances' solver inputs computed on the device in one optifax_setup_pulses
    call (the same quantities as build_inputs + to_specs; only scalars and domain
    walls come from the host)."""
    dev = torch.device(f"cuda:{device}")
    lib = nat.load()
    arr = (nat.OptifaxSetup * len(insts))()
    specs, keep = [], []
    max_n = max(i.n_points for i in insts)
    work = torch.empty(int(lib.optifax_setup_work_bytes(max_n)), dtype=torch.uint8, device=dev)
    for i, inst in enumerate(insts):
        win = ph.SimWindow(1040e-9, inst.n_points, inst.n_points * DT)
        xt = ph.Crystal(inst.length, inst.period)
        sc = ph.solver_scalars(xt, win)
        S = xt.n_steps
        walls = torch.from_numpy(np.ascontiguousarray(
            ph.qpm_walls(np.linspace(0.0, xt.length, S), xt.length, xt.period), dtype=np.float64)).to(dev)
        N = inst.n_points
        alpha = torch.empty(N, dtype=torch.float32, device=dev)
        beta = torch.empty(N, dtype=torch.float32, device=dev)
        G = torch.empty(S, dtype=torch.float32, device=dev)
        E = torch.empty(N, dtype=torch.complex64, device=dev)
        keep.append(walls)
        d = arr[i]
        d.n_points, d.n_steps = N, S
        d.window, d.dt, d.lambda_ref = win.temporal_range, win.dt, win.reference_wave
        d.length, d.step_size, d.celsius = xt.length, xt.step_size, xt.celsius
        d.g_scale = sc["g_scale"]
        d.walls, d.n_walls = walls.data_ptr() if walls.numel() else None, walls.numel()
        d.seed = int(inst.seed)
        d.pump_lambda, d.pump_t_rms = 1040e-9, ph.sech_t_rms(1040e-9, inst.tau)
        d.pump_energy, d.waist, d.n_medium = inst.power / 100e6, 15e-6, 1.0
        d.lambda_lo_nm, d.lambda_hi_nm = win.spectral_limits_nm
        d.alpha, d.beta, d.G, d.E = alpha.data_ptr(), beta.data_ptr(), G.data_ptr(), E.data_ptr()
        f32 = lambda v: float(np.float32(v))
        specs.append(sv.PulseSpec(E=E, alpha=alpha, beta=beta, G=G, w0=sc["w0"], bdiffw0=sc["bdiffw0"],
                                  h=f32(xt.step_size), dt=win.dt, max_err=f32(5e-2), min_err=f32(2.5e-3),
                                  sel=float(math.ceil(S / 4)), n_steps=S, trace_cap=trace_cap))
    s_ = int((stream or torch.cuda.current_stream(dev)).cuda_stream)
    nat.check(lib.optifax_setup_pulses(arr, len(insts), work.data_ptr(), work.numel(), s_), None,
              "optifax_setup_pulses")
    torch.cuda.synchronize(dev)
    return specs
