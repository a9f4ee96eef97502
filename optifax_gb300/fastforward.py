"""Surrogate fast-forward of synchronously pumped OPO round trips.

A trained FNO (optifax_gb300.surrogate) replaces the crystal pass for most
round trips; the solver checks it every ``check_every`` trips, takes over
whenever the check fails, and finishes every run (with its own steady-state
test).  No reference counterpart: the reference runs every trip through its
solver (OpticalSim.m:230-288).

Frequency crop (``Crop``): n_bins consecutive bins of the 2^14-point spectrum
starting at F_LO = 140 THz (the signal band 166-222 THz and the 288 THz pump fit
inside); bins below F_SPLIT = 250 THz are the signal band, the rest the pump
band.  Everything outside the crop is dropped: the cavity feeds back only the
signal band and the pump is injected fresh every trip.

Interaction picture: the network predicts the crystal output divided by the
crystal's linear propagation D_k = alpha_k^S exp(-i beta_k S) (known exactly),
so it learns only the nonlinear change, not the large dispersion phase.

Training pairs come from the solver itself: cavities of the 2^14-point, 5 mm
SPOPO geometry with pump power and width drawn from the sweep ranges (0.5-3 W,
100-300 fs, seeded), each run for n_trips round trips in one launch with the
per-trip crystal-output spectra recorded; pair t is (crystal input Y_t, crystal
output X_t) with Y_0 = FFT(E_0) and Y_{t+1} = X_t feedback + pump.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
import time
from typing import List, Optional

import numpy as np
import torch

from . import _native as nat
from . import opo
from .surrogate import FNO, COUT, CIN

F_LO = 140e12
F_SPLIT = 250e12
N_BINS = 4096


@dataclasses.dataclass
class Crop:
    n_points: int
    k0: int
    n_bins: int
    split: int
    pump_scale: float


def make_crop(win, pump_scale: float, n_bins: int = N_BINS, f_lo: float = F_LO, f_split: float = F_SPLIT) -> Crop:
    n = win.n_points
    df = 1.0 / (n * win.dt)
    f0 = win.f0
    k_lo = int(round((f_lo - f0) / df))
    split = int(math.ceil((f_split - (f0 + k_lo * df)) / df))
    if not (0 < split < n_bins <= n):
        raise ValueError("crop does not hold both bands")
    return Crop(n, k_lo % n, n_bins, split, float(pump_scale))


def reference_crop(spec: Optional[opo.CavitySpec] = None) -> Crop:
    """Crop with the pump scale of the 2 W, 200 fs pump of the given geometry."""
    spec = spec or opo.CavitySpec()
    ref = dataclasses.replace(spec, pump_power=2.0, pump_tau=200e-15)
    a = opo.build_cavity(ref)
    return make_crop(a.win, float(np.max(np.abs(a.pump))))


@dataclasses.dataclass
class EnvCrop:
    """Envelope representation: each band demodulated to its carrier and sampled
    n_bins times over the window (time-domain channels).  band = (kc_pump, lo_pump,
    hi_pump, kc_signal, lo_signal, hi_signal): carrier bins (natural FFT order) and
    the signed bin-offset range of each band."""

    n_points: int
    n_bins: int
    band: tuple
    pump_scale: float


def envelope(spectrum: np.ndarray, kc: int, lo: int, hi: int, n_bins: int) -> np.ndarray:
    """e_j = sum_{o in [lo, hi)} X[(kc + o) mod N] exp(2 pi i o j / n_bins) (host, FP64)."""
    n = spectrum.shape[-1]
    b = np.zeros(n_bins, dtype=np.complex128)
    o = np.arange(lo, hi)
    b[o % n_bins] = spectrum[(kc + o) % n]
    return n_bins * np.fft.ifft(b)


def make_env_crop(win, pump_k: np.ndarray, n_bins: int = N_BINS, f_lo: float = F_LO, f_split: float = F_SPLIT,
                  signal_band_nm=(1350.0, 1800.0), pump_wavelength: Optional[float] = None) -> EnvCrop:
    n = win.n_points
    df = 1.0 / (n * win.dt)
    f0 = win.f0
    rel = lambda f: (f - f0) / df
    split_rel = int(math.ceil(rel(f_split)))
    lo_rel = int(math.ceil(rel(f_lo)))
    kc_p = int(round(rel(opo.ph.C0 / (pump_wavelength or win.reference_wave))))
    f_s = 0.5 * (opo.ph.C0 / (signal_band_nm[1] * 1e-9) + opo.ph.C0 / (signal_band_nm[0] * 1e-9))
    kc_s = int(round(rel(f_s)))
    lo_p, hi_p = split_rel - kc_p, n_bins // 2
    lo_s, hi_s = lo_rel - kc_s, split_rel - kc_s
    if not (-n_bins // 2 <= lo_p < hi_p <= n_bins // 2 and -n_bins // 2 <= lo_s < hi_s <= n_bins // 2):
        raise ValueError("bands do not fit the envelope grid")
    band = (kc_p % n, lo_p, hi_p, kc_s % n, lo_s, hi_s)
    scale = float(np.max(np.abs(envelope(np.asarray(pump_k), band[0], lo_p, hi_p, n_bins))))
    return EnvCrop(n, n_bins, band, scale)


def reference_env_crop(spec: Optional[opo.CavitySpec] = None) -> EnvCrop:
    spec = spec or opo.CavitySpec()
    ref = dataclasses.replace(spec, pump_power=2.0, pump_tau=200e-15)
    a = opo.build_cavity(ref)
    return make_env_crop(a.win, a.pump, signal_band_nm=spec.signal_band_nm, pump_wavelength=spec.pump_wavelength)


def _band(crop: EnvCrop):
    return (ctypes.c_int32 * 6)(*[int(v) for v in crop.band])


def _ptr(t):
    return t.data_ptr() if t is not None else None


def _stream(dev):
    return int(torch.cuda.current_stream(dev).cuda_stream)


def encode(spectra: torch.Tensor, crop, sigma_in: Optional[torch.Tensor] = None, n_channels: int = CIN):
    """(P, N) complex64 spectra -> (x (P, n_channels, n_bins) float32, sigma (P,))."""
    spectra = spectra.contiguous()
    P = spectra.shape[0]
    dev = spectra.device
    x = torch.empty((P, n_channels, crop.n_bins), dtype=torch.float32, device=dev)
    sig = sigma_in.contiguous() if sigma_in is not None else torch.empty(P, dtype=torch.float32, device=dev)
    if isinstance(crop, EnvCrop):
        rc = nat.load().optifax_ff_encode_env(spectra.data_ptr(), spectra.stride(0), P, crop.n_points, crop.n_bins,
                                              _band(crop), crop.pump_scale, _ptr(sigma_in), x.data_ptr(), n_channels,
                                              None if sigma_in is not None else sig.data_ptr(), _stream(dev))
        nat.check(rc, None, "optifax_ff_encode_env")
        return x, sig
    rc = nat.load().optifax_ff_encode(spectra.data_ptr(), spectra.stride(0), P, crop.n_points, crop.k0,
                                      crop.n_bins, crop.split, crop.pump_scale,
                                      _ptr(sigma_in), x.data_ptr(), n_channels,
                                      None if sigma_in is not None else sig.data_ptr(), _stream(dev))
    nat.check(rc, None, "optifax_ff_encode")
    return x, sig


def decode_env(crop: EnvCrop, y: torch.Tensor, sigma: torch.Tensor, X_out: Optional[torch.Tensor] = None):
    """One network output (1, 4, n_bins) -> the two bands of an N-point spectrum."""
    if X_out is None:
        X_out = torch.empty(crop.n_points, dtype=torch.complex64, device=y.device)
    rc = nat.load().optifax_ff_decode_env(y.contiguous().data_ptr(), sigma.data_ptr(), crop.n_points, crop.n_bins,
                                          _band(crop), crop.pump_scale, X_out.data_ptr(), _stream(y.device))
    nat.check(rc, None, "optifax_ff_decode_env")
    return X_out


def step(crop, feedback, pump, tally_w, *, y=None, sigma=None, lin=None, X_in=None, X_out=None,
         Y_next=None, energy=None):
    """X from the network output y (decoded with sigma) or X_in, times lin; returns
    Y_next = X fb + pump (and fills energy = sum tally_w |X|^2 when given)."""
    dev = feedback.device
    if Y_next is None:
        Y_next = torch.empty(crop.n_points, dtype=torch.complex64, device=dev)
    if isinstance(crop, EnvCrop):
        if y is not None:
            X_in = decode_env(crop, y, sigma)
            y = sigma = None
        k0, nb, split = 0, crop.n_bins, 0
    else:
        k0, nb, split = crop.k0, crop.n_bins, crop.split
    rc = nat.load().optifax_ff_step(_ptr(y), _ptr(sigma), _ptr(X_in), feedback.data_ptr(), pump.data_ptr(),
                                    _ptr(lin), _ptr(tally_w), crop.n_points, k0, nb, split,
                                    crop.pump_scale, _ptr(X_out), Y_next.data_ptr(), _ptr(energy), _stream(dev))
    nat.check(rc, None, "optifax_ff_step")
    return Y_next


def linear_factor(sim: opo.OpticalSim) -> torch.Tensor:
    """The crystal's linear propagation per bin, D_k = alpha_k^S exp(-i beta_k S) (the
    dispersion sub-steps of a whole pass, natural FFT order)."""
    si = sim.arrays.si
    S = si.n_steps
    a = np.asarray(si.alpha, dtype=np.float64) ** S
    D = a * np.exp(-1j * np.asarray(si.beta, dtype=np.float64) * S)
    return torch.from_numpy(D.astype(np.complex64)).to(sim.dev)


def to_interaction(X: torch.Tensor, D: torch.Tensor) -> torch.Tensor:
    """X / D where |D| > 0, else 0."""
    m = D.abs() > 0
    den = torch.where(m, D.abs() ** 2, torch.ones_like(D.real))
    return torch.where(m, X * torch.conj(D) / den, torch.zeros_like(X))


# --------------------------------------------------------------------------
# Training data from the solver
# --------------------------------------------------------------------------
def training_specs(n: int, seed: int = 3, power=(0.5, 3.0), tau=(100e-15, 300e-15),
                   base: Optional[opo.CavitySpec] = None) -> List[opo.CavitySpec]:
    rng = np.random.default_rng(seed)
    base = base or opo.CavitySpec()
    return [dataclasses.replace(base, pump_power=float(rng.uniform(*power)), pump_tau=float(rng.uniform(*tau)),
                                seed=seed * 100000 + i) for i in range(n)]


def generate_raw(specs: List[opo.CavitySpec], n_trips: int, device: int = 0, group: int = 38):
    """Run the cavities (group at a time, one launch per group) and return the raw
    pairs: crystal-input spectra (P, N), interaction-picture crystal-output spectra
    (P, N), the trip index of every pair and the solver attempt count."""
    dev = torch.device(f"cuda:{device}")
    ins_all, outs_all, trip_idx = [], [], []
    attempts = 0
    for g0 in range(0, len(specs), group):
        sims = [opo.OpticalSim(s, device=device) for s in specs[g0:g0 + group]]
        Y0 = [torch.from_numpy(np.fft.fft(s.arrays.E0).astype(np.complex64)).to(dev) for s in sims]
        res = opo.run_many(sims, n_trips, history=True)
        for sim, r, y0 in zip(sims, res, Y0):
            attempts += int(np.sum(r.trips["attempts"]))
            hist = r.history[:r.trips_done]
            ins = torch.empty_like(hist)
            ins[0] = y0
            if hist.shape[0] > 1:
                ins[1:] = hist[:-1] * sim.feedback + sim.pump
            ins_all.append(ins)
            outs_all.append(to_interaction(hist, linear_factor(sim)))
            trip_idx.append(torch.arange(hist.shape[0]))
        del sims, res
    return torch.cat(ins_all), torch.cat(outs_all), torch.cat(trip_idx), attempts


def _host(x, dtype) -> np.ndarray:
    """A tensor (any device) or array as a host NumPy array of dtype."""
    if isinstance(x, torch.Tensor):
        x = x.detach().cpu().numpy()
    return np.asarray(x).astype(dtype, copy=False)


def phase_aligned_err(pred, true, mask) -> float:
    """min over a global phase phi of |pred e^{i phi} - true| / |true| on the masked bins.

    The resonated signal of a singly resonant OPO has no reference phase (the idler
    is not fed back, so the equations are invariant under a common rotation of the
    signal), so two fields that differ only by a global signal phase describe the
    same cavity state; the optimal phi is arg(sum conj(pred) true).  Computed on the
    host in FP64 (one spectrum each way per call), so a check adds no device kernels
    to the loop that calls it."""
    m = _host(mask, bool)
    a, b = _host(pred, np.complex128)[m], _host(true, np.complex128)[m]
    v = np.vdot(a, b)
    ph = v / abs(v) if abs(v) > 0 else 1.0
    return float(np.linalg.norm(a * ph - b) / max(np.linalg.norm(b), 1e-300))


def signal_mask(crop, n_points: int, device) -> torch.Tensor:
    """Bins of the signal channels of an envelope crop (natural FFT order)."""
    kc_s, lo_s, hi_s = crop.band[3], crop.band[4], crop.band[5]
    m = torch.zeros(n_points, dtype=torch.bool, device=device)
    m[(kc_s + torch.arange(lo_s, hi_s, device=device)) % n_points] = True
    return m


def align_signal_phase(ins: torch.Tensor, outs: torch.Tensor, mask: torch.Tensor) -> torch.Tensor:
    """Targets with the trip's global signal-phase change removed: each output's
    signal bins rotated so that their projection on the input's signal bins is real
    and positive (pump bins untouched).  The network then learns the map up to the
    signal's free phase, which is what the phase-aligned check compares."""
    v = torch.sum(torch.conj(ins[:, mask]).to(torch.complex128) * outs[:, mask].to(torch.complex128), dim=1)
    ph = torch.where(v.abs() > 0, torch.conj(v) / v.abs().clamp_min(1e-300), torch.ones_like(v))
    out = outs.clone()
    out[:, mask] = (outs[:, mask].to(torch.complex128) * ph[:, None]).to(outs.dtype)
    return out


def encode_pairs(ins: torch.Tensor, outs: torch.Tensor, crop, chunk: int = 1024):
    """Network inputs (P, 6, L) and targets (P, 4, L) of raw pairs (targets scaled
    with the input's sigma)."""
    xs, ts = [], []
    for i in range(0, ins.shape[0], chunk):
        x, sig = encode(ins[i:i + chunk], crop)
        t, _ = encode(outs[i:i + chunk], crop, sigma_in=sig, n_channels=COUT)
        xs.append(x)
        ts.append(t)
    return torch.cat(xs), torch.cat(ts)


def signal_rel_err(y: torch.Tensor, t: torch.Tensor) -> torch.Tensor:
    """Per-sample relative L2 error of the signal channels (2, 3)."""
    d = (y[:, 2:4] - t[:, 2:4]).flatten(1).norm(dim=1)
    return d / t[:, 2:4].flatten(1).norm(dim=1).clamp_min(1e-30)


def sample_weights(T: torch.Tensor) -> torch.Tensor:
    """Per-sample loss weights 1 / mean(target^2): every pair counts by its relative
    error, so the large normalised gains of the build-up trips do not swamp the rest."""
    return 1.0 / T.pow(2).mean(dim=(1, 2)).clamp_min(1e-12)


def evaluate(net: FNO, X: torch.Tensor, T: torch.Tensor, batch: Optional[int] = None) -> torch.Tensor:
    batch = batch or net.max_batch
    errs = []
    for i in range(0, X.shape[0], batch):
        y = net.forward(X[i:i + batch].contiguous())
        errs.append(signal_rel_err(y, T[i:i + batch]))
    return torch.cat(errs)


def train(net: FNO, X: torch.Tensor, T: torch.Tensor, *, epochs: int = 40, batch: int = 32, lr: float = 1e-3,
          val_frac: float = 0.05, seed: int = 3, weight_decay: float = 0.0, trip_idx=None, log=None) -> dict:
    """AdamW with cosine-decayed learning rate on shuffled minibatches, relative
    (per-sample weighted) squared error; returns the history.  Data parallel over the
    ranks of an initialised process group: every rank draws the same minibatch order
    (one seed), trains on its slice of each global minibatch (batch / world samples)
    and applies the gradients averaged over the ranks (surrogate.data_parallel_step),
    so the replicas stay identical; X and T are the full pair set on every rank."""
    from .surrogate import data_parallel_step
    world = (torch.distributed.get_world_size()
             if torch.distributed.is_available() and torch.distributed.is_initialized() else 1)
    rank = torch.distributed.get_rank() if world > 1 else 0
    if batch % world:
        raise ValueError("the global batch must be a multiple of the number of ranks")
    local = batch // world
    P = X.shape[0]
    g = torch.Generator().manual_seed(seed)
    perm = torch.randperm(P, generator=g)
    n_val = max(1, int(P * val_frac))
    val, tr = perm[:n_val], perm[n_val:]
    Wt = sample_weights(T)
    steps_per_epoch = max(1, len(tr) // batch)
    total = epochs * steps_per_epoch
    hist = {"train_loss": [], "val_signal_rel_l2": [], "epochs": epochs, "pairs": P, "val_pairs": n_val}
    step_i = 0
    t0 = time.perf_counter()
    vdev = val.to(X.device)
    for ep in range(epochs):
        order = tr[torch.randperm(len(tr), generator=g)]
        acc = torch.zeros(1, device=net.dev)
        for s_ in range(steps_per_epoch):
            idx = order[s_ * batch:(s_ + 1) * batch][rank * local:(rank + 1) * local].to(net.dev)
            cur = lr * 0.5 * (1.0 + math.cos(math.pi * step_i / total))
            acc += data_parallel_step(net, X.index_select(0, idx), T.index_select(0, idx), cur,
                                      sample_w=Wt.index_select(0, idx), weight_decay=weight_decay)
            step_i += 1
        hist["train_loss"].append(float(acc.item()) / steps_per_epoch)
        ve = evaluate(net, X[vdev], T[vdev])
        hist["val_signal_rel_l2"].append(float(ve.median()))
        if log:
            log(f"epoch {ep}: train {hist['train_loss'][-1]:.4e} val signal rel-L2 median "
                f"{hist['val_signal_rel_l2'][-1]:.4e}")
    if net.dev.type == "cuda":
        torch.cuda.synchronize(net.dev)
    hist["seconds"] = time.perf_counter() - t0
    hist["steps"] = step_i
    ve = evaluate(net, X[vdev], T[vdev]).cpu()
    hist["val_signal_rel_l2_quantiles"] = [float(v) for v in torch.quantile(ve, torch.tensor([0.1, 0.5, 0.9]))]
    # the same error for the identity map (output = input in the interaction picture)
    ident = signal_rel_err(X[vdev][:, :COUT], T[vdev]).cpu()
    hist["val_identity_rel_l2_median"] = float(ident.median())
    if trip_idx is not None:
        ti = trip_idx[val]
        bins = [(0, 20), (20, 60), (60, 10 ** 9)]
        hist["val_by_trip"] = {f"{a}-{b}": float(ve[(ti >= a) & (ti < b)].median())
                               for a, b in bins if bool(((ti >= a) & (ti < b)).any())}
        hist["val_identity_by_trip"] = {f"{a}-{b}": float(ident[(ti >= a) & (ti < b)].median())
                                        for a, b in bins if bool(((ti >= a) & (ti < b)).any())}
    return hist


# --------------------------------------------------------------------------
# The fast-forward OPO run
# --------------------------------------------------------------------------
def _to_time(Y: torch.Tensor) -> torch.Tensor:
    """Crystal input field (fftshifted time) from its spectrum: the solver's E_in
    (host FFT, once per hand-over to the solver)."""
    e = np.fft.ifft(Y.cpu().numpy().astype(np.complex128))
    return torch.from_numpy(e.astype(np.complex64)).to(Y.device)


def _to_spec(E: torch.Tensor) -> torch.Tensor:
    return torch.from_numpy(np.fft.fft(E.cpu().numpy().astype(np.complex128)).astype(np.complex64)).to(E.device)


def run_fast_forward(sim: opo.OpticalSim, net: Optional[FNO], crop, *, max_trips: int = 1000,
                     check_every: int = 10, check_tol: float = 0.05, finish_trips: int = 50,
                     flat_tol: float = 1e-3, steady_tol: float = 1e-4, steady_trips: int = 10,
                     phase_check: bool = True, check: str = "field") -> dict:
    """max_trips round trips from sim's current state.

    Blocks of check_every trips: the first trip of a block is the check (the
    network's prediction and a solver pass from the same input; the cavity
    continues from the solver's result); when the relative L2 difference over the
    fed-back band (after the best global signal phase, phase_aligned_err, unless
    phase_check=False) is within check_tol the other trips of the block run on the
    network, otherwise on the solver.  check="energy" compares the fed-back band's
    energy instead (relative error of sum |X|^2 over the band); both errors are
    recorded for every check either way.  The last finish_trips trips (and everything
    after the network's trips level out to flat_tol) run on the solver, which
    stops early once its steady-state test passes.  net=None runs the solver only.
    """
    dev = sim.dev
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    tw_sig = sim.tally_w[opo.TALLY_OUTPUT_SIGNAL]
    fbm = np.abs(sim.feedback.cpu().numpy()) > 0          # fed-back band (host mask)
    D = linear_factor(sim)
    energy = torch.zeros(1, dtype=torch.float64, device=dev)
    trips = sur_trips = sol_trips = 0
    checks, energies = [], []
    check_field, check_energy = [], []
    fallback_blocks = 0
    Y = _to_spec(sim.field) if net is not None else None
    surrogate_until = max_trips - finish_trips if net is not None else 0
    while trips < surrogate_until:
        # check trip
        x, sig = encode(Y.unsqueeze(0), crop)
        y = net.forward(x)
        Xs = torch.empty(crop.n_points, dtype=torch.complex64, device=dev)
        step(crop, sim.feedback, sim.pump, None, y=y, sigma=sig, lin=D, X_out=Xs)
        sim.field = _to_time(Y)
        r = sim.run(1, history=True)
        Xt = r.history[0]
        Y = step(crop, sim.feedback, sim.pump, tw_sig, X_in=Xt, energy=energy)
        energies.append(float(energy.item()))
        trips += 1
        sol_trips += 1
        xs, xt = _host(Xs, np.complex128)[fbm], _host(Xt, np.complex128)[fbm]
        ferr = phase_aligned_err(xs, xt, np.ones(xs.shape, bool)) if phase_check else \
            float(np.linalg.norm(xs - xt) / max(np.linalg.norm(xt), 1e-30))
        et = float(np.sum(np.abs(xt) ** 2))
        eerr = abs(float(np.sum(np.abs(xs) ** 2)) - et) / max(et, 1e-300)
        err = eerr if check == "energy" else ferr
        checks.append(err)
        check_field.append(ferr)
        check_energy.append(eerr)
        n = min(check_every - 1, surrogate_until - trips)
        if n <= 0:
            break
        if err <= check_tol:                         # NaN fails too
            for _ in range(n):
                x, sig = encode(Y.unsqueeze(0), crop)
                y = net.forward(x)
                Y = step(crop, sim.feedback, sim.pump, tw_sig, y=y, sigma=sig, lin=D, energy=energy)
                energies.append(float(energy.item()))
                trips += 1
                sur_trips += 1
            if not all(math.isfinite(e) for e in energies[-n:]):
                break
        else:
            sim.field = _to_time(Y)
            r = sim.run(n)
            trips += r.trips_done
            sol_trips += r.trips_done
            energies += [float(v) for v in r.trips["tally"][:, opo.TALLY_OUTPUT_SIGNAL]]
            Y = _to_spec(sim.field)
            fallback_blocks += 1
        if len(energies) > steady_trips:
            e = np.array(energies[-(steady_trips + 1):])
            if np.all(np.abs(np.diff(e)) <= flat_tol * np.abs(e[1:])):
                break
    finish = 0
    if trips < max_trips:
        if Y is not None:
            sim.field = _to_time(Y)
        r = sim.run(max_trips - trips, steady_tol=steady_tol, steady_trips=steady_trips)
        finish = r.trips_done
        trips += finish
        sol_trips += finish
        energies += [float(v) for v in r.trips["tally"][:, opo.TALLY_OUTPUT_SIGNAL]]
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t0
    flat = len(energies) > steady_trips and bool(np.all(
        np.abs(np.diff(energies[-(steady_trips + 1):])) <= steady_tol * np.abs(energies[-steady_trips:])))
    return {"trips": trips, "surrogate_trips": sur_trips, "solver_trips": sol_trips, "finish_trips": finish,
            "checks": checks, "check_field_err": check_field, "check_energy_err": check_energy,
            "check": check, "fallback_blocks": fallback_blocks, "wall_s": wall,
            "trips_per_s": trips / wall if wall > 0 else float("nan"),
            "final_output_signal_energy": energies[-1] if energies else float("nan"),
            "reached_steady_state": flat, "energies": energies, "field": sim.field}


def fp64_plain_trips(spec: opo.CavitySpec, n_trips: int = 2, device: int = 0, E0=None, trace_cap: int = 0,
                     entry: str = "propagate_fp64") -> dict:
    """Round trips through the plain FP64 solver (optifax_propagate_fp64; with
    entry="propagate_f32x2" the float-float pass) with the cavity transfer in FP64 on
    the host.  Timed with CUDA events on the launching stream around all n_trips
    trips (the host transfer between passes included).  Returns seconds per trip,
    the next crystal input, the first pass's crystal output (time domain,
    complex128) and, with trace_cap > 0, its step trace."""
    from . import solver as sv
    a = opo.build_cavity(spec)
    si = a.si
    dev = torch.device(f"cuda:{device}")
    t64 = lambda v: torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64)).to(dev)
    al, be, G = t64(si.alpha), t64(si.beta), t64(si.G)
    E = np.asarray(a.E0 if E0 is None else E0, dtype=np.complex128)
    attempts = 0
    first_A = first_trace = None
    stream = torch.cuda.current_stream(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    ev0.record(stream)
    for i in range(n_trips):
        A, st, tr = getattr(sv, entry)(torch.from_numpy(E).to(dev), al, be, G, w0=si.w0, bdiffw0=si.bdiffw0,
                                       h=si.h, dt=si.dt, n_steps=si.n_steps, max_err=si.max_err,
                                       min_err=si.min_err, sel=si.sel, trace_cap=trace_cap if i == 0 else 0)
        attempts += st["attempts"]
        A = A.cpu().numpy()
        if i == 0:
            first_A, first_trace = A, tr
        X = np.fft.fft(A)
        E = np.fft.ifft(X * a.feedback + a.pump)
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t0
    gpu_s = ev0.elapsed_time(ev1) / 1000.0
    return {"trips": n_trips, "wall_s": wall, "event_s": gpu_s, "s_per_trip": gpu_s / n_trips,
            "trips_per_s": n_trips / gpu_s, "attempts": attempts, "field": E,
            "first_pass_out": first_A, "first_pass_trace": first_trace}
