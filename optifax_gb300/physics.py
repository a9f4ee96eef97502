"""Host-side set-up of the crystal-pass solver inputs (FP64, NumPy).

This module produces the 14 solver arguments that OptiFax's ``OpticalSim.run``
hands to its crystal-pass solver (toolbox/lib/classes/OpticalSim.m:213-252),
plus the pump and noise fields of a synchronously pumped OPO.  It restates the
reference's set-up arithmetic:

* time/frequency grid: toolbox/lib/classes/SimWindow.m:61-163, fftax.m:1-5
* MgO:LN extraordinary index (Gayer 2008, 5% MgO CLN, column 1):
  toolbox/lib/internal/materials/n_mgoppln_gayer.m:11-37
* relative dispersion phase with the group delay at w0 removed:
  toolbox/lib/internal/phi_calc.m:5-45
* QPM sign per z-sample: toolbox/lib/internal/main/QPMcrystal.m:10-51
  (zero poling uncertainty, zero duty-cycle offset)
* sech^2 pump scaled to V/m: toolbox/lib/internal/sechPulse.m:9-15,
  toolbox/lib/classes/Laser.m:53,66-77,95-99
* solver-argument precompute: toolbox/lib/classes/OpticalSim.m:213-226,
  toolbox/lib/classes/NonlinearCrystal.m:52-61,141-144

Choices that the reference leaves to data files or does not define are
stated where they are made: crystal transmission (lossless inside the
simulation window's spectral limits, zero outside, which is what
``transmission.m:28`` does at the limits), air index 1, and the one-photon-
per-mode noise seed (the reference starts the intracavity field at zero).
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional, Sequence

import numpy as np

C0 = 299792458.0            # toolbox/static/CONST/c.m
EPS0 = 8.854e-12            # toolbox/static/CONST/eps0.m
HBAR = 1.054571817e-34


# --------------------------------------------------------------------------
# Grid
# --------------------------------------------------------------------------
@dataclasses.dataclass
class SimWindow:
    """Time/frequency grid (SimWindow.m with Constraint = "time")."""

    reference_wave: float          # [m]
    n_points: int
    temporal_range: float          # [s]
    spectral_limits_nm: tuple = (300.0, 6000.0)

    @property
    def times(self) -> np.ndarray:
        n = self.n_points
        return np.arange(-n // 2, n // 2, dtype=np.float64) / n * self.temporal_range

    @property
    def dt(self) -> float:
        t = self.times
        return float(t[1] - t[0])

    @property
    def rel_freqs(self) -> np.ndarray:
        n = self.n_points
        return np.arange(-n // 2, n // 2, dtype=np.float64) / (n * self.dt)

    @property
    def f0(self) -> float:
        return C0 / self.reference_wave

    @property
    def omegas(self) -> np.ndarray:
        return 2 * np.pi * (self.rel_freqs + self.f0)

    @property
    def rel_omegas(self) -> np.ndarray:
        return self.omegas - self.reference_omega

    @property
    def reference_omega(self) -> float:
        return 2 * np.pi * C0 / self.reference_wave

    @property
    def wavelengths(self) -> np.ndarray:
        with np.errstate(divide="ignore"):
            return 2 * np.pi * C0 / self.omegas

    @property
    def ref_index(self) -> int:
        """0-based index of w0 on the fftshifted grid (SimWindow.m:161-163)."""
        return self.n_points // 2

    @property
    def d_omega(self) -> float:
        w = self.omegas
        return float(w[1] - w[0])


# --------------------------------------------------------------------------
# Materials
# --------------------------------------------------------------------------
_GAYER = dict(a1=5.756, a2=0.0983, a3=0.2020, a4=189.32, a5=12.52, a6=1.32e-2,
              b1=2.860e-6, b2=4.700e-8, b3=6.113e-8, b4=1.516e-4)


def n_mgoln_e(lam_um: np.ndarray, celsius: float = 20.0) -> np.ndarray:
    """5% MgO:CLN extraordinary index, Gayer et al. APB 91, 343 (2008)."""
    g = _GAYER
    fn = (celsius - 24.5) * (celsius + 570.82)
    l2 = np.asarray(lam_um, dtype=np.float64) ** 2
    a3 = g["a3"] + g["b3"] * fn
    with np.errstate(divide="ignore", invalid="ignore"):
        n2 = ((g["a1"] + g["b1"] * fn) + (g["a2"] + g["b2"] * fn) / (l2 - a3 * a3)
              + (g["a4"] + g["b4"] * fn) / (l2 - g["a5"] ** 2) - g["a6"] * l2)
    n = np.sqrt(n2.astype(np.complex128)).real
    n = np.where(np.isfinite(n), n, 1.0)
    n[n < 1] = 1.0                 # Dielectric.m:43-44
    return n


def phi_calc(length: float, win: SimWindow, celsius: float = 20.0):
    """Relative and absolute phase of a crystal of length ``length``.

    Follows phi_calc.m:14-45: beta = w n / c, group delay by first
    differences, group delay at w0 subtracted, relative phase by trapezoidal
    integration over 0.2-20 um, spline extension elsewhere, then the value at
    w0 subtracted.
    """
    from scipy.interpolate import CubicSpline

    w = win.omegas
    lam = win.wavelengths
    n = n_mgoln_e(lam * 1e6, celsius)
    beta_abs = w * n / C0
    phi_abs = length * beta_abs
    gd_abs = np.concatenate([[0.0], np.diff(phi_abs) / np.diff(w)])
    r = win.ref_index
    gd_rel = gd_abs - gd_abs[r]
    w_rel = win.rel_omegas
    del_phi = gd_rel * np.concatenate([[0.0], np.diff(w_rel)])
    sel = (lam > 2e-7) & (lam < 2e-5)
    d = del_phi[sel]
    cum = np.concatenate([[0.0], np.cumsum(0.5 * (d[1:] + d[:-1]))])
    # interp1(..., 'spline') needs increasing abscissae
    ls = lam[sel]
    order = np.argsort(ls)
    spl = CubicSpline(ls[order], cum[order], bc_type="not-a-knot", extrapolate=True)
    phi_off = spl(lam)
    phi_rel = phi_off - phi_off[r]
    return phi_rel, phi_abs, n


# --------------------------------------------------------------------------
# Crystal
# --------------------------------------------------------------------------
def qpm_signs(n_steps: int, length: float, period) -> np.ndarray:
    """Domain sign per z-sample, z = linspace(0, L, n_steps).

    Constant period: QPMcrystal.m:20-51 with zero uncertainty and zero duty
    offset (all domains period/2, first domain sign -1, remainder domain to
    the crystal end).  ``period=("linear", p1, p2)`` gives an exact linear
    chirp of the local period from p1 at z=0 to p2 at z=L (walls where the
    accumulated QPM phase crosses multiples of pi).
    ``period=("chirpedgrating", p1, p2, a, tol)`` takes the domain widths of
    the reference's discretised power-law chirp (chirped_domain_widths).
    """
    z = np.linspace(0.0, length, n_steps)
    edges = np.concatenate([[0.0], qpm_walls(z, length, period)])
    q = np.searchsorted(edges, z, side="right")      # 1-based domain index
    q = np.mod(q, 2)
    return -(2.0 * q - 1.0)


def qpm_walls(z: np.ndarray, length: float, period) -> np.ndarray:
    """Domain-wall positions (ascending, < length) of qpm_signs' gratings."""
    if isinstance(period, (tuple, list)) and period[0] == "chirpedgrating":
        widths = chirped_domain_widths(z, *period[1:])
        walls = np.cumsum(widths)
        walls = walls[walls < length]      # a last domain past L is cut at L (QPMcrystal.m:44-50)
    elif isinstance(period, (tuple, list)) and period[0] == "linear":
        p1, p2 = float(period[1]), float(period[2])
        a = (p2 - p1) / length
        theta_end = (np.log1p(a * length / p1) / a) if a != 0 else length / p1
        m = np.arange(1, int(np.floor(2.0 * theta_end)) + 1, dtype=np.float64)
        walls = (p1 / a) * np.expm1(a * m / 2.0) if a != 0 else m * p1 / 2.0
        walls = walls[walls < length]
    else:
        p = float(period)
        n_dom = int(np.floor(2.0 * length / p))
        walls = np.cumsum(np.full(n_dom, p / 2.0))
        walls = walls[walls < length]
    return walls


def chirped_domain_widths(z: np.ndarray, p1: float, p2: float, a: float = 1.0,
                          tol: float = 0.1e-6) -> np.ndarray:
    """Domain widths of a power-law chirped grating (chirpedgrating.m:1-47).

    The local period p1 + (p2 - p1) (z/L)^a is quantised to multiples of tol
    (p1 raised by tol and the grid offset by p2 + tol/2 before rounding, as
    the reference does), halved to a domain width, and then sampled domain by
    domain: each domain takes the width at the current z-sample and advances
    by round(width / dz) samples, until the next domain would pass the end.
    ``a = 1`` is a linear chirp.
    """
    z = np.asarray(z, dtype=np.float64)
    p1 = p1 + tol
    zfrac = z / z.max()
    gr = p1 + (p2 - p1) * zfrac ** a - (p2 + tol / 2.0)
    # MATLAB round(): half away from zero
    q = np.sign(gr / tol) * np.floor(np.abs(gr / tol) + 0.5)
    domains = q * tol / 2.0 + p2 / 2.0
    dz = z[1] - z[0]
    n_dom = int(np.ceil(np.sum(dz / domains)))
    dsteps = np.sign(domains / dz) * np.floor(np.abs(domains / dz) + 0.5)
    out = np.zeros(n_dom)
    sid = 0                                  # 0-based stepID
    pos = 0.0
    zmax = z.max()
    for ii in range(n_dom):
        out[ii] = domains[sid]
        sid = sid + int(dsteps[sid])
        if sid > len(domains) - 1:
            sid = len(domains) - 1
        pos += out[ii]
        if pos + domains[sid] > zmax:
            return out[:ii + 1]
    return out


@dataclasses.dataclass
class Crystal:
    """Periodically poled MgO:LN crystal (NonlinearCrystal with "PPLN" bulk)."""

    length: float
    period: object = 30e-6
    d_eff: float = 14e-12
    celsius: float = 20.0
    step_size: float = 1e-7

    @property
    def chi2(self) -> float:
        # The solver resolves every domain, so the effective coefficient of a
        # first-order QPM grating is (2/pi) d.  d_eff is the post-QPM value, so
        # d = (pi/2) d_eff and chi2 = 2 d (NonlinearCrystal.m:54 convention).
        return 2.0 * (math.pi / 2.0) * self.d_eff

    @property
    def n_steps(self) -> int:
        return int(math.floor(self.length / self.step_size))     # NonlinearCrystal.m:71


def window_transmission(win: SimWindow) -> np.ndarray:
    """Lossless inside the window's spectral limits, zero outside (transmission.m:28)."""
    lam = win.wavelengths
    lo, hi = win.spectral_limits_nm
    t = ((lam >= lo * 1e-9) & (lam <= hi * 1e-9)).astype(np.float64)
    return t


@dataclasses.dataclass
class SolverInputs:
    """The 14 crystal-pass solver arguments (OpticalSim.m:238-252) plus context."""

    alpha: np.ndarray        # TStepShift, float32 N
    G: np.ndarray            # G33, float32 S
    w0: float                # float32 value
    bdiffw0: float           # double
    h: float                 # float32 value
    n_steps: int
    dt: float                # double
    beta: np.ndarray         # hBshift, float32 N
    max_err: float           # percent, float32 value
    min_err: float           # percent, float32 value
    sel: float
    n_chunks: int
    n_index: np.ndarray      # crystal index per fftshifted bin (natural FFT order)
    n0: float


def solver_scalars(xtal: Crystal, win: SimWindow) -> dict:
    """The scalar solver inputs of OpticalSim.run (w0, bdiffw0, n0, the G33
    magnitude) from the index at the reference bin and the one below it."""
    r = win.ref_index
    w = win.omegas[r - 1:r + 1]
    lam = win.wavelengths[r - 1:r + 1]
    n = n_mgoln_e(lam * 1e6, xtal.celsius)
    phi_abs = xtal.length * (w * n / C0)
    n0 = float(n[1])
    w0 = float(np.float32(win.reference_omega))
    beta0_w0 = float((2 * np.pi * n / lam)[1])
    # xtal.GroupDelay = phi2GD(Bulk.Phi, dw) (Optic.m:130-133, phi2GD.m:1-15):
    # backward first difference at the reference index, per unit length
    beta1_w0 = float((phi_abs[1] - phi_abs[0]) / win.d_omega / xtal.length)
    return {"n0": n0, "w0": w0, "bdiffw0": beta0_w0 - beta1_w0 * w0,
            "g_scale": xtal.chi2 * w0 / n0 / 4.0 / C0}


def solver_inputs(xtal: Crystal, win: SimWindow, error_bounds=(2.5e-3, 5e-2),
                  progress_plots: int = 5) -> SolverInputs:
    """OpticalSim.run precompute (OpticalSim.m:213-226)."""
    f32 = lambda v: float(np.float32(v))
    S = xtal.n_steps
    sel = float(math.ceil(S / (progress_plots - 1)))
    phi_rel, phi_abs, n = phi_calc(xtal.length, win, xtal.celsius)
    sc = solver_scalars(xtal, win)
    n0, w0, bdiffw0 = sc["n0"], sc["w0"], sc["bdiffw0"]
    P = qpm_signs(S, xtal.length, xtal.period)
    G = (P * xtal.chi2 * w0 / n0 / 4.0 / C0).astype(np.float32)
    T = window_transmission(win)
    with np.errstate(divide="ignore", invalid="ignore"):
        alpha = np.where(T > 0, T ** (1.0 / S), 0.0)
    beta = phi_rel / xtal.length * xtal.step_size
    beta = np.where((T > 0) & np.isfinite(beta), beta, 0.0)
    n_chunks = int(S / sel)
    if n_chunks * sel < S:
        n_chunks += 1
    return SolverInputs(
        alpha=np.fft.fftshift(alpha).astype(np.float32), G=G, w0=w0,
        bdiffw0=float(bdiffw0), h=f32(xtal.step_size), n_steps=S, dt=win.dt,
        beta=np.fft.fftshift(beta).astype(np.float32),
        max_err=f32(error_bounds[1]), min_err=f32(error_bounds[0]), sel=sel,
        n_chunks=n_chunks, n_index=np.fft.fftshift(n), n0=n0)


# --------------------------------------------------------------------------
# Fields
# --------------------------------------------------------------------------
def default_linewidth(lambda_c: float, dtau: float) -> float:
    """Laser.m:53 transform-limited linewidth for a sech^2 of FWHM dtau."""
    return (4 * C0 * 0.315 * dtau * lambda_c ** 2) / ((2 * C0 * dtau) ** 2 - (lambda_c * 0.315) ** 2)


def sech_t_rms(lambda_c: float, dtau: float) -> float:
    """sech width parameter of a transform-limited sech^2 of FWHM dtau (sechPulse.m)."""
    dlam = default_linewidth(lambda_c, dtau)
    edges = lambda_c + np.array([-dlam, dlam]) / 2.0
    nu_fwhm = float(np.ptp(C0 / edges))
    t_fwhm = 0.315 / nu_fwhm
    return t_fwhm / (2 * np.log(1 + 2 ** 0.5))


def sech_pump(win: SimWindow, lambda_c: float, dtau: float, avg_power: float,
              f_rep: float = 100e6, waist: float = 15e-6, n_medium: float = 1.0) -> np.ndarray:
    """sech^2 pump field [V/m] on the natural time grid (sechPulse.m, Laser.m:66-77).

    The field is centred at t = 0, transform limited, and scaled so that
    sum |E|^2 (c n eps0 / 2) (pi waist^2) dt equals the pulse energy.
    The reference computes the field at the reference wavelength; the pump
    carrier offset from it (lambda_c != reference) is applied as a linear
    temporal phase.
    """
    t = win.times
    t_rms = sech_t_rms(lambda_c, dtau)
    u = 1.0 / np.cosh(t / t_rms)
    w_p = 2 * np.pi * C0 / lambda_c
    u = u * np.exp(1j * (w_p - win.reference_omega) * t)
    area = np.pi * waist ** 2
    energy = avg_power / f_rep
    scale = np.sqrt(2.0 * energy / (np.sum(np.abs(u) ** 2) * win.dt * area * n_medium * EPS0 * C0))
    return (scale * u).astype(np.complex128)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    return z ^ (z >> np.uint64(31))


def counter_uniform(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """Counter-based uniform [0,1): SplitMix64 of (seed, stream, index)."""
    with np.errstate(over="ignore"):
        key = (np.uint64(seed) * np.uint64(0x100000001B3) + np.uint64(stream)) & np.uint64(0xFFFFFFFFFFFFFFFF)
        ctr = np.arange(n, dtype=np.uint64) + (key << np.uint64(20))
        r = _splitmix64(ctr)
    return (r >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def photon_noise(win: SimWindow, seed: int, waist: float = 15e-6, n_medium: float = 1.0,
                 mask: Optional[np.ndarray] = None) -> np.ndarray:
    """One photon per mode with uniform random phase, on the natural time grid.

    Spectral amplitude per FFT bin k (N-point FFT of the fftshifted field):
    |E_k|^2 = 2 hbar w_k N / (c n eps0 A dt), the energy of one photon hbar w_k
    (Parseval with the I2pow.m units).  Only bins with w_k > 0 and inside
    ``mask`` are seeded.  No counterpart in the reference, which starts the
    intracavity field at exactly zero (OpticalSim.m:120-123).
    """
    n = win.n_points
    w = np.fft.ifftshift(win.omegas)                 # natural FFT order
    area = np.pi * waist ** 2
    amp = np.sqrt(np.maximum(2 * HBAR * w * n / (C0 * n_medium * EPS0 * area * win.dt), 0.0))
    m = w > 0
    if mask is not None:
        m &= np.fft.ifftshift(mask.astype(bool))
    phase = 2 * np.pi * counter_uniform(seed, n)
    spec = np.where(m, amp * np.exp(1j * phase), 0.0)
    et_shift = np.fft.ifft(spec)                     # fftshifted time
    return np.fft.ifftshift(et_shift)


def energy_from_shifted(et_shift: np.ndarray, win: SimWindow, waist: float, n_medium: float = 1.0):
    """Pulse energy [J] of fftshifted fields (..., N) via Parseval (I2pow.m:15-20)."""
    n = et_shift.shape[-1]
    ek = np.fft.fft(et_shift, axis=-1)
    return np.sum(np.abs(ek) ** 2, axis=-1) * (C0 * n_medium * EPS0 / 2) * np.pi * waist ** 2 * win.dt / n


def smoothed_top_hat(x: np.ndarray, a: float, b: float, w: float) -> np.ndarray:
    """smoothedTopHat.m:40 (tanh form)."""
    return 0.5 * (np.tanh((x - a) / w) - np.tanh((x - b) / w))
