"""Seeded synthetic crystal-pass cases shared by the tests (sech^2 pump + photon noise)."""
from __future__ import annotations

import numpy as np

from optifax_gb300 import physics as ph


def make_case(N=1024, length=0.2e-3, window=None, power=1.0, tau=None, period=30e-6,
              seed=0, error_bounds=(2.5e-3, 5e-2), lambda_ref=1040e-9, B=1, d_eff=14e-12,
              progress_plots=5, waist=15e-6):
    """Crystal-pass inputs with the reference's conventions.

    The grid keeps dt = 6 ps / 2^13 unless ``window`` is given; the pulse
    width defaults to min(200 fs, window/12).  Returns the
    solver inputs and the fftshifted in-crystal field(s) E (B, N) complex128.
    """
    if window is None:
        window = N * (6e-12 / 2 ** 13)
    if tau is None:
        tau = min(200e-15, window / 12)     # keep the pulse clear of the absorbing boundary
    win = ph.SimWindow(lambda_ref, N, window)
    xt = ph.Crystal(length, period, d_eff=d_eff)
    si = ph.solver_inputs(xt, win, error_bounds=error_bounds, progress_plots=progress_plots)
    Es = []
    for b in range(B):
        pump = ph.sech_pump(win, 1040e-9, tau, power * (1.0 + 0.1 * b), waist=waist)
        noise = ph.photon_noise(win, seed + b, waist=waist, mask=ph.window_transmission(win))
        e = np.fft.fftshift(pump + noise)
        ek = np.fft.fft(e) * np.sqrt(1.0 / si.n_index)   # refract into the crystal
        Es.append(np.fft.ifft(ek))
    return win, si, np.array(Es)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
