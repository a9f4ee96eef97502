"""Known answers of the host-side solver-input set-up (optifax_gb300/physics.py).

The reference ships no fixtures for its set-up (SimWindow.m, phi_calc.m,
QPMcrystal.m, chirpedgrating.m, sechPulse.m / Laser.m), so each piece is pinned
by a property its definition fixes exactly.
"""
import numpy as np
import pytest

from optifax_gb300 import physics as ph


@pytest.fixture(scope="module")
def win():
    return ph.SimWindow(1040e-9, 2 ** 13, 6e-12)


def test_constant_period_grating_flips_every_half_period():
    """QPMcrystal.m with zero uncertainty: domains of period/2 from z = 0, the first of
    sign -1, so sign(z) = -1 on even half-periods and +1 on odd ones."""
    L, period, n = 1e-3, 30e-6, 10000
    s = ph.qpm_signs(n, L, period)
    z = np.linspace(0.0, L, n)
    expect = np.where(np.floor(z / (period / 2)) % 2 == 0, -1.0, 1.0)
    assert np.array_equal(s, expect)
    assert int(np.sum(s[1:] != s[:-1])) == int(np.floor(2 * L / period))


def test_linear_chirp_walls_sit_on_half_turns_of_the_qpm_phase():
    """Exact linear chirp p(z) = p1 + (p2 - p1) z / L: wall m where the QPM phase
    int_0^z dz' / p(z') reaches m / 2; the last domains are p2 / 2 wide."""
    L, p1, p2 = 1e-3, 28e-6, 32e-6
    z = np.linspace(0.0, L, 10000)
    walls = ph.qpm_walls(z, L, ("linear", p1, p2))
    a = (p2 - p1) / L
    theta = np.log1p(a * walls / p1) / a
    assert np.max(np.abs(theta - np.arange(1, len(walls) + 1) / 2)) < 1e-9
    assert walls[-1] < L <= walls[-1] + p2
    assert abs((walls[-1] - walls[-2]) / (p2 / 2) - 1) < 5e-3


def test_relative_phase_has_no_value_or_delay_at_the_reference(win):
    """phi_calc.m: the group delay at w0 is removed and the phase at w0 subtracted."""
    phi_rel, phi_abs, n = ph.phi_calc(1e-3, win)
    r, w = win.ref_index, win.omegas
    assert phi_rel[r] == 0.0
    gd_rel = (phi_rel[r + 1] - phi_rel[r - 1]) / (w[r + 1] - w[r - 1])
    gd_abs = (phi_abs[r + 1] - phi_abs[r - 1]) / (w[r + 1] - w[r - 1])
    assert abs(gd_rel) < 1e-6 * gd_abs
    assert 2.10 < n[r] < 2.20                      # MgO:LN extraordinary index near 1 um


def test_sech_pump_carries_the_pulse_energy_and_width(win):
    """Laser.m / sechPulse.m: average power / repetition rate per pulse (I2pow.m units),
    transform-limited sech^2 of the given intensity FWHM."""
    E = ph.sech_pump(win, 1040e-9, 200e-15, 2.0, f_rep=100e6, waist=15e-6)
    energy = ph.energy_from_shifted(np.fft.fftshift(E), win, 15e-6)
    assert abs(energy / 2e-8 - 1) < 1e-12
    inten = np.abs(E) ** 2
    above = win.times[inten >= inten.max() / 2]
    assert abs((above.max() - above.min() + win.dt) / 200e-15 - 1) < 0.01


def test_photon_noise_holds_one_photon_per_seeded_mode(win):
    mask = ph.window_transmission(win)
    noise = ph.photon_noise(win, seed=3, waist=15e-6, mask=mask)
    spec = np.fft.fft(np.fft.fftshift(noise))
    e_mode = np.abs(spec) ** 2 * (ph.C0 * ph.EPS0 / 2) * np.pi * (15e-6) ** 2 * win.dt / win.n_points
    w = np.fft.ifftshift(win.omegas)
    seeded = (w > 0) & np.fft.ifftshift(mask.astype(bool))
    assert seeded.sum() > win.n_points // 2
    assert np.max(np.abs(e_mode[seeded] / (ph.HBAR * w[seeded]) - 1)) < 1e-9
    assert np.all(e_mode[~seeded] < 1e-30 * e_mode[seeded].max())
    phases = np.exp(1j * np.angle(spec[seeded]))
    assert abs(phases.mean()) < 5 / np.sqrt(seeded.sum())


def test_counter_stream_is_reproducible_and_prefix_stable():
    a = ph.counter_uniform(7, 1000)
    assert np.array_equal(a[:100], ph.counter_uniform(7, 100))
    assert np.array_equal(a, ph.counter_uniform(7, 1000))
    assert not np.array_equal(a, ph.counter_uniform(8, 1000))
    assert not np.array_equal(a, ph.counter_uniform(7, 1000, stream=1))
    assert a.min() >= 0.0 and a.max() < 1.0 and abs(a.mean() - 0.5) < 0.05
