"""Known answers of the cavity set-up (opo.build_cavity): the per-mode transfer that
closes every round trip, the injected pump and the energy tallies
(OpticalSim.m:230-288; OpticalPulse.m:137-197,256-261,518-527; Cavity.m:50-87).
The output coupler works in regime "R" (intracavity sqrt(R), output sqrt(T)); the
crystal's refraction in and out cancels on the fed-back field (r_out r_in = 1)."""
import dataclasses

import numpy as np
import pytest

from optifax_gb300 import opo, physics as ph


@pytest.fixture(scope="module")
def spec():
    return opo.CavitySpec(n_points=2 ** 13, window=6e-12, crystal_length=1e-3)


@pytest.fixture(scope="module")
def cav(spec):
    return opo.build_cavity(spec)


def test_feedback_is_the_filter_times_the_coupler(spec, cav):
    lam_nm = np.fft.ifftshift(cav.win.wavelengths) * 1e9
    lo, hi = spec.signal_band_nm
    mid = (lam_nm > lo + 10 * spec.filter_edge_nm) & (lam_nm < hi - 10 * spec.filter_edge_nm)
    # the filter is a tanh top-hat: 20 edge widths out it passes sqrt((1 - tanh 20) / 2) ~ 2e-9
    out = (lam_nm < lo - 20 * spec.filter_edge_nm) | (lam_nm > hi + 20 * spec.filter_edge_nm)
    assert mid.any() and out.any()
    assert np.allclose(np.abs(cav.feedback[mid]), np.sqrt(1.0 - spec.oc_output), rtol=1e-6)
    assert np.max(np.abs(cav.feedback[out])) < 1e-6
    assert np.all(np.abs(cav.feedback) <= np.sqrt(1.0 - spec.oc_output) * (1 + 1e-12))


def test_delay_turns_the_phase_only(spec, cav):
    d = 10e-15
    delayed = opo.build_cavity(dataclasses.replace(spec, delay=d))
    dw = np.fft.ifftshift(cav.win.rel_omegas)
    assert np.allclose(delayed.feedback, cav.feedback * np.exp(-1j * d * dw), rtol=1e-12, atol=1e-15)


def test_pump_carries_the_pulse_energy(spec, cav):
    """Average power / repetition rate at the crystal input, counted with the
    intracavity energy weight (air units: the refraction into the crystal undone)."""
    energy = float(np.sum(cav.tally_w[2] * np.abs(cav.pump) ** 2))
    assert abs(energy / (spec.pump_power / spec.f_rep) - 1) < 1e-9


def test_first_input_is_pump_plus_one_photon_per_mode(spec, cav):
    seed_k = np.fft.fft(cav.E0) - cav.pump                      # the noise, refracted into the crystal
    e_mode = cav.tally_w[2] * np.abs(seed_k) ** 2               # back in air units: J per mode
    w = np.fft.ifftshift(cav.win.omegas)
    seeded = (w > 0) & np.fft.ifftshift(ph.window_transmission(cav.win).astype(bool))
    assert np.allclose(e_mode[seeded], ph.HBAR * w[seeded], rtol=1e-6)
