"""The precision study's error metrics (config 4) on fields with known differences."""
import numpy as np

from optifax_gb300 import precision


def _ref(n=1024, seed=0):
    rng = np.random.default_rng(seed)
    t = np.arange(n) - n / 2
    return np.exp(-(t / 40.0) ** 2) * np.exp(1j * 0.01 * t ** 2) + 1e-3 * (rng.standard_normal(n) +
                                                                            1j * rng.standard_normal(n))


def test_a_global_phase_is_a_pure_spectral_phase_error():
    ref = _ref()
    m = precision.metrics(ref * np.exp(0.1j), ref)
    assert abs(m["rel_l2"] - 2 * np.sin(0.05)) < 1e-12
    assert m["energy_rel"] < 1e-14
    assert abs(m["spectral_phase_rms_rad"] - 0.1) < 1e-12


def test_a_gain_is_an_amplitude_and_energy_error_only():
    ref = _ref()
    m = precision.metrics(1.01 * ref, ref)
    assert abs(m["rel_l2"] - 0.01) < 1e-12
    assert abs(m["energy_rel"] - (1.01 ** 2 - 1)) < 1e-12
    assert m["spectral_phase_rms_rad"] < 1e-12


def test_bins_below_the_floor_carry_no_phase_error():
    """Scrambling the phase of the spectral bins under 1e-3 of the peak power leaves the
    spectral phase error at zero (they are outside the weighted set)."""
    ref = _ref()
    fr = np.fft.fft(ref)
    pw = np.abs(fr) ** 2
    weak = pw <= 1e-3 * pw.max()
    assert weak.any() and (~weak).any()
    fa = fr.copy()
    fa[weak] *= np.exp(1j * np.random.default_rng(1).uniform(-np.pi, np.pi, weak.sum()))
    m = precision.metrics(np.fft.ifft(fa), ref)
    assert m["bins"] == int((~weak).sum())
    assert m["spectral_phase_rms_rad"] < 1e-9
    assert m["rel_l2"] > 0
