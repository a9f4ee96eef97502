"""Fast-forward crop geometry (CPU)."""
import numpy as np


def test_crop_holds_signal_band_and_pump():
    from optifax_gb300 import fastforward as ff, opo
    spec = opo.CavitySpec()
    a = opo.build_cavity(spec)
    crop = ff.reference_crop(spec)
    N = crop.n_points
    f = a.win.f0 + np.fft.fftfreq(N, d=a.win.dt)
    idx = (crop.k0 + np.arange(crop.n_bins)) % N
    fc = f[idx]
    assert np.all(np.diff(fc) > 0)                       # contiguous, increasing
    assert fc[0] <= ff.F_LO + 1e11 and fc[crop.split - 1] < ff.F_SPLIT <= fc[crop.split]
    fb = np.abs(a.feedback) > 1e-6 * np.abs(a.feedback).max()   # the filter edges decay smoothly
    assert np.all(np.isin(np.nonzero(fb)[0], idx[:crop.split]))   # every fed-back bin is in the signal crop
    pk = np.argmax(np.abs(a.pump))
    assert pk in idx[crop.split:]


def test_envelope_bands_abut_and_hold_the_feedback_band():
    from optifax_gb300 import fastforward as ff, opo
    spec = opo.CavitySpec()
    a = opo.build_cavity(spec)
    crop = ff.reference_env_crop(spec)
    kp, lop, hip, ks, los, his = crop.band
    N = crop.n_points
    rel = lambda kc, o: ((kc + o + N // 2) % N) - N // 2          # signed global bin
    assert rel(ks, his) == rel(kp, lop)                          # signal band ends where the pump band starts
    sig_bins = {(ks + o) % N for o in range(los, his)}
    fb = np.nonzero(np.abs(a.feedback) > 1e-6 * np.abs(a.feedback).max())[0]
    assert set(fb.tolist()) <= sig_bins
    assert int(np.argmax(np.abs(a.pump))) in {(kp + o) % N for o in range(lop, hip)}
    e = ff.envelope(a.pump, kp, lop, hip, crop.n_bins)
    assert abs(np.max(np.abs(e)) - crop.pump_scale) <= 1e-6 * crop.pump_scale
