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
