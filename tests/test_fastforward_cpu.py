"""Fast-forward crop geometry, envelope resampling and host helpers (CPU)."""
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


def test_envelope_is_an_exact_resampling_of_its_band():
    """envelope() places the band's bins on an n_bins grid and inverse-transforms them:
    the transform of the envelope gives the band's bins back exactly, and nothing else."""
    from optifax_gb300 import fastforward as ff
    rng = np.random.default_rng(0)
    N, L, kc, lo, hi = 4096, 256, 1000, -40, 90
    X = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    e = ff.envelope(X, kc, lo, hi, L)
    b = np.fft.fft(e) / L
    o = np.arange(lo, hi)
    assert np.allclose(b[o % L], X[(kc + o) % N], rtol=0, atol=1e-12)
    rest = np.ones(L, bool)
    rest[o % L] = False
    assert np.max(np.abs(b[rest])) < 1e-12


def test_interaction_picture_and_error_helpers():
    import torch
    from optifax_gb300 import fastforward as ff
    rng = np.random.default_rng(1)
    D = torch.from_numpy(np.exp(1j * rng.uniform(0, 6, 64)) * rng.uniform(0.5, 1.0, 64))
    D[5] = 0
    X = torch.from_numpy(rng.standard_normal(64) + 1j * rng.standard_normal(64))
    Y = ff.to_interaction(X * D, D)
    keep = torch.ones(64, dtype=torch.bool)
    keep[5] = False
    assert torch.allclose(Y[keep], X[keep], atol=1e-12) and Y[5] == 0
    t = torch.from_numpy(rng.standard_normal((3, 4, 16)))
    y = t.clone()
    y[:, 2:4] *= 1.1                                              # signal channels 10 % off
    assert torch.allclose(ff.signal_rel_err(y, t), torch.full((3,), 0.1, dtype=t.dtype), atol=1e-12)
    assert torch.allclose(ff.sample_weights(t), 1.0 / t.pow(2).mean(dim=(1, 2)))


def test_phase_aligned_error_ignores_a_global_signal_phase():
    import torch
    from optifax_gb300 import fastforward as ff
    g = torch.Generator().manual_seed(0)
    x = torch.randn(64, generator=g, dtype=torch.float64) + 1j * torch.randn(64, generator=g, dtype=torch.float64)
    m = torch.zeros(64, dtype=torch.bool)
    m[10:40] = True
    assert ff.phase_aligned_err(x * complex(0.6, 0.8), x, m) < 1e-14
    y = x.clone()
    y[20] += 0.5
    direct = float((x[m] - y[m]).abs().norm() / y[m].abs().norm())
    assert abs(ff.phase_aligned_err(x, y, m) - direct) < 0.05 * direct


def test_align_signal_phase_rotates_only_the_signal_bins():
    import torch
    from optifax_gb300 import fastforward as ff
    g = torch.Generator().manual_seed(1)
    ins = (torch.randn(3, 32, generator=g) + 1j * torch.randn(3, 32, generator=g)).to(torch.complex64)
    m = torch.zeros(32, dtype=torch.bool)
    m[4:20] = True
    rot = torch.tensor([complex(0, 1), complex(-1, 0), complex(0.6, -0.8)], dtype=torch.complex64)
    outs = ins.clone()
    outs[:, m] = ins[:, m] * rot[:, None]
    al = ff.align_signal_phase(ins, outs, m)
    assert torch.allclose(al[:, m], ins[:, m], atol=1e-6)
    assert torch.equal(al[:, ~m], outs[:, ~m])
