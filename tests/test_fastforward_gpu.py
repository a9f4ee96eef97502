"""Fast-forward helpers and the surrogate/solver hand-over.  Marked gpu."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_encode_and_step_match_numpy():
    from optifax_gb300 import fastforward as ff, physics as ph
    win = ph.SimWindow(1040e-9, 2 ** 14, 12e-12)
    crop = ff.make_crop(win, pump_scale=3.0)
    rng = np.random.default_rng(0)
    N, L, s = crop.n_points, crop.n_bins, crop.split
    Y = (rng.normal(size=(2, N)) + 1j * rng.normal(size=(2, N))).astype(np.complex64)
    dev = torch.device("cuda:0")
    x, sig = ff.encode(torch.from_numpy(Y).to(dev), crop)
    x, sig = x.cpu().numpy(), sig.cpu().numpy()
    idx = (crop.k0 + np.arange(L)) % N
    for p in range(2):
        c = Y[p, idx].astype(np.complex128)
        sg = np.sqrt(np.mean(np.abs(c[:s]) ** 2))
        assert abs(sig[p] - sg) <= 1e-5 * sg
        assert np.allclose(x[p, 2, :s] + 1j * x[p, 3, :s], c[:s] / sg, atol=1e-5)
        assert np.allclose(x[p, 0, s:] + 1j * x[p, 1, s:], c[s:] / 3.0, atol=1e-5)
        assert np.all(x[p, 0, :s] == 0) and np.all(x[p, 2, s:] == 0)
        assert np.allclose(x[p, 4], np.log10(sg / 3.0), atol=1e-5)
        assert np.allclose(x[p, 5], np.arange(L) / L)
    fb = (rng.normal(size=N) + 1j * rng.normal(size=N)).astype(np.complex64)
    pump = (rng.normal(size=N) + 1j * rng.normal(size=N)).astype(np.complex64)
    tw = rng.uniform(size=N).astype(np.float32)
    lin = np.exp(1j * rng.uniform(0, 2 * np.pi, N)).astype(np.complex64)
    y = x[0, :4].copy()
    e = torch.zeros(1, dtype=torch.float64, device=dev)
    Xo = torch.empty(N, dtype=torch.complex64, device=dev)
    Yn = ff.step(crop, torch.from_numpy(fb).to(dev), torch.from_numpy(pump).to(dev), torch.from_numpy(tw).to(dev),
                 y=torch.from_numpy(y).to(dev), sigma=torch.tensor([sig[0]], device=dev),
                 lin=torch.from_numpy(lin).to(dev), X_out=Xo, energy=e)
    X = np.zeros(N, dtype=np.complex128)
    X[idx] = Y[0, idx] * lin[idx]                      # decode(encode(Y)) is the crop of Y, times lin
    assert np.allclose(Xo.cpu().numpy(), X, atol=1e-4)
    assert np.allclose(Yn.cpu().numpy(), X * fb + pump, atol=1e-3)
    ref_e = np.sum(tw * np.abs(X) ** 2)
    assert abs(e.item() - ref_e) <= 1e-5 * ref_e


def test_untrained_surrogate_falls_back_and_solver_finishes():
    """An untrained network fails its first check; the solver takes over and the
    trip accounting stays exact."""
    from optifax_gb300 import fastforward as ff, opo
    from optifax_gb300.surrogate import FNO
    spec = opo.CavitySpec(crystal_length=0.5e-3)
    crop = ff.reference_crop(spec)
    net = FNO(n_bins=crop.n_bins, max_batch=1, seed=0)
    sim = opo.OpticalSim(spec)
    r = ff.run_fast_forward(sim, net, crop, max_trips=25, check_every=5, check_tol=0.05, finish_trips=5)
    assert r["checks"] and not (r["checks"][0] <= 0.05)
    assert r["fallback_blocks"] >= 1
    assert r["trips"] == r["surrogate_trips"] + r["solver_trips"]
    assert r["trips"] <= 25


def test_envelope_encode_decode_round_trip():
    from optifax_gb300 import fastforward as ff, opo
    spec = opo.CavitySpec()
    a = opo.build_cavity(spec)
    crop = ff.reference_env_crop(spec)
    kp, lop, hip, ks, los, his = crop.band
    rng = np.random.default_rng(1)
    N, L = crop.n_points, crop.n_bins
    Y = (rng.normal(size=(2, N)) + 1j * rng.normal(size=(2, N))).astype(np.complex64)
    dev = torch.device("cuda:0")
    x, sig = ff.encode(torch.from_numpy(Y).to(dev), crop)
    xh, sg = x.cpu().numpy(), sig.cpu().numpy()
    for p in range(2):
        ep = ff.envelope(Y[p].astype(np.complex128), kp, lop, hip, L)
        es = ff.envelope(Y[p].astype(np.complex128), ks, los, his, L)
        s = np.sqrt(np.mean(np.abs(es) ** 2))
        assert abs(sg[p] - s) <= 1e-4 * s
        assert np.abs(xh[p, 0] + 1j * xh[p, 1] - ep / crop.pump_scale).max() <= 1e-4 * np.abs(ep).max() / crop.pump_scale
        assert np.abs(xh[p, 2] + 1j * xh[p, 3] - es / s).max() <= 1e-4 * np.abs(es).max() / s
        assert np.allclose(xh[p, 5], np.arange(L) / L)
    X = ff.decode_env(crop, x[0:1, :4].contiguous(), sig[0:1]).cpu().numpy()
    ref = np.zeros(N, dtype=np.complex128)
    for kc, lo, hi in ((kp, lop, hip), (ks, los, his)):
        idx = (kc + np.arange(lo, hi)) % N
        ref[idx] = Y[0, idx]
    assert np.abs(X - ref).max() <= 1e-4 * np.abs(ref).max()


def test_trained_surrogate_beats_the_identity_map_on_unseen_trips():
    """The shipped network (trained on 20,480 solver pairs from cavities with seeds
    300000 + i) on trips 20..39 of the config-2 cavity itself (seed 1, not in the
    training set): its phase-aligned signal error is below the identity map's, the
    prediction "the crystal pass changes nothing" in the interaction picture, and so
    is its error in the fed-back band's energy, which the fast-forward loop's energy
    check compares; on some of these trips that check (5 %) passes."""
    from optifax_gb300 import fastforward as ff, opo
    from optifax_gb300.surrogate import FNO, pretrained
    spec = opo.CavitySpec()
    params, meta = pretrained()
    crop = ff.reference_env_crop(spec)
    net = FNO(n_bins=crop.n_bins, max_batch=32, params=params)
    sim = opo.OpticalSim(spec)
    r = sim.run(40, history=True)
    ins = torch.empty_like(r.history)
    ins[0] = torch.from_numpy(np.fft.fft(sim.arrays.E0).astype(np.complex64)).cuda()
    ins[1:] = r.history[:-1] * sim.feedback + sim.pump
    outs = ff.to_interaction(r.history, ff.linear_factor(sim))
    tgt = ff.align_signal_phase(ins, outs, ff.signal_mask(crop, ins.shape[1], ins.device))
    X, T = ff.encode_pairs(ins[20:], tgt[20:], crop)
    err_net = ff.evaluate(net, X, T).cpu().numpy()
    err_id = ff.signal_rel_err(X[:, :4], T).cpu().numpy()
    assert np.median(err_net) < np.median(err_id), (np.median(err_net), np.median(err_id))
    assert np.mean(err_net < err_id) >= 0.6, np.mean(err_net < err_id)
    # the fast-forward loop's energy check on the same trips: relative error of the
    # fed-back band's energy, the network's predicted crystal output against the
    # solver's, beside the identity map's (linear propagation only)
    D = ff.linear_factor(sim)
    fbm = np.abs(sim.feedback.cpu().numpy()) > 0
    e_net, e_id = [], []
    for t in range(20, 40):
        x, sig = ff.encode(ins[t:t + 1], crop)
        Xs = torch.empty(crop.n_points, dtype=torch.complex64, device=ins.device)
        ff.step(crop, sim.feedback, sim.pump, None, y=net.forward(x), sigma=sig, lin=D, X_out=Xs)
        et = np.sum(np.abs(r.history[t].cpu().numpy().astype(np.complex128)[fbm]) ** 2)
        for pred, out in ((Xs, e_net), (ins[t] * D, e_id)):
            out.append(abs(np.sum(np.abs(pred.cpu().numpy().astype(np.complex128)[fbm]) ** 2) - et) / et)
    e_net, e_id = np.array(e_net), np.array(e_id)
    assert np.median(e_net) < np.median(e_id), (np.median(e_net), np.median(e_id))
    assert np.sum(e_net <= 0.05) >= 2, e_net          # trips on which a 5 % energy check passes
    assert np.mean(e_net < e_id) >= 0.6, np.mean(e_net < e_id)
