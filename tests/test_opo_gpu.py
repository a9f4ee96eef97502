"""Fused multi-trip OPO on the GPU vs an FP64 round-trip loop around the oracle.  Marked gpu.

The oracle loop restates OpticalSim.run (toolbox/lib/classes/OpticalSim.m:230-288)
with the per-trip optics as per-mode products in FP64.  Checked per trip:
step schedule, pump-band and intracavity energies, and the next-trip crystal
input field.
"""
import numpy as np
import pytest
import torch

from tests._cases import rel_l2

pytestmark = pytest.mark.gpu


def oracle_opo(orc, arr, n_trips):
    si = arr.si
    E = arr.E0.copy()
    out = []
    for _ in range(n_trips):
        r = orc.run(E, si.alpha, si.G, si.beta, w0=si.w0, bdiffw0=si.bdiffw0, h=si.h,
                    n_steps=si.n_steps, dt=si.dt, max_err=si.max_err, min_err=si.min_err,
                    sel=si.sel, trace_cap=100000)
        X = np.fft.fft(r.A[0])
        tallies = arr.tally_w @ (np.abs(X) ** 2)
        out.append((r.stats[0], tallies, r.trace[0]))
        E = np.fft.ifft(X * arr.feedback + arr.pump)
    return E, out


def _compare(oracle, spec, n_trips, tally_tol, field_tol):
    from optifax_gb300 import opo
    sim = opo.OpticalSim(spec)
    res = sim.run(n_trips)
    torch.cuda.synchronize()
    assert res.trips_done == n_trips
    E_ref, ref = oracle_opo(oracle, sim.arrays, n_trips)
    worst = 0.0
    for n in range(n_trips):
        st, tal, tr = ref[n]
        g = res.trips[n]
        assert g["status"] == 0
        assert g["attempts"] == st["attempts"] and g["accepted"] == st["accepted"]
        for i in (opo.TALLY_INTRACAVITY, opo.TALLY_PUMP_BAND):
            rel = abs(g["tally"][i] - tal[i]) / abs(tal[i])
            worst = max(worst, rel)
            assert rel <= tally_tol(n), (n, i, g["tally"][i], tal[i])
    err = rel_l2(res.field.cpu().numpy(), E_ref)
    assert err <= field_tol, err
    return worst, err


def test_opo_round_trips_low_gain(oracle):
    """Signal stays near the noise floor: energies within 1e-6, field within 1e-4."""
    from optifax_gb300 import opo
    spec = opo.CavitySpec(n_points=1024, window=1024 * 6e-12 / 2 ** 13, crystal_length=0.3e-3,
                          pump_tau=60e-15, pump_power=0.5, seed=1)
    _compare(oracle, spec, 5, lambda n: 1e-6, 1e-4)


def test_opo_round_trips_high_gain(oracle):
    """Strong parametric gain amplifies the FP32 rounding noise that enters
    the one-photon signal seed (the oracle's seed carries FP64 noise), by the
    single-pass gain every trip; once the signal depletes the pump the pump-band
    energies inherit that relative difference.  The bound therefore widens
    with the trip index: 1e-6 on the first pass, 1e-4 on the second, 1e-2 after."""
    from optifax_gb300 import opo
    spec = opo.CavitySpec(n_points=1024, window=1024 * 6e-12 / 2 ** 13, crystal_length=0.4e-3,
                          pump_tau=60e-15, pump_power=3.0, seed=1)
    _compare(oracle, spec, 5, lambda n: 1e-6 if n == 0 else (1e-4 if n == 1 else 1e-2), 1e-2)


def test_opo_steady_state_stop():
    """The device-side steady-state test ends the run early and reports the trips done."""
    from optifax_gb300 import opo
    spec = opo.CavitySpec(n_points=1024, window=1024 * 6e-12 / 2 ** 13, crystal_length=0.2e-3,
                          pump_tau=60e-15, pump_power=0.5, seed=2)
    sim = opo.OpticalSim(spec)
    # a loose tolerance on the intracavity energy is met after a few trips
    res = sim.run(50, steady_tol=0.5, steady_trips=3, steady_tally=opo.TALLY_INTRACAVITY)
    assert 3 < res.trips_done < 50
    assert np.all(res.trips["status"] == 0)


def test_opo_diagnostics_esd_and_step_records():
    """ESD trip sums and per-trip stepmods records (OpticalSim.averageSimPulses and
    StepSizeModifiers) against the recorded per-trip crystal outputs."""
    from optifax_gb300 import opo
    spec = opo.CavitySpec(n_points=2048, window=2048 * 6e-12 / 2 ** 13, crystal_length=0.2e-3,
                          pump_tau=100e-15, pump_power=1.5, seed=3)
    sim = opo.OpticalSim(spec)
    res = sim.run(3, history=True, esd=True, step_records=True)
    X = res.history.cpu().numpy().astype(np.complex128)
    w = sim.arrays.esd_w
    ref = np.stack([np.sum(w[i] * np.abs(X) ** 2, axis=0) for i in range(2)])
    got = res.esd.cpu().numpy()
    for i in range(2):
        assert np.abs(got[i] - ref[i]).max() <= 1e-5 * ref[i].max()
    # without a history buffer the library keeps the trip output in its own scratch
    sim2 = opo.OpticalSim(spec)
    res2 = sim2.run(3, esd=True)
    assert np.array_equal(res2.esd.cpu().numpy(), got)
    av = sim.esd_averages(res)
    assert np.allclose(av["out"], got[0] / 3, rtol=1e-6, atol=0)
    assert np.all(av["pump_depletion"][av["wavelength_nm"] > 1100] == 0)
    smt = res.step_size_modifiers.cpu().numpy()
    assert smt.shape == (3, sim.arrays.si.n_steps)
    for r in range(3):
        s_ = smt[r][smt[r] > 0]
        assert np.all(s_ == np.round(s_)) and s_.max() <= 64
        # one record per accepted step (accepted steps sit at strictly increasing k < S)
        assert len(s_) == res.trips["accepted"][r]
