"""The GNLSE oracle (oracle/gnlse_oracle.py) against known answers, on the CPU.

gnlsefib.m's own integrator is MATLAB's ode45 (not available), so parity is
unpinned; these checks establish that the restated equation and conventions are
right: a fundamental soliton keeps its shape and advances its phase by
gamma P0 z / 2 (anomalous dispersion, no Raman, no shock), pure dispersion with
loss is exact, the photon number sum |AW|^2 / W is conserved with self-steepening
and Raman scattering, and a recorded schedule replays bit for bit.
"""
import numpy as np
import pytest

from oracle import gnlse_oracle as go

B2, GAMMA, T0 = -1.183e-26, 0.11, 28.4e-15


def _grid(n=1024, window=2e-12):
    return np.arange(-n // 2, n // 2) * (window / n)


def test_fundamental_soliton():
    T = _grid()
    P0 = abs(B2) / (GAMMA * T0 ** 2)
    A = np.sqrt(P0) / np.cosh(T / T0)
    ops = go.gnlse_ops(T, 0.0, GAMMA, [B2], 0.0, 0.0, 0.0)
    z0 = np.pi / 2 * T0 ** 2 / abs(B2)                 # soliton period
    r = go.propagate(ops, A, 2 * z0, 5)
    for i, z in enumerate(r.Z):
        assert np.max(np.abs(np.abs(r.AT[i]) - np.abs(A))) / np.sqrt(P0) < 2e-5
        ph = np.angle(r.AT[i][len(T) // 2] / A[len(T) // 2])
        expect = (GAMMA * P0 * z / 2 + np.pi) % (2 * np.pi) - np.pi
        assert abs(ph - expect) < 1e-5


def test_dispersion_and_loss_exact():
    T = _grid()
    A = 30.0 / np.cosh(T / T0) * np.exp(1j * 0.3 * T / T0)
    ops = go.gnlse_ops(T, 0.0, 0.0, [B2, 8e-41], 1.5, 0.0, 0.0)
    z = 0.05
    r = go.propagate(ops, A, z, 3)
    exact = np.fft.fft(np.fft.ifft(A) * np.exp(-0.5 * ops.alpha * z) * np.exp(1j * ops.B * z))
    assert np.linalg.norm(r.AT[-1] - exact) / np.linalg.norm(exact) < 1e-13


def test_photon_number_conserved_with_shock_and_raman():
    n = 2048
    T = _grid(n, 4e-12)
    w0 = 2 * np.pi * 299792458.0 / 835e-9
    P0 = 600.0
    A = np.sqrt(P0) / np.cosh(T / T0)
    RT = go.raman_response(T)
    ops = go.gnlse_ops(T, w0, GAMMA, [B2, 8.1e-41, -9.5e-56], 0.0, 0.18, RT)
    r = go.propagate(ops, A, 0.01, 3)
    Wabs = np.fft.fftshift(ops.W)                      # centred V + w0
    photons = [np.sum(np.abs(aw) ** 2 / Wabs) for aw in r.AW]
    assert abs(photons[-1] / photons[0] - 1) < 1e-8
    energy = [np.sum(np.abs(aw) ** 2) for aw in r.AW]
    assert abs(energy[-1] / energy[0] - 1) > 1e-5      # Raman moves energy (to the red): not conserved


def test_replay_reproduces_schedule():
    T = _grid(512, 1.5e-12)
    A = np.sqrt(300.0) / np.cosh(T / T0)
    ops = go.gnlse_ops(T, 0.0, GAMMA, [B2], 0.0, 0.0, 0.0)
    a = go.propagate(ops, A, 0.05, 4)
    b = go.propagate(ops, A, 0.05, 4, forced=a.steps)
    assert a.steps == b.steps
    assert np.array_equal(a.AT, b.AT)
    assert any(ok == 0 for _, ok in a.steps) or a.attempts == a.accepted


def test_raman_term_is_the_causal_convolution():
    """gnlsefib.m's RS = dT fR fft(ifft(|A|^2) RW), RW = n ifft(fftshift(hR)), is the
    causal circular convolution dT fR sum_j hR(j dT) |A|^2_{l-j} (convolution theorem
    with MATLAB's fft/ifft): the time origin and fftshift placement are right."""
    n = 128
    T = _grid(n, 2e-12)
    rng = np.random.default_rng(3)
    IT = rng.uniform(0.0, 2.0, n)
    hR = go.raman_response(T)
    ops = go.gnlse_ops(T, 0.0, 1.0, [0.0], 0.0, 0.18, hR)
    RS = ops.dT * ops.fr * np.fft.fft(np.fft.ifft(IT) * ops.RW)
    hs = np.fft.fftshift(hR)                          # hR(j dT) at index j (zero for t < 0)
    direct = np.array([ops.dT * ops.fr * sum(hs[j] * IT[(l - j) % n] for j in range(n)) for l in range(n)])
    assert np.max(np.abs(RS - direct)) <= 1e-12 * np.max(np.abs(direct))
    assert np.all(hs[n // 2 + 1:] == 0.0)             # causal: nothing from the future


def test_pure_self_phase_modulation_is_exact():
    """No dispersion, no Raman response, no shock term (w0 = 0): dA/dz = i gamma |A|^2 A
    keeps |A| and turns the phase by gamma |A|^2 z at every instant."""
    n = 512
    T = _grid(n, 2e-12)
    A = np.sqrt(1000.0) / np.cosh(T / 50e-15)
    ops = go.gnlse_ops(T, 0.0, 0.11, [0.0], 0.0, 0.0, 0.0)
    r = go.propagate(ops, A, 0.01, 3)
    for i, z in enumerate(r.Z):
        exact = A * np.exp(1j * 0.11 * np.abs(A) ** 2 * z)
        assert np.linalg.norm(r.AT[i] - exact) / np.linalg.norm(exact) < 1e-6


@pytest.mark.parametrize("n,loss,raman,shock", [(1024, 0.0, True, True), (2048, 0.5, True, True),
                                               (512, 0.0, False, False)])
def test_c_restatement_matches_numpy(n, loss, raman, shock):
    """oracle/gnlse_oracle.c against this file's propagate(): the same step schedule and
    fields to FP64 rounding (the FFTs differ), also when replaying a forced schedule."""
    T = _grid(n, 2e-12 * n / 1024)
    w0 = 2 * np.pi * 299792458.0 / 835e-9 if shock else 0.0
    RT = go.raman_response(T) if raman else 0.0
    ops = go.gnlse_ops(T, w0, 0.11, [-1.183e-26, 8.1e-41, -9.5e-56], loss, 0.18 if raman else 0.0, RT)
    A = np.sqrt(1000.0) / np.cosh(T / 28.4e-15)
    ref = go.propagate(ops, A, 0.01, 4)
    own = go.propagate_c(ops, A, 0.01, 4)[0]
    rep = go.propagate_c(ops, A, 0.01, 4, forced=ref.steps)[0]
    assert own.steps == ref.steps and own.attempts == ref.attempts and own.accepted == ref.accepted
    assert np.allclose(own.Z, ref.Z, rtol=0, atol=0)
    for r in (own, rep):
        for i in range(4):
            assert np.linalg.norm(r.AT[i] - ref.AT[i]) <= 1e-12 * np.linalg.norm(ref.AT[i])
            assert np.linalg.norm(r.AW[i] - ref.AW[i]) <= 1e-12 * np.linalg.norm(ref.AW[i])


def test_c_restatement_batch_in_parallel_equals_one_by_one():
    n = 512
    T = _grid(n, 1.5e-12)
    w0 = 2 * np.pi * 299792458.0 / 835e-9
    ops = go.gnlse_ops(T, w0, 0.11, [-1.183e-26, 8.1e-41], 0.0, 0.18, go.raman_response(T))
    A = np.stack([np.sqrt(p) / np.cosh(T / 28.4e-15) for p in (300.0, 900.0, 2000.0)])
    batch = go.propagate_c(ops, A, 0.01, 3, nthreads=3)
    for b in range(3):
        one = go.propagate_c(ops, A[b], 0.01, 3, nthreads=1)[0]
        assert batch[b].steps == one.steps
        assert np.array_equal(batch[b].AT, one.AT) and np.array_equal(batch[b].AW, one.AW)
    with pytest.raises(RuntimeError):                                     # forced schedule runs out
        go.propagate_c(ops, A[0], 0.01, 3, forced=batch[0].steps[:2])
