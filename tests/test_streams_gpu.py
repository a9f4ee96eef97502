"""Calls on caller-given CUDA streams.  Marked gpu.

One handle serves calls on different streams: the handle's descriptors and
exchange scratch are shared by its calls, so a call on another stream than the
previous call's waits for that call's work (optifax_context's end-of-call event).
Each result must equal the same pass run alone on the current stream.  The Python
wrappers given a side stream prepare their inputs, launch and read back on that
stream (solver.on_stream): the statistics they return are those of a finished run.
"""
import numpy as np
import pytest
import torch

from tests._cases import make_case, rel_l2

pytestmark = pytest.mark.gpu


def _spec(si, E, dev):
    from optifax_gb300 import solver as sv
    return sv.PulseSpec(
        E=torch.from_numpy(E.astype(np.complex64)).to(dev),
        alpha=torch.from_numpy(si.alpha).to(dev), beta=torch.from_numpy(si.beta).to(dev),
        G=torch.from_numpy(si.G).to(dev), w0=si.w0, bdiffw0=si.bdiffw0, h=si.h, dt=si.dt,
        max_err=si.max_err, min_err=si.min_err, sel=si.sel, n_steps=si.n_steps)


def test_one_handle_two_streams():
    """Two 8192-point passes (clusters of two CTAs, so the exchange scratch is in
    use) issued back to back on two streams through one handle."""
    from optifax_gb300 import solver as sv
    dev = torch.device("cuda:0")
    win, si, E = make_case(N=8192, length=0.2e-3, power=2.0, B=2)
    alone = []
    for b in range(2):
        outs, stats = sv.propagate([_spec(si, E[b], dev)])
        torch.cuda.synchronize()
        alone.append((outs[0].cpu().numpy(), sv.decode_stats(stats)[0]))
    specs = [_spec(si, E[b], dev) for b in range(2)]
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    o1, st1 = sv.propagate([specs[0]], stream=s1)
    o2, st2 = sv.propagate([specs[1]], stream=s2)
    torch.cuda.synchronize()
    for (A, st_alone), o, st in zip(alone, (o1, o2), (st1, st2)):
        got = sv.decode_stats(st)[0]
        assert got["status"] == 0 and got["attempts"] == st_alone["attempts"], (got, st_alone)
        assert rel_l2(o[0].cpu().numpy(), A) <= 1e-6


def test_gnlse_on_side_stream_returns_finished_stats():
    from optifax_gb300 import gnlse
    n = 1024
    T = np.arange(-n // 2, n // 2) * (2e-12 / n)
    w0 = 2 * np.pi * 299792458.0 / 835e-9
    ops = gnlse.fibre_operators(T, w0, 0.11, [-1.183e-26, 8.1e-41, -9.5e-56], 0.0, 0.18,
                                gnlse.raman_response(T))
    A = np.sqrt(900.0) / np.cosh(T / 28.4e-15)
    ref = gnlse.propagate(ops, A, 0.01, 3, w0=w0)
    s = torch.cuda.Stream()
    side = gnlse.propagate(ops, A, 0.01, 3, w0=w0, stream=s)
    s.synchronize()
    assert ref.stats[0]["attempts"] > 0 and side.stats == ref.stats
    assert np.array_equal(side.AT.cpu().numpy(), ref.AT.cpu().numpy())


def test_opo_on_side_stream_matches_current_stream():
    from optifax_gb300 import opo
    spec = opo.CavitySpec(n_points=1024, window=1024 * 6e-12 / 2 ** 13, crystal_length=0.2e-3,
                          pump_tau=60e-15, pump_power=0.5, seed=2)
    ref = opo.OpticalSim(spec).run(4)
    s = torch.cuda.Stream()
    side = opo.OpticalSim(spec).run(4, stream=s)
    s.synchronize()
    assert side.trips_done == ref.trips_done == 4
    assert np.array_equal(side.trips["attempts"], ref.trips["attempts"])
    assert rel_l2(side.field.cpu().numpy(), ref.field.cpu().numpy()) <= 1e-6
