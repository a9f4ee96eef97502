"""Accuracy at the bench's own workload: the 2^14-point, 5 mm SPOPO cavity.  Marked gpu.

The FP32 propagator's crystal pass is compared with the plain FP64 solver (the
persistent FP64 kernel, itself equal to the FP64 oracle on every schedule of
tests/test_fp64_gpu.py) from the same crystal input: a built-up cavity field
after five round trips.  Both take the same step schedule, the field agrees to
rel-L2 <= 1e-4 and the crystal-output energy to <= 1e-6.  The reference's own
FP32 CUDA kernels (OPO_CUDA_BATCH_XTAL.cu, compiled unmodified, with cuFFT),
given the same input and taking the same schedule, differ from FP64 by far more
(cuFFT's FP32 round trips drift): the tolerance is met here because of this
engine's precision design, not because the path is easy.  Over round trips the
difference grows (the cavity amplifies it), so the multi-trip check bounds two
trips.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-4          # rel-L2 of the crystal-output field
ENERGY_TOL = 1e-6         # crystal-output (intracavity) energy
TWO_TRIP_TOL = 1e-3       # next crystal input after two round trips


def _spec():
    from optifax_gb300.opo import CavitySpec
    return CavitySpec(n_points=2 ** 14, window=12e-12, crystal_length=5e-3, period=30e-6, pump_power=2.0,
                      pump_tau=200e-15, oc_output=0.10, delay=0.0, seed=1)


@pytest.fixture(scope="module")
def built_up():
    from optifax_gb300 import opo
    sim = opo.OpticalSim(_spec())
    sim.run(5)
    torch.cuda.synchronize()
    return sim, sim.field.cpu().numpy().astype(np.complex128)


def _fp32_pass(si, E, cap):
    from optifax_gb300 import solver as sv
    dev = torch.device("cuda:0")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    p = sv.PulseSpec(E=t(E.astype(np.complex64)), alpha=t(si.alpha), beta=t(si.beta), G=t(si.G), w0=si.w0,
                     bdiffw0=si.bdiffw0, h=si.h, dt=si.dt, max_err=si.max_err, min_err=si.min_err, sel=si.sel,
                     n_steps=si.n_steps, trace_cap=cap)
    outs, st = sv.propagate([p])
    st = sv.decode_stats(st)[0]
    return np.fft.fft(outs[0].cpu().numpy().astype(np.complex128)), p.trace.cpu().numpy()[:st["attempts"]]


def _wide_pass(si, E, cap, entry="propagate_fp64"):
    from optifax_gb300 import solver as sv
    dev = torch.device("cuda:0")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    A, st, tr = getattr(sv, entry)(t(E.astype(np.complex128)), t(si.alpha.astype(np.float64)),
                                   t(si.beta.astype(np.float64)), t(si.G.astype(np.float64)), w0=si.w0,
                                   bdiffw0=si.bdiffw0, h=si.h, dt=si.dt, n_steps=si.n_steps, max_err=si.max_err,
                                   min_err=si.min_err, sel=si.sel, trace_cap=cap)
    assert st["status"] == 0
    return np.fft.fft(A.cpu().numpy()), tr


def _key(tr):
    return np.stack([tr[:, 0], tr[:, 1], (tr[:, 2] >> 3) & 1], axis=1)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_full_pass_matches_fp64(built_up):
    sim, E = built_up
    si, arr = sim.arrays.si, sim.arrays
    cap = 4 * si.n_steps
    E32in = E.astype(np.complex64).astype(np.complex128)
    X32, tr32 = _fp32_pass(si, E32in, cap)
    X64, tr64 = _wide_pass(si, E32in, cap)
    assert np.array_equal(_key(tr32), _key(tr64)), "FP32 and FP64 step schedules differ"
    assert _rel(X32, X64) <= FIELD_TOL, _rel(X32, X64)
    e32, e64 = arr.tally_w @ np.abs(X32) ** 2, arr.tally_w @ np.abs(X64) ** 2
    intracavity = 2
    assert abs(e32[intracavity] - e64[intracavity]) <= ENERGY_TOL * e64[intracavity]


def test_reference_kernels_drift_more_on_the_same_input(built_up):
    """The reference's own FP32 kernels from the same input, on the same schedule:
    their difference from FP64 is at least ten times the propagator's."""
    from oracle import ref_mex
    ok, why = ref_mex.available()
    if not ok:
        pytest.skip(why)
    sim, E = built_up
    si = sim.arrays.si
    cap = 4 * si.n_steps
    E32in = E.astype(np.complex64).astype(np.complex128)
    X32, _ = _fp32_pass(si, E32in, cap)
    X64, tr64 = _wide_pass(si, E32in, cap)
    r = ref_mex.run(E32in.astype(np.complex64), si.alpha, si.G, si.beta, w0=si.w0, bdiffw0=si.bdiffw0, h=si.h,
                    n_steps=si.n_steps, dt=si.dt, max_err=si.max_err, min_err=si.min_err, sel=si.sel,
                    trace_cap=cap)
    Xr = np.fft.fft(r.A[0].astype(np.complex128))
    assert np.array_equal(_key(r.trace[:r.attempts]), _key(tr64))
    assert _rel(Xr, X64) >= 10 * _rel(X32, X64), (_rel(Xr, X64), _rel(X32, X64))


def test_two_round_trips_match_fp64(built_up):
    from optifax_gb300 import opo
    sim, E = built_up
    arr = sim.arrays
    si = arr.si
    E32in = E.astype(np.complex64).astype(np.complex128)
    sim2 = opo.OpticalSim(_spec())
    sim2.field = torch.from_numpy(E32in.astype(np.complex64)).cuda()
    r = sim2.run(2)
    e32 = r.field.cpu().numpy().astype(np.complex128)
    e64 = E32in
    for _ in range(2):
        X, _ = _wide_pass(si, e64, 0)
        e64 = np.fft.ifft(X * arr.feedback + arr.pump)
    assert _rel(e32, e64) <= TWO_TRIP_TOL, _rel(e32, e64)
