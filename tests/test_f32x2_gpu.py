"""The float-float crystal pass (optifax_propagate_f32x2).  Marked gpu.

At low gain it equals the FP64 oracle (same schedule, rel-L2 <= 1e-10: its
~48-bit field is a little short of FP64's 53 bits).  At high gain -- the
config-2 cavity's first pass from the one-photon-per-mode seed, where the
parametric gain amplifies the FP32 field's rounding to a few percent -- it stays
within 1e-4 of the FP64 solver, as the FP32 propagator cannot.
"""
import numpy as np
import pytest
import torch

from tests._cases import make_case, rel_l2

pytestmark = pytest.mark.gpu

LOW_GAIN_TOL = 1e-10
HIGH_GAIN_TOL = 1e-4


def _wide(entry, si, E, variant=0, trace_cap=400000):
    from optifax_gb300 import solver as sv
    dev = torch.device("cuda:0")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    A, st, tr = getattr(sv, entry)(t(np.asarray(E, dtype=np.complex128)), t(si.alpha.astype(np.float64)),
                                   t(si.beta.astype(np.float64)), t(np.asarray(si.G, dtype=np.float64)),
                                   w0=si.w0, bdiffw0=si.bdiffw0, h=si.h, dt=si.dt, n_steps=si.n_steps,
                                   max_err=si.max_err, min_err=si.min_err, sel=si.sel, variant=variant,
                                   trace_cap=trace_cap)
    return A.cpu().numpy(), st, tr


@pytest.mark.parametrize("N,variant", [(1024, 0), (2048, 2), (4096, 3), (16384, 0)])
def test_f32x2_matches_oracle(oracle, N, variant):
    win, si, E = make_case(N=N, length=0.2e-3 if N <= 4096 else 0.05e-3, power=2.0)
    A, st, tr = _wide("propagate_f32x2", si, E[0], variant)
    tm, abc, ch = {0: (oracle.TIME_SHIFTED, oracle.ABC_SOFT, oracle.CHUNKS_CEIL),
                   2: (oracle.TIME_UNSHIFTED, oracle.ABC_NONE, oracle.CHUNKS_TRUNC),
                   3: (oracle.TIME_UNSHIFTED, oracle.ABC_HARD, oracle.CHUNKS_TRUNC)}[variant]
    ref = oracle.run(E[0], si.alpha, si.G, si.beta, w0=si.w0, bdiffw0=si.bdiffw0, h=si.h, n_steps=si.n_steps,
                     dt=si.dt, max_err=si.max_err, min_err=si.min_err, sel=si.sel, method=oracle.HEUN_MEX,
                     time_mode=tm, abc_mode=abc, chunk_mode=ch, trace_cap=400000)
    assert st["status"] == 0
    assert np.array_equal(ref.trace[0][:, :2], tr[:, :2]), "step schedules differ"
    assert rel_l2(A, ref.A[0]) <= LOW_GAIN_TOL, rel_l2(A, ref.A[0])


def test_f32x2_high_gain_first_pass():
    """Config-2 cavity, first pass from pump + one photon per mode (5 mm, 2^14)."""
    from optifax_gb300 import opo
    arr = opo.build_cavity(opo.CavitySpec(n_points=2 ** 14, window=12e-12, crystal_length=5e-3, pump_power=2.0,
                                          pump_tau=200e-15, seed=1))
    si = arr.si
    A64, st64, _ = _wide("propagate_fp64", si, arr.E0, trace_cap=0)
    A2, st2, _ = _wide("propagate_f32x2", si, arr.E0, trace_cap=0)
    err = rel_l2(np.fft.fft(A2), np.fft.fft(A64))
    assert st2["status"] == 0 and err <= HIGH_GAIN_TOL, (err, st2["attempts"], st64["attempts"])


def test_f32x2_rejects_nee_and_bad_sizes():
    from optifax_gb300 import solver as sv, _native as nat
    win, si, E = make_case(N=1024, length=0.1e-3)
    with pytest.raises(nat.OptifaxError):
        _wide("propagate_f32x2", si, E[0], variant=5)
    with pytest.raises(nat.OptifaxError):
        sv.propagate_f32x2(torch.zeros(1000, dtype=torch.complex128, device="cuda"),
                           torch.zeros(1000, dtype=torch.float64, device="cuda"),
                           torch.zeros(1000, dtype=torch.float64, device="cuda"),
                           torch.from_numpy(si.G.astype(np.float64)).cuda(), w0=si.w0, bdiffw0=si.bdiffw0,
                           h=si.h, dt=si.dt, n_steps=si.n_steps, max_err=si.max_err, min_err=si.min_err,
                           sel=si.sel)
