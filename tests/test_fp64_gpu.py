"""The plain full-FP64 GPU crystal pass against the FP64 oracle.  Marked gpu.

Both compute in double precision from the same (FP32-valued) inputs, so the
step schedules must be identical and the output fields agree to FP64 rounding
of two different FFTs and sin/cos implementations: relative L2 <= 1e-11.  The
cases cover every cluster shape of the persistent FP64 kernel (1 to 16 CTAs,
512 to 65536 points) and its NEE_CPU.m instantiation.
"""
import numpy as np
import pytest
import torch

from tests._cases import make_case, rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11


def _fp64_gpu(si, E, variant, trace_cap=200000, G=None):
    from optifax_gb300 import solver as sv
    dev = torch.device("cuda:0")
    g = si.G if G is None else G
    A, st, tr = sv.propagate_fp64(
        torch.from_numpy(np.ascontiguousarray(E, dtype=np.complex128)).to(dev),
        torch.from_numpy(si.alpha.astype(np.float64)).to(dev),
        torch.from_numpy(si.beta.astype(np.float64)).to(dev),
        torch.from_numpy(np.ascontiguousarray(g, dtype=np.float64)).to(dev),
        w0=si.w0, bdiffw0=si.bdiffw0, h=si.h, dt=si.dt, n_steps=si.n_steps,
        max_err=si.max_err, min_err=si.min_err, sel=si.sel, variant=variant, trace_cap=trace_cap)
    torch.cuda.synchronize()
    return A.cpu().numpy(), st, tr


def _oracle(oracle, si, E, variant, G=None, shared=False):
    if variant == 5:
        return oracle.run(E, si.alpha, si.G if G is None else G, si.beta, w0=si.w0, bdiffw0=si.bdiffw0,
                          h=si.h, n_steps=si.n_steps, dt=si.dt, max_err=si.max_err, min_err=si.min_err,
                          sel=si.sel, method=oracle.HEUN_NEE, g_per_pulse=G is not None,
                          shared_schedule=shared, trace_cap=200000)
    tm, abc, ch = {0: (oracle.TIME_SHIFTED, oracle.ABC_SOFT, oracle.CHUNKS_CEIL),
                   1: (oracle.TIME_SHIFTED, oracle.ABC_SOFT, oracle.CHUNKS_CEIL),
                   2: (oracle.TIME_UNSHIFTED, oracle.ABC_NONE, oracle.CHUNKS_TRUNC),
                   3: (oracle.TIME_UNSHIFTED, oracle.ABC_HARD, oracle.CHUNKS_TRUNC)}[variant]
    return oracle.run(E, si.alpha, si.G if G is None else G, si.beta, w0=si.w0, bdiffw0=si.bdiffw0,
                      h=si.h, n_steps=si.n_steps, dt=si.dt, max_err=si.max_err, min_err=si.min_err,
                      sel=si.sel, method=oracle.HEUN_MEX, time_mode=tm, abc_mode=abc, chunk_mode=ch,
                      g_per_pulse=G is not None, shared_schedule=shared, trace_cap=200000)


@pytest.mark.parametrize("N,variant", [(1024, 0), (2048, 0), (1024, 2), (2048, 3), (512, 1), (1024, 5), (2048, 5),
                                       (4096, 0), (8192, 2), (16384, 0), (16384, 5), (32768, 0), (65536, 3)])
def test_fp64_single_pulse(oracle, N, variant):
    win, si, E = make_case(N=N, length=0.2e-3 if N <= 2048 else 0.03e-3, power=2.0)
    A, st, tr = _fp64_gpu(si, E[0], variant)
    ref = _oracle(oracle, si, E[0], variant)
    assert st["status"] == 0
    assert np.array_equal(ref.trace[0][:, :2], tr[:, :2]), "step schedules differ"
    assert np.array_equal(ref.trace[0][:, 2] & 11, tr[:, 2] & 11)
    assert st["attempts"] == ref.stats[0]["attempts"]
    assert st["z_steps"] == ref.stats[0]["z_steps"]
    err = rel_l2(A, ref.A[0])
    assert err <= FP64_TOL, err


def test_fp64_batch_shared_schedule(oracle):
    """B = 2 pulses with a G row each: one schedule for the batch, as the MEX."""
    win, si, E = make_case(N=1024, length=0.2e-3, power=1.5, B=2)
    G2 = np.stack([si.G, si.G[::-1].copy()])
    A, st, tr = _fp64_gpu(si, E, 0, G=G2)
    ref = _oracle(oracle, si, E, 0, G=G2, shared=True)
    assert np.array_equal(ref.trace[0][:, :2], tr[:, :2])
    for b in range(2):
        assert rel_l2(A[b], ref.A[b]) <= FP64_TOL


def test_fp64_rejects_bad_arguments():
    from optifax_gb300 import solver as sv, _native as nat
    win, si, E = make_case(N=1024, length=0.1e-3)
    dev = torch.device("cuda:0")
    with pytest.raises(nat.OptifaxError):
        sv.propagate_fp64(torch.zeros(1000, dtype=torch.complex128, device=dev),
                          torch.zeros(1000, dtype=torch.float64, device=dev),
                          torch.zeros(1000, dtype=torch.float64, device=dev),
                          torch.from_numpy(si.G.astype(np.float64)).to(dev),
                          w0=si.w0, bdiffw0=si.bdiffw0, h=si.h, dt=si.dt, n_steps=si.n_steps,
                          max_err=si.max_err, min_err=si.min_err, sel=si.sel)
    with pytest.raises(nat.OptifaxError):
        _fp64_gpu(si, E[0], 4)
