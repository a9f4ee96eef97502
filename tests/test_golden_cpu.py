"""The FP64 oracle against golden outputs of the reference's own CUDA kernels (CPU).

tests/golden/*.npz were written by tests/golden/make_reference_fixtures.py, which
runs OptiFax's MEX kernels (OPO_CUDA_BATCH_XTAL.cu, _NO_BC.cu, _HARD_BC.cu and
ode23/OPO_CUDA_ODE23.cu, compiled unmodified) on a GPU.  Each file holds the inputs
exactly as the kernels received them and their outputs.  Here the oracle replays the
kernels' own step decisions and must reproduce their step schedule and stepmods
record exactly, and their field and Ap snapshots within FIELD_TOL: the drift of the
reference's FP32 cuFFT round trips, which tests/test_reference_kernels_gpu.py
measures on the GPU (5e-5 to 5.3e-4 on these cases).  For the Heun files the
oracle's own decisions, unreplayed, give the same schedule too; RK23's frequent
rejections leave some decisions close enough to the thresholds for FP32 and FP64
to part, so it is compared under replay only.
"""
import glob
import os

import numpy as np
import pytest

from tests._cases import rel_l2

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FILES = sorted(glob.glob(os.path.join(HERE, "*.npz")))
FIELD_TOL = 1e-3


def _conventions(orc, method, variant, N):
    """(method, time mode, absorber, chunk rule, stepmods limit) of each MEX file."""
    if method == "rk23":
        return orc.RK23_MEX, orc.TIME_UNSHIFTED, orc.ABC_SOFT, orc.CHUNKS_TRUNC, (N // 256) * 256
    lim = -(-N // 128) * 128
    return {0: (orc.HEUN_MEX, orc.TIME_SHIFTED, orc.ABC_SOFT, orc.CHUNKS_CEIL, lim),
            2: (orc.HEUN_MEX, orc.TIME_UNSHIFTED, orc.ABC_NONE, orc.CHUNKS_TRUNC, lim),
            3: (orc.HEUN_MEX, orc.TIME_UNSHIFTED, orc.ABC_HARD, orc.CHUNKS_TRUNC, lim)}[variant]


def test_fixtures_present():
    assert len(FILES) >= 7, FILES


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f)[:-4] for f in FILES])
def test_oracle_reproduces_reference_kernels(oracle, path):
    g = np.load(path)
    method, variant = str(g["method"]), int(g["variant"])
    w0, bdiffw0, h, S, dt, max_err, min_err, sel = [float(v) for v in g["scalars"]]
    E, trace = g["E"], g["trace"]
    N = E.shape[-1]
    m, tm, abc, ch, lim = _conventions(oracle, method, variant, N)
    r = oracle.run(E.astype(np.complex128), g["alpha"], g["G"], g["beta"], w0=w0, bdiffw0=bdiffw0, h=h,
                   n_steps=int(S), dt=dt, max_err=max_err, min_err=min_err, sel=sel, method=m, time_mode=tm,
                   abc_mode=abc, chunk_mode=ch, stepmods_limit=lim, trace_cap=200000, forced=trace[:, 2] & 3)
    tr = r.trace[0]
    assert len(tr) == len(trace)
    assert np.array_equal(tr[:, :2], trace[:, :2]), "step schedules differ under replay"
    assert np.array_equal(tr[:, 2] & 8, trace[:, 2] & 8), "accept/reject differs"
    assert np.sum((trace[:, 2] & 8) == 0) > 0, "the case should exercise rejections"
    assert np.array_equal(r.stepmods.astype(np.float32), g["stepmods"]), "stepmods record differs"
    err = rel_l2(g["A"], r.A[0])
    assert err <= FIELD_TOL, err
    if method == "heun":
        # Heun: the oracle's own FP64 decisions equal the kernels' FP32 ones on these cases
        own = oracle.run(E.astype(np.complex128), g["alpha"], g["G"], g["beta"], w0=w0, bdiffw0=bdiffw0, h=h,
                         n_steps=int(S), dt=dt, max_err=max_err, min_err=min_err, sel=sel, method=m,
                         time_mode=tm, abc_mode=abc, chunk_mode=ch, stepmods_limit=lim, trace_cap=200000)
        assert np.array_equal(own.trace[0][:, :2], trace[:, :2]), "own schedule differs"
    if "Ap" in g.files:
        ref_ap = g["Ap"]
        ap = r.Ap.reshape(-1, N)[:ref_ap.shape[0]]
        errs = [rel_l2(ref_ap[c], ap[c]) for c in range(ref_ap.shape[0]) if np.any(ap[c])]
        assert errs and max(errs) <= FIELD_TOL, errs
