"""The reference's own CUDA kernels against the FP64 oracle and the GB300 propagator.
Marked gpu.

oracle/_ref/opo_cuda_batch_xtal.cubin is OPO_CUDA_BATCH_XTAL.cu compiled unmodified;
oracle/ref_mex.cpp drives its kernels with cuFFT as the MEX driver does.  This pins
the oracle (and through it the propagator) to the reference's own arithmetic: the
time convention, the shock-term stencil, G indexing, the absorber, the dispersion
sign and power, the chunk clamps, the k - 1 on reject and the Ap / stepmods records.

Each comparison runs on one step schedule: the reference's own decisions are
replayed in the oracle and the propagator (the oracle's own decisions are also
checked against the reference's).  FIELD_TOL bounds the field difference that the
reference's FP32 arithmetic leaves.
"""
import numpy as np
import pytest
import torch

from tests._cases import make_case, rel_l2

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-3


@pytest.fixture(scope="module")
def refmex():
    from oracle import ref_mex
    ok, why = ref_mex.available()
    if not ok:
        pytest.skip(why)
    return ref_mex


def _ref_run(refmex, si, E, forced=None):
    return refmex.run(E, si.alpha, si.G, si.beta, w0=si.w0, bdiffw0=si.bdiffw0, h=si.h,
                      n_steps=si.n_steps, dt=si.dt, max_err=si.max_err, min_err=si.min_err,
                      sel=si.sel, forced=forced)


def _oracle_run(oracle, si, E, forced=None):
    E64 = np.asarray(E, np.complex64).astype(np.complex128)
    return oracle.run(E64, si.alpha, si.G, si.beta, w0=si.w0, bdiffw0=si.bdiffw0, h=si.h,
                      n_steps=si.n_steps, dt=si.dt, max_err=si.max_err, min_err=si.min_err,
                      sel=si.sel, trace_cap=200000, forced=forced)


CASES = [(1024, 0.2e-3, 2.0), (2048, 0.3e-3, 2.0), (4096, 0.2e-3, 3.0)]


@pytest.mark.parametrize("N,length,power", CASES)
def test_oracle_matches_reference_kernels(oracle, refmex, N, length, power):
    win, si, E = make_case(N=N, length=length, power=power)
    ref = _ref_run(refmex, si, E[0])
    dec = ref.trace[:, 2] & 3
    orc = _oracle_run(oracle, si, E[0], forced=dec)
    otr = orc.trace[0]
    assert len(otr) == len(ref.trace)
    assert np.array_equal(otr[:, :2], ref.trace[:, :2]), "step schedules differ under replay"
    assert np.array_equal(otr[:, 2] & 8, ref.trace[:, 2] & 8)
    err = rel_l2(ref.A[0], orc.A[0])
    nch = ref.Ap.shape[1]
    ap_orc = orc.Ap.reshape(-1, N)[:nch]
    ap_err = max(rel_l2(ref.Ap[0, c], ap_orc[c]) for c in range(nch) if np.any(ap_orc[c]))
    own = (ref.trace[:, 2] >> 4) & 3
    orc_own = _oracle_run(oracle, si, E[0])
    same_sched = len(orc_own.trace[0]) == len(ref.trace) and \
        np.array_equal(orc_own.trace[0][:, :2], ref.trace[:, :2])
    print(dict(N=N, attempts=ref.attempts, rejected=int(np.sum((ref.trace[:, 2] & 8) == 0)),
               field_err=err, ap_err=ap_err, oracle_own_schedule_equal=same_sched,
               ref_seconds=ref.seconds))
    assert np.array_equal(own, dec)
    assert np.array_equal(orc.stepmods.astype(np.float32), ref.stepmods), "stepmods record differs"
    assert err <= FIELD_TOL, err
    assert ap_err <= FIELD_TOL, ap_err


@pytest.mark.parametrize("N,length,power,cta", [(1024, 0.2e-3, 2.0, 0), (4096, 0.2e-3, 3.0, 0),
                                                (4096, 0.2e-3, 3.0, 1024)])
def test_propagator_matches_reference_kernels(refmex, N, length, power, cta):
    from optifax_gb300 import _native as nat
    from tests.test_parity_gpu import _gpu_pass
    win, si, E = make_case(N=N, length=length, power=power)
    ref = _ref_run(refmex, si, E[0])
    A, Ap, sm, tr, st = _gpu_pass(si, E[0], nat.HEUN, nat.VARIANT_BATCH_XTAL, cta,
                                  forced=(ref.trace[:, 2] & 3))
    assert st["status"] == 0, st
    assert np.array_equal(tr[:, :2], ref.trace[:, :2]), "step schedules differ under replay"
    err = rel_l2(A, ref.A[0])
    ap_err = max(rel_l2(Ap[c], ref.Ap[0, c]) for c in range(Ap.shape[0]) if np.any(ref.Ap[0, c]))
    print(dict(N=N, cta=cta, attempts=st["attempts"], field_err=err, ap_err=ap_err))
    assert np.array_equal(sm, ref.stepmods), "stepmods record differs"
    assert err <= FIELD_TOL, err
    assert ap_err <= FIELD_TOL, ap_err


def test_reference_kernels_batch_shares_one_schedule(oracle, refmex):
    """B = 2 pulses in one call: one schedule (flags OR-ed over the batch), per-pulse G rows."""
    win, si, E = make_case(N=1024, length=0.2e-3, power=1.5, B=2)
    G2 = np.stack([si.G, si.G[::-1].copy()])
    ref = refmex.run(E, si.alpha, G2, si.beta, w0=si.w0, bdiffw0=si.bdiffw0, h=si.h,
                     n_steps=si.n_steps, dt=si.dt, max_err=si.max_err, min_err=si.min_err, sel=si.sel)
    orc = oracle.run(np.asarray(E, np.complex64).astype(np.complex128), si.alpha, G2, si.beta,
                     w0=si.w0, bdiffw0=si.bdiffw0, h=si.h, n_steps=si.n_steps, dt=si.dt,
                     max_err=si.max_err, min_err=si.min_err, sel=si.sel, g_per_pulse=True,
                     shared_schedule=True, trace_cap=200000, forced=ref.trace[:, 2] & 3)
    assert np.array_equal(orc.trace[0][:, :2], ref.trace[:, :2])
    for b in range(2):
        err = rel_l2(ref.A[b], orc.A[b])
        print(dict(b=b, field_err=err))
        assert err <= FIELD_TOL, err


@pytest.mark.parametrize("N,length,power", CASES + [(16384, 0.05e-3, 2.0)])
def test_difference_is_the_reference_fft_drift(oracle, refmex, N, length, power):
    """Where the reference's kernels and the oracle differ.  On the full case's step
    schedule, three runs of each: full; linear only (G = 0); FFT only (G = 0, beta = 0,
    alpha = 1, so each accepted step is absorber, FFT, IFFT and 1/N).

    Measured on a GB300: the FFT-only runs differ as much as the full ones (2.2e-4,
    6.4e-4, 2.7e-4, 9.7e-5 against 1.6e-4, 5.3e-4, 2.2e-4, 7.9e-5), growing with the
    number of accepted steps at 2-3e-7 per forward+inverse pair: cuFFT's FP32
    twiddles leave each mode a small gain per round trip, which adds up linearly.
    The propagator's twiddles carry their exact-inverse correction and do not drift.
    The nonlinear change itself, A(full) - A(G = 0) (4-8 % of the field), agrees to
    at most 3.8 times that drift; a convention error in the drive (time origin,
    shock-term sign, G index) would put it at order one."""
    win, si, E = make_case(N=N, length=length, power=power)
    ref = _ref_run(refmex, si, E[0])
    dec = ref.trace[:, 2] & 3
    E64 = np.asarray(E[0], np.complex64).astype(np.complex128)
    kw = dict(w0=si.w0, bdiffw0=si.bdiffw0, h=si.h, n_steps=si.n_steps, dt=si.dt,
              max_err=si.max_err, min_err=si.min_err, sel=si.sel)

    def both(G, beta, alpha):
        r = refmex.run(E[0], alpha, G, beta, forced=dec, **kw)
        o = oracle.run(E64, alpha, G, beta, forced=dec, trace_cap=200000, **kw)
        assert np.array_equal(o.trace[0][:, :2], r.trace[:, :2])
        return r.A[0].astype(np.complex128), o.A[0]

    G0 = np.zeros_like(si.G)
    rf, of = both(si.G, si.beta, si.alpha)
    rl, ol = both(G0, si.beta, si.alpha)
    rt, ot = both(G0, np.zeros_like(si.beta), np.ones_like(si.alpha))
    e_full, e_lin, e_fft = rel_l2(rf, of), rel_l2(rl, ol), rel_l2(rt, ot)
    e_nl = rel_l2(rf - rl, of - ol)
    accepted = int(np.sum((ref.trace[:, 2] & 8) != 0))
    print(dict(N=N, accepted=accepted, err_full=e_full, err_linear=e_lin, err_fft_only=e_fft,
               err_nonlinear_change=e_nl, nl_change_rel=rel_l2(of, ol)))
    assert e_full <= FIELD_TOL
    assert e_full <= 1.5 * e_fft + 1e-5, "difference larger than the FFT drift explains"
    assert e_nl <= 8.0 * e_fft, "nonlinear change differs beyond the FFT drift"


# ---------------------------------------------------------------------------
# RK23: the reference's ode23/OPO_CUDA_ODE23.cu kernels (unshifted time, step
# doubling, FSAL, integer sel, truncated chunk count; one pulse per call)
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def refode23():
    from oracle import ref_mex
    ok, why = ref_mex.available(ref_mex.CUBIN_ODE23)
    if not ok:
        pytest.skip(why)
    return ref_mex


def _oracle_rk23(oracle, si, E, forced=None):
    N = E.shape[-1]
    E64 = np.asarray(E, np.complex64).astype(np.complex128)
    return oracle.run(E64, si.alpha, si.G, si.beta, w0=si.w0, bdiffw0=si.bdiffw0, h=si.h,
                      n_steps=si.n_steps, dt=si.dt, max_err=si.max_err, min_err=si.min_err,
                      sel=si.sel, method=oracle.RK23_MEX, time_mode=oracle.TIME_UNSHIFTED,
                      abc_mode=oracle.ABC_SOFT, chunk_mode=oracle.CHUNKS_TRUNC,
                      stepmods_limit=(N // 256) * 256, trace_cap=200000, forced=forced)


@pytest.mark.parametrize("N,length,power", [(1024, 0.2e-3, 2.0), (2048, 0.3e-3, 2.0), (8192, 0.2e-3, 1.0)])
def test_oracle_rk23_matches_reference_ode23_kernels(oracle, refode23, N, length, power):
    win, si, E = make_case(N=N, length=length, power=power)
    kw = dict(w0=si.w0, bdiffw0=si.bdiffw0, h=si.h, n_steps=si.n_steps, dt=si.dt,
              max_err=si.max_err, min_err=si.min_err, sel=si.sel)
    ref = refode23.run_ode23(E[0], si.alpha, si.G, si.beta, **kw)
    dec = ref.trace[:, 2] & 3
    orc = _oracle_rk23(oracle, si, E[0], forced=dec)
    assert np.array_equal(orc.trace[0][:, :2], ref.trace[:, :2]), "step schedules differ under replay"
    orc_own = _oracle_rk23(oracle, si, E[0])
    same_sched = len(orc_own.trace[0]) == len(ref.trace) and \
        np.array_equal(orc_own.trace[0][:, :2], ref.trace[:, :2])
    # FFT-only drift of the reference on the same schedule (G = 0, beta = 0, alpha = 1)
    rt = refode23.run_ode23(E[0], np.ones_like(si.alpha), np.zeros_like(si.G), np.zeros_like(si.beta),
                            forced=dec, **kw)
    ot = oracle.run(np.asarray(E[0], np.complex64).astype(np.complex128), np.ones_like(si.alpha),
                    np.zeros_like(si.G), np.zeros_like(si.beta), method=oracle.RK23_MEX,
                    time_mode=oracle.TIME_UNSHIFTED, abc_mode=oracle.ABC_SOFT,
                    chunk_mode=oracle.CHUNKS_TRUNC, forced=dec, trace_cap=200000, **kw)
    err = rel_l2(ref.A[0], orc.A[0])
    e_fft = rel_l2(rt.A[0], ot.A[0])
    nch = ref.Ap.shape[1]
    ap_orc = orc.Ap.reshape(-1, N)[:nch]
    ap_err = max(rel_l2(ref.Ap[0, c], ap_orc[c]) for c in range(nch) if np.any(ap_orc[c]))
    print(dict(N=N, attempts=ref.attempts, rejected=int(np.sum((ref.trace[:, 2] & 8) == 0)),
               field_err=err, fft_only_err=e_fft, ap_err=ap_err, oracle_own_schedule_equal=same_sched,
               ref_seconds=ref.seconds))
    assert np.array_equal(orc.stepmods.astype(np.float32), ref.stepmods), "stepmods record differs"
    assert err <= FIELD_TOL, err
    assert err <= 1.5 * e_fft + 1e-5, "difference larger than the FFT drift explains"


@pytest.mark.parametrize("N,cta", [(1024, 0), (8192, 4096)])
def test_propagator_rk23_matches_reference_ode23_kernels(refode23, N, cta):
    from optifax_gb300 import _native as nat
    from tests.test_parity_gpu import _gpu_pass
    win, si, E = make_case(N=N, length=0.2e-3, power=2.0)
    ref = refode23.run_ode23(E[0], si.alpha, si.G, si.beta, w0=si.w0, bdiffw0=si.bdiffw0, h=si.h,
                             n_steps=si.n_steps, dt=si.dt, max_err=si.max_err, min_err=si.min_err,
                             sel=si.sel)
    A, Ap, sm, tr, st = _gpu_pass(si, E[0], nat.RK23, nat.VARIANT_ODE23, cta,
                                  forced=(ref.trace[:, 2] & 3))
    assert st["status"] == 0, st
    assert np.array_equal(tr[:, :2], ref.trace[:, :2]), "step schedules differ under replay"
    err = rel_l2(A, ref.A[0])
    print(dict(N=N, cta=cta, attempts=st["attempts"], field_err=err))
    assert np.array_equal(sm, ref.stepmods), "stepmods record differs"
    assert err <= FIELD_TOL, err


# ---------------------------------------------------------------------------
# The other Heun MEX files: BATCH_OP (one shared G), NO_BC (unshifted time, no
# absorber), HARD_BC (unshifted time, zeroing absorber); int sel, truncated chunks
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("variant", [1, 2, 3])
def test_heun_variants_match_reference_kernels(oracle, variant):
    import dataclasses
    from oracle import ref_mex
    from optifax_gb300 import _native as nat
    from tests.test_parity_gpu import _gpu_pass, _oracle_pass
    ok, why = ref_mex.available(ref_mex.HEUN_CUBINS[variant])
    if not ok:
        pytest.skip(why)
    win, si, E = make_case(N=2048, length=0.2e-3, power=2.0)
    E64 = np.asarray(E[0], np.complex64).astype(np.complex128)
    kw = dict(w0=si.w0, bdiffw0=si.bdiffw0, h=si.h, n_steps=si.n_steps, dt=si.dt,
              max_err=si.max_err, min_err=si.min_err, sel=si.sel, variant=variant)
    ref = ref_mex.run(E[0], si.alpha, si.G, si.beta, **kw)
    dec = ref.trace[:, 2] & 3
    orc = _oracle_pass(oracle, si, E64, nat.HEUN, variant, forced=dec)
    own = _oracle_pass(oracle, si, E64, nat.HEUN, variant)
    assert np.array_equal(orc.trace[0][:, :2], ref.trace[:, :2]), "step schedules differ under replay"
    same_sched = len(own.trace[0]) == len(ref.trace) and np.array_equal(own.trace[0][:, :2], ref.trace[:, :2])
    A, Ap, sm, tr, st = _gpu_pass(si, E[0], nat.HEUN, variant, 0, forced=dec)
    assert st["status"] == 0, st
    assert np.array_equal(tr[:, :2], ref.trace[:, :2])
    # FFT-only drift of the reference on the same schedule
    lin0 = dataclasses.replace(si, G=np.zeros_like(si.G), beta=np.zeros_like(si.beta),
                               alpha=np.ones_like(si.alpha))
    rt = ref_mex.run(E[0], lin0.alpha, lin0.G, lin0.beta, forced=dec, **kw)
    ot = _oracle_pass(oracle, lin0, E64, nat.HEUN, variant, forced=dec)
    err = rel_l2(ref.A[0], orc.A[0])
    err_gpu = rel_l2(A, ref.A[0])
    e_fft = rel_l2(rt.A[0], ot.A[0])
    print(dict(variant=variant, attempts=ref.attempts, oracle_own_schedule_equal=same_sched,
               field_err=err, propagator_err=err_gpu, fft_only_err=e_fft))
    assert np.array_equal(orc.stepmods.astype(np.float32), ref.stepmods)
    assert np.array_equal(sm, ref.stepmods)
    assert err <= FIELD_TOL and err_gpu <= FIELD_TOL
    assert err <= 1.5 * e_fft + 1e-5, "difference larger than the FFT drift explains"
