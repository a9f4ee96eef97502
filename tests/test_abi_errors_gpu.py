"""The C ABI rejects bad arguments with a status code and a message, never an abort
(include/optifax.h).  Marked gpu: a handle needs a device.

The reference's gateway checks only its argument count (OPO_mex_BATCH.cpp:38-40)
and misreads anything else; here every entry point validates before it touches
the device.  Every device pointer below is NULL (or, where a check needs a
non-NULL value, the pulse's own inputs stay NULL), so that no case can reach a
launch even if the check under test did not fire: the per-pulse validation
rejects NULL inputs before any device work.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

INVALID, UNSUPPORTED = 1, 2
FAKE = 16          # a non-NULL value for pointers the library only tests for NULL here


@pytest.fixture(scope="module")
def ctx():
    from optifax_gb300 import solver
    return solver.context(0)


def _pulse(**kw):
    from optifax_gb300 import _native as nat
    p = nat.OptifaxPulse()
    p.n_points, p.n_steps = 1024, 100
    p.w0, p.h, p.dt, p.bdiffw0 = 1.8e15, 1e-7, 7.3e-16, 1.0
    p.max_err, p.min_err, p.sel = 2.5e-3, 1.25e-4, 25.0
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _err(ctx):
    return ctx.lib.optifax_last_error(ctx.handle).decode()


@pytest.mark.parametrize("pulse_kw,call_kw,word", [
    ({}, dict(method=2), "method"),
    ({}, dict(variant=17), "variant"),
    ({}, dict(method=1, variant=5), "NEE"),
    ({}, dict(cta_points=1000), "cta_points"),
    (dict(n_points=1000), {}, "n_points"),
    (dict(n_points=131072), {}, "n_points"),
    (dict(n_steps=0), {}, "n_steps"),
    (dict(sel=0.5), {}, "sel"),
    (dict(h=0.0), {}, "positive"),
    ({}, {}, "required"),                       # E_in, A_out, alpha, beta, G are NULL
])
def test_propagate_rejects(ctx, pulse_kw, call_kw, word):
    args = dict(method=0, variant=0, cta_points=0)
    args.update(call_kw)
    arr = (type(_pulse()) * 1)(_pulse(**pulse_kw))
    rc = ctx.lib.optifax_propagate(ctx.handle, arr, 1, args["method"], args["variant"], args["cta_points"],
                                   None, None)
    assert rc == INVALID, (rc, _err(ctx))
    assert word in _err(ctx)


def test_propagate_rejects_empty_batches(ctx):
    assert ctx.lib.optifax_propagate(ctx.handle, None, 1, 0, 0, 0, None, None) == INVALID
    arr = (type(_pulse()) * 1)(_pulse())
    assert ctx.lib.optifax_propagate(ctx.handle, arr, 0, 0, 0, 0, None, None) == INVALID


def test_opo_run_rejects(ctx):
    from optifax_gb300 import opo
    lib = ctx.lib
    lib.optifax_opo_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(opo.OptifaxOpo), ctypes.c_int32,
                                    ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    assert lib.optifax_opo_run(ctx.handle, None, 1, 0, 0, None, None) == INVALID

    def run(**kw):
        cv = opo.OptifaxOpo()
        cv.pass_ = _pulse()
        cv.feedback, cv.pump, cv.n_trips = FAKE, FAKE, 3
        for k, v in kw.items():
            setattr(cv, k, v)
        return lib.optifax_opo_run(ctx.handle, (opo.OptifaxOpo * 1)(cv), 1, 0, 0, None, None)

    assert run(feedback=None) == INVALID and "feedback" in _err(ctx)
    assert run(n_trips=0) == INVALID and "n_trips" in _err(ctx)
    assert run(n_tally=5) == INVALID and "n_tally" in _err(ctx)
    assert run(steady_tally=4) == INVALID and "steady" in _err(ctx)
    assert run() == INVALID and "required" in _err(ctx)       # the pass's own inputs are NULL


def test_mex_batch_rejects(ctx):
    lib = ctx.lib

    def call(variant=0, n_pulses=1, ap_chunks=4, Ap_out=FAKE, sm_out=FAKE):
        return lib.optifax_opo_mex_batch(ctx.handle, None, None, None, 1.8e15, 1.0, 1e-7, 100, 7.3e-16, None,
                                         2.5e-3, 1.25e-4, 25.0, None, None, 1024, n_pulses, ap_chunks, variant,
                                         None, Ap_out, sm_out, None)

    assert call(variant=17) == INVALID and "variant" in _err(ctx)
    assert call(n_pulses=0) == INVALID and "n_pulses" in _err(ctx)
    assert call(Ap_out=None) == INVALID and "Ap_out" in _err(ctx)
    assert call(ap_chunks=2) == INVALID and "chunks" in _err(ctx)        # 100 steps / sel 25 = 4 chunks
    assert call() == INVALID and "required" in _err(ctx)                 # E and the tables are NULL


def test_gnlse_rejects(ctx):
    from optifax_gb300 import _native as nat
    lib = ctx.lib
    assert lib.optifax_gnlse(ctx.handle, None, 1, None) == INVALID

    def call(**kw):
        p = nat.OptifaxGnlsePulse()
        p.n_points, p.n_saves = 1024, 3
        p.gamma, p.dT, p.length, p.rtol, p.atol = 0.11, 2e-15, 0.01, 1e-5, 1e-12
        for k, v in kw.items():
            setattr(p, k, v)
        return lib.optifax_gnlse(ctx.handle, (nat.OptifaxGnlsePulse * 1)(p), 1, None)

    assert call(n_points=1000) == UNSUPPORTED and "n_points" in _err(ctx)
    assert call(n_saves=1) == INVALID
    assert call() == INVALID and "pulse 0" in _err(ctx)                   # A, B, W and outputs are NULL


def test_status_strings(ctx):
    lib = ctx.lib
    assert lib.optifax_status_string(INVALID).decode() == "invalid argument"
    assert lib.optifax_status_string(UNSUPPORTED).decode() == "unsupported configuration"
