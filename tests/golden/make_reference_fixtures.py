"""Golden fixtures from the reference's own CUDA kernels (run on a GPU).

    python tests/golden/make_reference_fixtures.py [OUT_DIR]

Runs OptiFax's MEX kernels, compiled unmodified from the reference's sources into
oracle/_ref/*.cubin and driven as its MEX driver drives them (oracle/ref_mex.py), on
small seeded crystal passes (tests/_cases.make_case), and writes one compressed .npz
per case into OUT_DIR (default: this directory): the inputs exactly as the kernels
received them (FP32 field and arrays, the scalars), and the kernels' outputs (field,
stepmods, per-attempt trace, and the Ap snapshots for the 1024-point cases).
tests/test_golden_cpu.py checks the FP64 oracle against these files without a GPU.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# name: (method, variant, N, length [m], pump power [W]); variant 0 BATCH_XTAL,
# 2 NO_BC, 3 HARD_BC (Heun); RK23 runs the ODE23 kernels
CASES = {
    "heun_xtal_n1024": ("heun", 0, 1024, 0.2e-3, 2.0),
    "heun_xtal_n2048": ("heun", 0, 2048, 0.3e-3, 2.0),
    "heun_xtal_n4096": ("heun", 0, 4096, 0.2e-3, 3.0),
    "heun_nobc_n1024": ("heun", 2, 1024, 0.2e-3, 2.0),
    "heun_hardbc_n1024": ("heun", 3, 1024, 0.2e-3, 2.0),
    "rk23_n1024": ("rk23", 0, 1024, 0.2e-3, 2.0),
    "rk23_n2048": ("rk23", 0, 2048, 0.3e-3, 2.0),
}


def main(out_dir):
    from oracle import ref_mex
    from tests._cases import make_case
    os.makedirs(out_dir, exist_ok=True)
    for name, (method, variant, N, length, power) in CASES.items():
        win, si, E = make_case(N=N, length=length, power=power)
        kw = dict(w0=si.w0, bdiffw0=si.bdiffw0, h=si.h, n_steps=si.n_steps, dt=si.dt,
                  max_err=si.max_err, min_err=si.min_err, sel=si.sel)
        if method == "heun":
            r = ref_mex.run(E[0], si.alpha, si.G, si.beta, variant=variant, **kw)
        else:
            r = ref_mex.run_ode23(E[0], si.alpha, si.G, si.beta, **kw)
        extra = {"Ap": r.Ap[0]} if N == 1024 else {}
        np.savez_compressed(
            os.path.join(out_dir, name + ".npz"), method=method, variant=variant,
            E=np.asarray(E[0], np.complex64), alpha=np.asarray(si.alpha, np.float32),
            beta=np.asarray(si.beta, np.float32), G=np.asarray(si.G, np.float32),
            scalars=np.array([si.w0, si.bdiffw0, si.h, si.n_steps, si.dt, si.max_err, si.min_err, si.sel]),
            A=r.A[0], stepmods=r.stepmods, trace=r.trace, **extra)
        print(name, "attempts", r.attempts, "rejected", int(np.sum((r.trace[:, 2] & 8) == 0)))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__)))
