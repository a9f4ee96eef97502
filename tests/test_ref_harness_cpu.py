"""The reference-kernel harness (oracle/Makefile target `ref`) builds without a GPU:
the harness library exports its entry points and, where the reference source is
present, the five MEX kernel files compile unmodified into cubins."""
import os
import shutil
import subprocess

import pytest

ORACLE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle")


def test_reference_harness_builds_and_exports():
    if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("no CUDA toolkit")
    subprocess.run(["make", "-s", "-C", ORACLE, "ref"], check=True)
    lib = os.path.join(ORACLE, "_build", "libref_mex.so")
    assert os.path.exists(lib)
    if shutil.which("nm") is None:
        pytest.skip("no nm to list the exports")
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    for sym in ("refmex_run", "refmex_run_ode23", "refmex_last_error"):
        assert sym in out, sym
    from oracle import ref_mex
    cubins = ref_mex.HEUN_CUBINS + [ref_mex.CUBIN_ODE23]
    if any(os.path.exists(c) for c in cubins):      # the reference source was there: all five built
        for cubin in cubins:
            assert os.path.exists(cubin), cubin
