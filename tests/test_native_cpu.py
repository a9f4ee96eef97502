"""The C-ABI library builds, loads and exports every symbol include/optifax.h declares (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^\s*(?:int|int64_t|const char\s*\*)\s+(optifax_\w+)\s*\(", src, flags=re.M)
    return names


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ["optifax_create", "optifax_destroy", "optifax_opo_mex_batch", "optifax_propagate"]:
        assert n in names


def test_library_exports_all_declared_symbols():
    from optifax_gb300 import _native as nat
    from optifax_gb300 import build
    build.build()
    lib = ctypes.CDLL(build.LIB)
    for n in declared_functions():
        assert hasattr(lib, n), n
    assert set(nat.EXPORTS) <= set(declared_functions())


def test_status_strings_and_null_handle():
    from optifax_gb300 import _native as nat
    lib = nat.load()
    assert lib.optifax_status_string(0) == b"ok"
    assert lib.optifax_status_string(1) == b"invalid argument"
    assert lib.optifax_destroy(None) == 5
    assert lib.optifax_propagate(None, None, 0, 0, 0, 0, None, None) == 5
    assert lib.optifax_gnlse(None, None, 0, None) == 5
    g = ctypes.c_void_p()
    assert lib.optifax_propagate_graph(None, None, 0, 0, 0, 0, None, ctypes.byref(g)) == 5
    assert lib.optifax_graph_launch(None, None) == 1
    assert lib.optifax_graph_destroy(None) == 1
    assert lib.optifax_graph_kernels(None) == 0


def test_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from optifax_gb300 import _native as nat
    lib = nat.load()
    h = ctypes.c_void_p()
    assert lib.optifax_create(ctypes.byref(h), 0) == 3


def test_struct_layouts_match_ctypes(tmp_path):
    """The ctypes mirrors of the ABI structs have the C compiler's offsets and sizes."""
    import shutil
    import subprocess
    from optifax_gb300 import _native as nat
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"optifax_gnlse_pulse": nat.OptifaxGnlsePulse, "optifax_gnlse_stats": nat.OptifaxGnlseStats,
               "optifax_pulse": nat.OptifaxPulse, "optifax_setup": nat.OptifaxSetup}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "optifax.h"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, cls in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)


def test_stream_wrapper_passes_through_without_a_stream():
    """solver.on_stream leaves calls without a stream as they are (no CUDA use) and keeps
    the wrapped function's name, signature checks and errors."""
    import numpy as np
    from optifax_gb300 import solver, gnlse, opo, _native as nat
    calls = []

    @solver.on_stream
    def f(x, *, stream=None):
        calls.append(stream)
        return x + 1

    assert f(1) == 2 and calls == [None] and f.__name__ == "f"
    for fn in (solver.propagate, solver.opo_mex_batch, solver.propagate_fp64, opo.run_many, gnlse.propagate):
        assert fn.__wrapped__ is not None
    T = np.arange(-500, 500) * 1e-15
    ops = gnlse.fibre_operators(T, 0.0, 0.11, [-1e-26], 0.0, 0.0, 0.0)
    with pytest.raises(nat.OptifaxError):
        gnlse.propagate(ops, np.ones(1000), 0.01, 3)
