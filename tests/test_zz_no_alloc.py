"""The allocation-free crystal pass (optifax_propagate_noalloc) against the
allocating entry point (optifax_propagate).  Marked gpu.

Callers that cannot allocate device memory while they run -- a solver inside a
MATLAB MEX function, whose device memory belongs to MATLAB's gpuArray manager,
an application that hands all device memory to its own caching allocator, or a
latency-critical loop that cannot let cudaMalloc/cudaFree synchronise the
device -- use optifax_propagate_noalloc, which keeps its working memory in a
fixed static device array.  Two calls in a row must each reproduce the
allocating entry point's output within the parity tolerance (1e-4 rel-L2),
which also shows that the second call is not disturbed by what the first left
in the shared array.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest
import torch

from tests._cases import make_case, rel_l2

pytestmark = pytest.mark.gpu


def _pulse_struct(nat, E, out, al, be, G, si):
    d = nat.OptifaxPulse()
    d.n_points, d.n_steps = E.numel(), si.n_steps
    d.E_in, d.A_out = E.data_ptr(), out.data_ptr()
    d.alpha, d.beta, d.G = al.data_ptr(), be.data_ptr(), G.data_ptr()
    d.w0, d.h, d.bdiffw0, d.dt = si.w0, si.h, si.bdiffw0, si.dt
    d.max_err, d.min_err, d.sel = si.max_err, si.min_err, si.sel
    return d


@pytest.mark.parametrize("N", [16384, 8192])
def test_noalloc_matches_allocating_entry(N):
    from optifax_gb300 import _native as nat
    from optifax_gb300 import solver as sv
    win, si, E = make_case(N=N, length=0.1e-3, power=2.0)
    dev = torch.device("cuda:0")
    Et = torch.from_numpy(E[0].astype(np.complex64)).to(dev)
    al = torch.from_numpy(si.alpha).to(dev)
    be = torch.from_numpy(si.beta).to(dev)
    G = torch.from_numpy(si.G).to(dev)
    spec = sv.PulseSpec(E=Et, alpha=al, beta=be, G=G, w0=si.w0, bdiffw0=si.bdiffw0, h=si.h, dt=si.dt,
                        max_err=si.max_err, min_err=si.min_err, sel=si.sel, n_steps=si.n_steps)
    outs, _ = sv.propagate([spec], method=nat.HEUN, variant=nat.VARIANT_BATCH_XTAL, cta_points=4096)
    torch.cuda.synchronize()
    ref = outs[0].cpu().numpy()
    lib = nat.load()
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        out = torch.zeros_like(Et)
        stats = torch.zeros((1, nat.STATS_BYTES // 4), dtype=torch.int32, device=dev)
        d = _pulse_struct(nat, Et, out, al, be, G, si)
        rc = lib.optifax_propagate_noalloc(ctypes.byref(d), nat.VARIANT_BATCH_XTAL, stats.data_ptr(), stream)
        assert rc == 0, rc
        torch.cuda.synchronize()
        st = sv.decode_stats(stats)[0]
        assert st["status"] == 0 and st["attempts"] > 0
        assert rel_l2(out.cpu().numpy(), ref) <= 1e-4, (call, rel_l2(out.cpu().numpy(), ref))


def test_noalloc_rejects_sizes_beyond_maximum():
    from optifax_gb300 import _native as nat
    lib = nat.load()
    d = nat.OptifaxPulse()
    d.n_points = 32768
    assert lib.optifax_propagate_noalloc(ctypes.byref(d), 0, None, None) == 2   # OPTIFAX_ERR_UNSUPPORTED
