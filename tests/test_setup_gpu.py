"""Device-side setup precompute against the host (NumPy) precompute.  Marked gpu."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_device_setup_matches_host():
    from optifax_gb300 import sweep
    insts = [sweep.Instance(4096, 1.0e-3, 30e-6, 2.0, 200e-15, 11),
             sweep.Instance(8192, 0.6e-3, 28.7e-6, 0.7, 120e-15, 12),
             sweep.Instance(2 ** 16, 2.0e-3, 31.3e-6, 3.0, 290e-15, 13),
             sweep.Instance(4096, 0.8e-3, ("linear", 28e-6, 32e-6), 1.5, 150e-15, 14)]
    dev_specs = sweep.build_specs_device(insts)
    host_specs = sweep.to_specs([sweep.build_inputs(i) for i in insts])
    for d, h in zip(dev_specs, host_specs):
        assert d.n_steps == h.n_steps and d.w0 == h.w0 and d.bdiffw0 == h.bdiffw0 and d.sel == h.sel
        assert torch.equal(d.alpha, h.alpha)
        assert torch.equal(d.G, h.G)
        bd, bh = d.beta.cpu().numpy(), h.beta.cpu().numpy()
        assert np.abs(bd - bh).max() <= 1e-6 * np.abs(bh).max()
        ed, eh = d.E.cpu().numpy().astype(np.complex128), h.E.cpu().numpy().astype(np.complex128)
        assert np.linalg.norm(ed - eh) / np.linalg.norm(eh) <= 1e-6
