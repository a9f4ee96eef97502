"""Surrogate network kernels (BF16 tensor cores) against the FP64 oracle.  Marked gpu.

The GPU path rounds weights (as the oracle does) and also activations to BF16,
so outputs agree to a few 1e-3 and gradients to about 1e-2 (relative L2).
"""
import numpy as np
import pytest
import torch

from oracle import fno_oracle as fo

pytestmark = pytest.mark.gpu

Y_TOL = 2e-2
G_TOL = 5e-2


def _blocks():
    out = [("P", fo.OFF_P, fo.OFF_PB), ("p", fo.OFF_PB, fo.OFF_L0)]
    for l in range(fo.NLAYER):
        o = fo.OFF_L0 + l * fo.LAYER_SIZE
        out += [(f"Ws{l}", o, o + fo.LAYER_WS), (f"Wp{l}", o + fo.LAYER_WS, o + fo.LAYER_WS + 4096),
                (f"b{l}", o + fo.LAYER_WS + 4096, o + fo.LAYER_SIZE)]
    out += [("Q", fo.OFF_Q, fo.OFF_QB), ("q", fo.OFF_QB, fo.N_PARAMS)]
    return out


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("L,B", [(256, 3), (128, 1)])
def test_fno_forward_backward_match_oracle(L, B):
    from optifax_gb300.surrogate import FNO, init_params
    from optifax_gb300.gemm import tc_error
    rng = np.random.default_rng(L + B)
    p = init_params(3, spec_scale=8.0)
    x = rng.normal(size=(B, fo.CIN, L)).astype(np.float32)
    t = rng.normal(size=(B, fo.COUT, L)).astype(np.float32)
    net = FNO(n_bins=L, max_batch=4, params=p)
    dev = net.dev
    xg, tg = torch.from_numpy(x).to(dev), torch.from_numpy(t).to(dev)
    y = net.forward(xg).cpu().numpy()
    grads = torch.zeros(fo.N_PARAMS, dtype=torch.float32, device=dev)
    sw = rng.uniform(0.5, 2.0, size=B).astype(np.float32)
    loss = float(net.backward(xg, tg, grads, sample_w=torch.from_numpy(sw).to(dev)).item())
    g = grads.cpu().numpy()
    torch.cuda.synchronize()
    assert tc_error() == 0
    lref, gref, yref = fo.loss_and_grads(p, x, t, weights_bf16=True, sample_w=sw)
    assert _rel(y, yref) <= Y_TOL
    assert abs(loss - lref) <= Y_TOL * lref
    bad = {n: _rel(g[a:b], gref[a:b]) for n, a, b in _blocks() if _rel(g[a:b], gref[a:b]) > G_TOL}
    assert not bad, bad


def test_fno_adam_reduces_loss():
    from optifax_gb300.surrogate import FNO, init_params
    rng = np.random.default_rng(5)
    L, B = 256, 4
    net = FNO(n_bins=L, max_batch=B, params=init_params(1))
    x = torch.from_numpy(rng.normal(size=(B, 6, L)).astype(np.float32)).to(net.dev)
    tgt = x[:, :4] * 0.5 + 0.1
    l0 = float(net.backward(x, tgt.contiguous()).item())
    for _ in range(60):
        net.backward(x, tgt.contiguous())
        net.adam(3e-3)
    l1 = float(net.backward(x, tgt.contiguous()).item())
    assert l1 < 0.2 * l0, (l0, l1)


def test_fno_set_grads_feeds_adam():
    """set_grads replaces the gradients AdamW uses: two networks whose own backwards
    differ (split-K atomics make gradients differ in the last bits from run to run)
    take the identical step once given the same gradient vector; zero gradients leave
    the parameters as they are (no weight decay).  This is the data-parallel path."""
    from optifax_gb300.surrogate import FNO, N_PARAMS, init_params
    rng = np.random.default_rng(6)
    L, B = 256, 2
    p0 = init_params(2)
    a = FNO(n_bins=L, max_batch=B, params=p0)
    b = FNO(n_bins=L, max_batch=B, params=p0)
    c = FNO(n_bins=L, max_batch=B, params=p0)
    x = torch.from_numpy(rng.normal(size=(B, 6, L)).astype(np.float32)).to(a.dev)
    tgt = (x[:, :4] * 0.3).contiguous()
    g = torch.empty(N_PARAMS, dtype=torch.float32, device=a.dev)
    a.backward(x, tgt, grads=g)
    a.set_grads(g)
    a.adam(1e-3)
    b.backward(x, tgt)
    b.set_grads(g)
    b.adam(1e-3)
    assert torch.equal(a.params(), b.params())
    assert not torch.equal(a.params(), torch.as_tensor(p0, dtype=torch.float32, device=a.dev))
    c.backward(x, tgt)
    c.set_grads(torch.zeros(N_PARAMS, dtype=torch.float32, device=c.dev))
    before = c.params().clone()
    c.adam(1e-3)
    assert torch.equal(before, c.params())
