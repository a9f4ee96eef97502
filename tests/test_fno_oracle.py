"""The surrogate network's FP64 oracle against central finite differences (CPU)."""
import numpy as np

from oracle import fno_oracle as fo


def test_oracle_gradients_match_finite_differences():
    from optifax_gb300.surrogate import init_params, N_PARAMS
    assert N_PARAMS == fo.N_PARAMS
    rng = np.random.default_rng(1)
    L, B = 128, 2
    p = init_params(3, spec_scale=8.0).astype(np.float64)
    x = rng.normal(size=(B, fo.CIN, L))
    t = rng.normal(size=(B, fo.COUT, L))
    loss, g, _ = fo.loss_and_grads(p, x, t, weights_bf16=False)
    idx = [fo.OFF_P + 3, fo.OFF_PB + 5,
           fo.OFF_L0 + 7, fo.OFF_L0 + 2 * 64 * 32 * 2 + 33,            # spectral weights, layer 0
           fo.OFF_L0 + fo.LAYER_WS + 100,                            # pointwise weight, layer 0
           fo.OFF_L0 + fo.LAYER_WS + 64 * 64 + 9,                    # bias, layer 0
           fo.OFF_L0 + 2 * fo.LAYER_SIZE + 12345,                    # spectral weight, layer 2
           fo.OFF_L0 + 3 * fo.LAYER_SIZE + fo.LAYER_WS + 77,         # pointwise weight, layer 3
           fo.OFF_Q + 70, fo.OFF_QB + 2]
    for i in idx:
        e = 1e-6 * max(1.0, abs(p[i]))
        pp, pm = p.copy(), p.copy()
        pp[i] += e
        pm[i] -= e
        lp = fo.loss_and_grads(pp, x, t, weights_bf16=False)[0]
        lm = fo.loss_and_grads(pm, x, t, weights_bf16=False)[0]
        fd = (lp - lm) / (2 * e)
        assert abs(fd - g[i]) <= 1e-5 * max(1e-6, abs(fd)) + 1e-9, (i, fd, g[i])
