"""FP64 numpy restatement of the crystal-pass surrogate network (forward, loss, backward).

TEST INFRASTRUCTURE ONLY: the oracle for the GPU kernels in
optifax_gb300/csrc/ofx_fno.cu.  Only tests/ may import it.  The network has no
counterpart in the reference (OptiFax has no learned component), so this file
restates the architecture the GPU code implements, with the same parameter
layout, using numpy's FFT for the spectral transforms and hand-written reverse
mode for the gradients:

    h0 = P x + p
    z_l = irfft(pad(W_l * rfft(h_l)[:32])) + Wp_l h_l + b_l,  h_{l+1} = gelu(z_l) (l < 3), h_4 = z_3
    y = x[:4] + Q h_4 + q,   loss = mean((y - target)^2)

Gradients use the real-pair convention g_z = dL/dRe z + i dL/dIm z, under which
T = S W gives g_S = g_T conj(W) and g_W = conj(S) g_T.
"""
from __future__ import annotations

import math

import numpy as np

W, MODES, NLAYER, CIN, COUT = 64, 32, 4, 6, 4
LAYER_WS = W * W * MODES * 2
LAYER_SIZE = LAYER_WS + W * W + W
OFF_P = 0
OFF_PB = OFF_P + W * CIN
OFF_L0 = OFF_PB + W
OFF_Q = OFF_L0 + NLAYER * LAYER_SIZE
OFF_QB = OFF_Q + COUT * W
N_PARAMS = OFF_QB + COUT


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round FP32 values to the nearest BF16 (ties to even), returned as float64."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params: np.ndarray, weights_bf16: bool = True) -> dict:
    """Split the flat vector; weight matrices rounded to BF16 as the kernels use them
    (biases stay FP32)."""
    p = np.asarray(params, dtype=np.float64)
    rw = (lambda a: bf16_round(a)) if weights_bf16 else (lambda a: a)
    out = {"P": rw(p[OFF_P:OFF_PB]).reshape(W, CIN), "p": p[OFF_PB:OFF_L0].copy(), "layers": []}
    for l in range(NLAYER):
        o = OFF_L0 + l * LAYER_SIZE
        ws = rw(p[o:o + LAYER_WS]).reshape(W, W, MODES, 2)
        wp = rw(p[o + LAYER_WS:o + LAYER_WS + W * W]).reshape(W, W)
        b = p[o + LAYER_WS + W * W:o + LAYER_SIZE].copy()
        out["layers"].append((ws[..., 0] + 1j * ws[..., 1], wp, b))
    out["Q"] = rw(p[OFF_Q:OFF_QB]).reshape(COUT, W)
    out["q"] = p[OFF_QB:].copy()
    return out


def pack_grads(g: dict) -> np.ndarray:
    flat = np.zeros(N_PARAMS)
    flat[OFF_P:OFF_PB] = g["P"].ravel()
    flat[OFF_PB:OFF_L0] = g["p"]
    for l, (gws, gwp, gb) in enumerate(g["layers"]):
        o = OFF_L0 + l * LAYER_SIZE
        flat[o:o + LAYER_WS] = np.stack([gws.real, gws.imag], axis=-1).ravel()
        flat[o + LAYER_WS:o + LAYER_WS + W * W] = gwp.ravel()
        flat[o + LAYER_WS + W * W:o + LAYER_SIZE] = gb
    flat[OFF_Q:OFF_QB] = g["Q"].ravel()
    flat[OFF_QB:] = g["q"]
    return flat


def _erf(a):
    return np.vectorize(math.erf)(a)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_d(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def _spec(h):
    return np.fft.fft(h, axis=-1)[..., :MODES]


def _ispec(T, L):
    full = np.zeros(T.shape[:-1] + (L // 2 + 1,), dtype=np.complex128)
    full[..., :MODES] = T
    return np.fft.irfft(full, n=L, axis=-1)


def forward(params, x, weights_bf16=True):
    """x (B, 6, L) -> (y (B, 4, L), cache)."""
    w = unpack(params, weights_bf16)
    x = np.asarray(x, dtype=np.float64)
    L = x.shape[-1]
    h = np.einsum("ci,bix->bcx", w["P"], x) + w["p"][None, :, None]
    cache = {"x": x, "h": [h], "z": [], "S": [], "w": w}
    for l, (ws, wp, b) in enumerate(w["layers"]):
        S = _spec(h)
        T = np.einsum("bcm,com->bom", S, ws)
        z = _ispec(T, L) + np.einsum("oc,bcx->box", wp, h) + b[None, :, None]
        cache["S"].append(S)
        cache["z"].append(z)
        h = gelu(z) if l < NLAYER - 1 else z
        cache["h"].append(h)
    y = x[:, :COUT] + np.einsum("jc,bcx->bjx", w["Q"], h) + w["q"][None, :, None]
    return y, cache


def loss_and_grads(params, x, target, weights_bf16=True, sample_w=None):
    """(loss, flat gradient vector, y); loss = sum_b w_b sum (y_b - t_b)^2 / y.size."""
    y, c = forward(params, x, weights_bf16)
    w = c["w"]
    t = np.asarray(target, dtype=np.float64)
    n = y.size
    sw = np.ones(y.shape[0]) if sample_w is None else np.asarray(sample_w, dtype=np.float64)
    loss = float(np.sum(sw[:, None, None] * (y - t) ** 2) / n)
    dy = 2.0 * sw[:, None, None] * (y - t) / n
    g = {"Q": np.einsum("bjx,bcx->jc", dy, c["h"][NLAYER]), "q": dy.sum(axis=(0, 2)), "layers": [None] * NLAYER}
    dh = np.einsum("jc,bjx->bcx", w["Q"], dy)
    L = y.shape[-1]
    for l in range(NLAYER - 1, -1, -1):
        ws, wp, b = w["layers"][l]
        z = c["z"][l]
        dz = dh * gelu_d(z) if l < NLAYER - 1 else dh
        hl = c["h"][l]
        gb = dz.sum(axis=(0, 2))
        gwp = np.einsum("box,bcx->oc", dz, hl)
        dh_pw = np.einsum("oc,box->bcx", wp, dz)
        cm = np.full(MODES, 2.0)
        cm[0] = 1.0
        gT = np.fft.fft(dz, axis=-1)[..., :MODES] * cm / L
        gT[..., 0] = gT[..., 0].real
        S = c["S"][l]
        gws = np.einsum("bcm,bom->com", np.conj(S), gT)
        gS = np.einsum("bom,com->bcm", gT, np.conj(ws))
        full = np.zeros(gS.shape[:-1] + (L,), dtype=np.complex128)
        full[..., :MODES] = gS
        dh_spec = np.real(np.fft.ifft(full, axis=-1) * L)
        g["layers"][l] = (gws, gwp, gb)
        dh = dh_pw + dh_spec
    g["P"] = np.einsum("bcx,bix->ci", dh, c["x"])
    g["p"] = dh.sum(axis=(0, 2))
    return loss, pack_grads(g), y

