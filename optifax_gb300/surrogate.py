"""Fourier-neural-operator surrogate of the crystal pass (BF16 tensor-core kernels).

``FNO`` wraps the optifax_fno_* C ABI (forward, backward, AdamW on the GPU; the
network is described in optifax_gb300/csrc/ofx_fno.cu).  The rest of this module
maps OPO fields to network channels and back.  The reference has no learned
component; this is new.

Field encoding (``Encoder``): the crystal-input and crystal-output spectra of a
2^14-point pass (natural FFT order of the fftshifted field) are cropped to
``n_bins`` consecutive frequency bins starting at ``f_lo``.  Channels 0/1 hold the
pump band (frequencies at or above ``f_split``) scaled by the fixed pump scale,
channels 2/3 the signal band (below ``f_split``) scaled by the input signal's own
RMS ``sigma``; channel 4 is the constant log10(sigma / pump scale), so the
network sees amplitude and shape separately (the small-signal map is linear),
and channel 5 the bin coordinate j / n_bins (the layers are otherwise
translation-equivariant along the bins).
The output uses the same scales, so an output decodes with the input's sigma.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
from typing import Optional

import numpy as np
import torch

from . import _native as nat

W, MODES, NLAYER, CIN, COUT = 64, 32, 4, 6, 4
LAYER_WS = W * W * MODES * 2
LAYER_SIZE = LAYER_WS + W * W + W
OFF_P, OFF_PB = 0, W * CIN
OFF_L0 = OFF_PB + W
OFF_Q = OFF_L0 + NLAYER * LAYER_SIZE
OFF_QB = OFF_Q + COUT * W
N_PARAMS = OFF_QB + COUT


def init_params(seed: int = 0, spec_scale: float = 1.0) -> np.ndarray:
    """Seeded initial parameters: uniform fan-in scaling, small projection (the
    residual path starts near the identity)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, dtype=np.float32)
    p[OFF_P:OFF_PB] = rng.uniform(-1, 1, W * CIN) / math.sqrt(CIN)
    for l in range(NLAYER):
        o = OFF_L0 + l * LAYER_SIZE
        p[o:o + LAYER_WS] = rng.uniform(-1, 1, LAYER_WS) * spec_scale / (W * math.sqrt(2.0))
        p[o + LAYER_WS:o + LAYER_WS + W * W] = rng.uniform(-1, 1, W * W) / math.sqrt(W)
    p[OFF_Q:OFF_QB] = rng.uniform(-1, 1, COUT * W) * 0.1 / math.sqrt(W)
    return p


def pretrained(name: str = "fno_env_spopo"):
    """(FP32 parameter vector, training record) of a network shipped in
    optifax_gb300/data: ``fno_env_spopo`` is trained on 20,480 pairs of 5 mm crystal
    passes of the 2^14-point SPOPO cavity generated by the solver (envelope
    representation, phase-aligned targets; the record names the command)."""
    import json
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
    params = np.load(os.path.join(here, name + ".npy")).astype(np.float32)
    with open(os.path.join(here, name + ".json")) as f:
        meta = json.load(f)
    if params.size != N_PARAMS:
        raise ValueError(f"{name}: {params.size} parameters, the network has {N_PARAMS}")
    return params, meta


class FNO:
    """One network on one device: n_bins frequency bins, up to max_batch samples per call."""

    def __init__(self, n_bins: int = 4096, max_batch: int = 32, device: int = 0, params=None, seed: int = 0):
        self.lib = nat.load()
        if self.lib.optifax_fno_param_count() != N_PARAMS:
            raise RuntimeError("parameter layout mismatch between library and host code")
        self.n_bins, self.max_batch, self.device = n_bins, max_batch, device
        self.dev = torch.device(f"cuda:{device}")
        h = ctypes.c_void_p()
        nat.check(self.lib.optifax_fno_create(ctypes.byref(h), n_bins, max_batch, device), None, "optifax_fno_create")
        self.h = h
        self.step = 0
        self.loss_dev = torch.zeros(1, dtype=torch.float32, device=self.dev)
        self.set_params(init_params(seed) if params is None else params)

    def _s(self, stream):
        return int((stream or torch.cuda.current_stream(self.dev)).cuda_stream)

    def set_params(self, params, stream=None):
        t = torch.as_tensor(np.asarray(params, dtype=np.float32) if not isinstance(params, torch.Tensor) else params,
                            dtype=torch.float32).to(self.dev).contiguous()
        nat.check(self.lib.optifax_fno_set_params(self.h, t.data_ptr(), self._s(stream)), None, "fno_set_params")
        torch.cuda.synchronize(self.dev)
        self.step = 0

    def params(self, stream=None) -> torch.Tensor:
        out = torch.empty(N_PARAMS, dtype=torch.float32, device=self.dev)
        nat.check(self.lib.optifax_fno_get_params(self.h, out.data_ptr(), self._s(stream)), None, "fno_get_params")
        return out

    def _check_x(self, x, C):
        if x.dtype != torch.float32 or not x.is_cuda or x.dim() != 3 or x.shape[1] != C or x.shape[2] != self.n_bins:
            raise ValueError(f"expected CUDA float32 (B, {C}, {self.n_bins})")
        if x.shape[0] > self.max_batch:
            raise ValueError("batch larger than max_batch")
        return x.contiguous()

    def forward(self, x: torch.Tensor, stream=None) -> torch.Tensor:
        x = self._check_x(x, CIN)
        y = torch.empty((x.shape[0], COUT, self.n_bins), dtype=torch.float32, device=self.dev)
        nat.check(self.lib.optifax_fno_forward(self.h, x.data_ptr(), y.data_ptr(), x.shape[0], self._s(stream)),
                  None, "fno_forward")
        return y

    def backward(self, x: torch.Tensor, target: torch.Tensor, grads: Optional[torch.Tensor] = None,
                 sample_w: Optional[torch.Tensor] = None, stream=None):
        """Forward + backward of sum_b w_b |y_b - t_b|^2 / numel; returns the device loss
        tensor (1,) (grads copied if given)."""
        x = self._check_x(x, CIN)
        target = self._check_x(target, COUT)
        if sample_w is not None:
            sample_w = sample_w.to(torch.float32).contiguous()
            if sample_w.numel() != x.shape[0] or sample_w.device != self.dev:
                raise ValueError("sample_w must hold one weight per sample on the network's device")
        nat.check(self.lib.optifax_fno_backward(self.h, x.data_ptr(), target.data_ptr(),
                                                sample_w.data_ptr() if sample_w is not None else None, x.shape[0],
                                                self.loss_dev.data_ptr(),
                                                grads.data_ptr() if grads is not None else None, self._s(stream)),
                  None, "fno_backward")
        return self.loss_dev

    def set_grads(self, grads: torch.Tensor, stream=None):
        """Replace the gradients of the last backward (e.g. by their mean over ranks)."""
        if grads.dtype != torch.float32 or grads.numel() != N_PARAMS or grads.device != self.dev:
            raise ValueError("grads must be float32, one per parameter, on the network's device")
        nat.check(self.lib.optifax_fno_set_grads(self.h, grads.contiguous().data_ptr(), self._s(stream)), None,
                  "fno_set_grads")

    def adam(self, lr: float, betas=(0.9, 0.999), eps: float = 1e-8, weight_decay: float = 0.0, stream=None):
        self.step += 1
        nat.check(self.lib.optifax_fno_adam(self.h, float(lr), float(betas[0]), float(betas[1]), float(eps),
                                            float(weight_decay), self.step, self._s(stream)), None, "fno_adam")

    def close(self):
        if getattr(self, "h", None):
            self.lib.optifax_fno_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def data_parallel_step(net, x, target, lr: float, *, sample_w=None, weight_decay: float = 0.0, grads=None,
                       reduce=None):
    """One data-parallel training step: forward + backward on this rank's shard, the
    gradients averaged over the ranks (``reduce``, default dist.all_reduce_mean_),
    then AdamW on every rank with the same gradients, so the replicas stay
    identical.  With one rank this is the plain step.  Each rank's loss is normalised
    by its own shard, so equal shard sizes give exactly the full-batch gradient."""
    from . import dist
    reduce = reduce or dist.all_reduce_mean_
    world = (torch.distributed.get_world_size()
             if torch.distributed.is_available() and torch.distributed.is_initialized() else 1)
    if world == 1 and reduce is dist.all_reduce_mean_:
        loss = net.backward(x, target, sample_w=sample_w)
    else:
        if grads is None:
            grads = torch.empty(N_PARAMS, dtype=torch.float32, device=x.device)
        loss = net.backward(x, target, grads=grads, sample_w=sample_w)
        reduce(grads)
        net.set_grads(grads)
    net.adam(lr, weight_decay=weight_decay)
    return loss
