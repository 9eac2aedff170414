"""Learned preconditioner for the CG source inversion (no counterpart in the reference).

A 4-level convolutional U-Net on the source grid (276k parameters, BF16 on the tcgen05 tensor
cores with FP32 accumulation, kernels in csrc/unet.cu) maps a scaled Jacobi-preconditioned
residual to a correction over Jacobi:

    u = dinv * r,  s = rms(u),  f = log(dinv) - mean(log(dinv))
    M(r) = u + s * net(u / s, f)

It is trained on the GPU, by its own forward and backward kernels and Adam, on (residual,
correction) pairs taken from plain Jacobi-CG trajectories of the inversion over random lens
draws, and used inside flexible CG (lentils_fcg_solve) with the Jacobi direction as the
per-iteration fallback.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _native as N
from .gridding import _ptr

# (cin, cout, kernel size, relu, level) of the 8 convolutions, in parameter order
LAYERS = [
    (2, 32, 3, True, 0),
    (32, 64, 3, True, 1),
    (64, 128, 3, True, 2),
    (128, 128, 3, True, 3),
    (128, 64, 1, True, 2),
    (64, 32, 3, True, 1),
    (32, 32, 3, True, 0),
    (32, 1, 1, False, 0),
]


def param_count():
    return sum(co * k * k * ci + co for ci, co, k, _, _ in LAYERS)


def init_params(seed=0, out_scale=0.1):
    """He-normal weights, zero biases; the output layer scaled by `out_scale` so that a fresh
    network is a small perturbation of Jacobi."""
    rng = np.random.default_rng(seed)
    parts = []
    for li, (ci, co, k, _, _) in enumerate(LAYERS):
        std = math.sqrt(2.0 / (ci * k * k))
        if li == len(LAYERS) - 1:
            std *= out_scale
        parts.append(rng.normal(0.0, std, co * k * k * ci))
        parts.append(np.zeros(co))
    return np.concatenate(parts).astype(np.float32)


def unpack(params):
    """Flat parameters -> list of (weights [cout, k*k, cin], bias [cout]) arrays."""
    out, o = [], 0
    for ci, co, k, _, _ in LAYERS:
        n = co * k * k * ci
        w = np.asarray(params[o:o + n]).reshape(co, k * k, ci)
        o += n
        b = np.asarray(params[o:o + co])
        o += co
        out.append((w, b))
    return out


def features(dinv):
    """f = log(dinv) - mean(log(dinv)) on the GPU (same kernel the solver uses)."""
    d = dinv.contiguous().float()
    f = torch.empty_like(d)
    N.check(N.lib().lentils_unet_features(_ptr(d), _ptr(f), d.numel(),
                                          ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return f


def scaled_inputs(r, dinv, feat, e=None):
    """Network inputs (and the training target for a correction e) of the preconditioner form,
    batched over the leading dimension: (u / s, f, (e - u) / s)."""
    u = dinv * r
    s = torch.sqrt(torch.mean(u.double() ** 2, dim=(-2, -1), keepdim=True)).float()
    s = torch.where(s > 0, s, torch.ones_like(s))
    x = u / s
    f = feat.expand_as(x)
    if e is None:
        return x.contiguous(), f.contiguous()
    return x.contiguous(), f.contiguous(), ((e - u) / s).contiguous()


class UNet:
    """Device-resident network (lentils_unet_*): forward, gradients, Adam steps and the
    preconditioner application. Arrays are (B, H, W) float32 CUDA tensors."""

    def __init__(self, H, W, max_batch=32, params=None, seed=0):
        self.H, self.W, self.max_batch = int(H), int(W), int(max_batch)
        p = init_params(seed) if params is None else np.ascontiguousarray(params, np.float32)
        if p.size != param_count():
            raise ValueError(f"expected {param_count()} parameters, got {p.size}")
        self._h = ctypes.c_void_p()
        N.check(N.lib().lentils_unet_create(ctypes.byref(self._h), self.H, self.W,
                                            self.max_batch, p.ctypes.data, self._sp()))

    @staticmethod
    def _sp():
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h is not None and self._h.value:
            N.lib().lentils_unet_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, *arrs):
        B = arrs[0].shape[0]
        for a in arrs:
            if a.dtype != torch.float32 or not a.is_cuda or tuple(a.shape) != (B, self.H, self.W):
                raise ValueError("expected (B, H, W) float32 CUDA tensors")
        if not 1 <= B <= self.max_batch:
            raise ValueError(f"batch {B} outside 1..{self.max_batch}")
        return B

    def forward(self, x, f):
        x, f = x.contiguous(), f.contiguous()
        B = self._check(x, f)
        out = torch.empty_like(x)
        N.check(N.lib().lentils_unet_forward(self._h, _ptr(x), _ptr(f), _ptr(out), B, self._sp()))
        return out

    def gradients(self, x, f, tgt):
        """(flat FP32 gradient of the mean squared error, loss) without updating."""
        x, f, tgt = x.contiguous(), f.contiguous(), tgt.contiguous()
        B = self._check(x, f, tgt)
        g = np.empty(param_count(), np.float32)
        loss = ctypes.c_float()
        N.check(N.lib().lentils_unet_gradients(self._h, _ptr(x), _ptr(f), _ptr(tgt), B,
                                               g.ctypes.data, ctypes.byref(loss), self._sp()))
        return g, float(loss.value)

    def train_step(self, x, f, tgt, lr, loss_out=None):
        """One Adam step; loss_out (1-element float32 CUDA tensor) receives the batch loss."""
        B = self._check(x, f, tgt)
        N.check(N.lib().lentils_unet_train_step(self._h, _ptr(x), _ptr(f), _ptr(tgt), B,
                                                float(lr),
                                                _ptr(loss_out) if loss_out is not None else None,
                                                self._sp()))

    @property
    def params(self):
        p = np.empty(param_count(), np.float32)
        N.check(N.lib().lentils_unet_get_params(self._h, p.ctypes.data))
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        N.check(N.lib().lentils_unet_set_params(self._h, p.ctypes.data, self._sp()))
        torch.cuda.current_stream().synchronize()

    def precondition(self, r, dinv, feat):
        """z = M(r) for one (H, W) or flat residual."""
        r, dinv, feat = (t.contiguous().float() for t in (r, dinv, feat))
        z = torch.empty_like(r)
        N.check(N.lib().lentils_unet_precondition(self._h, _ptr(r), _ptr(dinv), _ptr(feat),
                                                  _ptr(z), self._sp()))
        return z

    def error_flag(self):
        f = ctypes.c_int()
        N.check(N.lib().lentils_unet_error_flag(self._h, ctypes.byref(f)))
        return f.value
