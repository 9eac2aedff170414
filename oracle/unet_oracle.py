"""CPU oracle for the learned preconditioner's network: PyTorch FP64 autograd on the CPU.

TEST INFRASTRUCTURE ONLY (tests and smoke checks import it; the product never does).
The network has no counterpart in the reference; this restates the architecture the GPU
kernels implement, independently, with torch.nn.functional:

    e1 = relu(conv3x3(x0, 2->32))              x0 = (scaled residual, diagonal feature)
    e2 = relu(conv3x3(avgpool2(e1), 32->64))
    e3 = relu(conv3x3(avgpool2(e2), 64->128))
    b  = relu(conv3x3(avgpool2(e3), 128->128))
    c3 = relu(conv1x1(up2(b) + e3, 128->64))
    c2 = relu(conv3x3(up2(c3) + e2, 64->32))
    c1 = relu(conv3x3(up2(c2) + e1, 32->32))
    out = conv1x1(c1, 32->1)

with up2 = nearest-neighbour upsampling, zero padding, flat parameters per layer
[weights (cout, kh*k+kw, cin), bias (cout)], and mean-squared-error loss.

emulate_bf16=True rounds every stored tensor to BF16 where the GPU kernels store BF16:
weights, the packed input, every activation (the output stays unrounded) in the forward pass,
and the gradient of every stored tensor in the backward pass (rounding treated as the identity
for differentiation). The result then differs from the kernels only by FP32 accumulation order.
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as Fn

LAYERS = [  # cin, cout, k, relu
    (2, 32, 3, True), (32, 64, 3, True), (64, 128, 3, True), (128, 128, 3, True),
    (128, 64, 1, True), (64, 32, 3, True), (32, 32, 3, True), (32, 1, 1, False),
]


def _bf16(x):
    return x.to(torch.bfloat16).to(torch.float64)


class _Store(torch.autograd.Function):
    """Forward: round to BF16 (optional); backward: round the incoming gradient to BF16."""

    @staticmethod
    def forward(ctx, x, round_fwd):
        return _bf16(x) if round_fwd else x.clone()

    @staticmethod
    def backward(ctx, g):
        return _bf16(g), None


def _unpack(params):
    p = torch.as_tensor(np.asarray(params, np.float64))
    out, o = [], 0
    for ci, co, k, _ in LAYERS:
        n = co * k * k * ci
        w = p[o:o + n].reshape(co, k, k, ci).permute(0, 3, 1, 2).contiguous()
        o += n
        b = p[o:o + co].clone()
        o += co
        out.append((w, b))
    return out


def _net(wb, x0, emulate):
    def st(t, round_fwd=True):
        return _Store.apply(t, round_fwd) if emulate else t

    def conv(i, x):
        w, b = wb[i]
        ci, co, k, relu = LAYERS[i]
        y = Fn.conv2d(x, w, b, padding=k // 2)
        return torch.relu(y) if relu else y

    def up(t):
        return t.repeat_interleave(2, dim=2).repeat_interleave(2, dim=3)

    e1 = st(conv(0, x0))
    p1 = st(Fn.avg_pool2d(e1, 2))
    e2 = st(conv(1, p1))
    p2 = st(Fn.avg_pool2d(e2, 2))
    e3 = st(conv(2, p2))
    p3 = st(Fn.avg_pool2d(e3, 2))
    b = st(conv(3, p3))
    u3 = st(up(b) + e3)
    c3 = st(conv(4, u3))
    u2 = st(up(c3) + e2)
    c2 = st(conv(5, u2))
    u1 = st(up(c2) + e1)
    c1 = st(conv(6, u1))
    out = st(conv(7, c1), round_fwd=False)
    return out[:, 0]


def _prepare(params, x, f, emulate, requires_grad):
    wb = _unpack(params)
    if emulate:
        wb = [(_bf16(w), b) for w, b in wb]
    leaves = []
    for w, b in wb:
        w.requires_grad_(requires_grad)
        b.requires_grad_(requires_grad)
        leaves += [w, b]
    x = torch.as_tensor(np.asarray(x, np.float64))
    f = torch.as_tensor(np.asarray(f, np.float64))
    x0 = torch.stack([x, f], dim=1)
    if emulate:
        x0 = _bf16(x0)
    return wb, leaves, x0


def forward(params, x, f, emulate_bf16=True):
    """Network output (B, H, W) float64 for inputs x, f of shape (B, H, W)."""
    wb, _, x0 = _prepare(params, x, f, emulate_bf16, False)
    with torch.no_grad():
        return _net(wb, x0, emulate_bf16).numpy()


def loss_and_grads(params, x, f, tgt, emulate_bf16=True):
    """(mean squared error, flat gradient in the parameter layout) in float64."""
    wb, leaves, x0 = _prepare(params, x, f, emulate_bf16, True)
    out = _net(wb, x0, emulate_bf16)
    t = torch.as_tensor(np.asarray(tgt, np.float64))
    loss = torch.mean((out - t) ** 2)
    loss.backward()
    g = []
    for w, b in wb:
        g.append(w.grad.permute(0, 2, 3, 1).reshape(-1))
        g.append(b.grad.reshape(-1))
    return float(loss.detach()), torch.cat(g).numpy()
