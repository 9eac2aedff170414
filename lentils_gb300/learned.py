"""Learned preconditioner for the CG source inversion (no counterpart in the reference).

A 4-level convolutional U-Net on the source grid (276k parameters, BF16 on the tcgen05 tensor
cores with FP32 accumulation, kernels in csrc/unet.cu) maps a scaled Jacobi-preconditioned
residual to the direction of the error it stands for:

    u = dinv * r,  s = rms(u),  f = log(dinv) - mean(log(dinv))
    M(r) = gamma * u + s * net(u / s, f),     net trained on e / rms(e), e = A^-1 r

Flexible CG takes the step length from a line search, so only the direction of M(r) matters;
gamma (default 0) mixes in the Jacobi direction.

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


def _rms(t):
    s = torch.sqrt(torch.mean(t.double() ** 2, dim=(-2, -1), keepdim=True)).float()
    return torch.where(s > 0, s, torch.ones_like(s))


def scaled_inputs(r, dinv, feat, e=None):
    """Network inputs (and the training target for a correction e) of the preconditioner form,
    batched over the leading dimension: (u / rms(u), f, e / rms(e))."""
    u = dinv * r
    x = u / _rms(u)
    f = feat.expand_as(x)
    if e is None:
        return x.contiguous(), f.contiguous()
    return x.contiguous(), f.contiguous(), (e / _rms(e)).contiguous()


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

    def backward(self, dout, lr=0.0, want_grad=False):
        """Backward pass from the most recent forward() for the output gradient dout (same
        shape); Adam step if lr > 0; returns the flat gradient if want_grad."""
        dout = dout.contiguous()
        B = self._check(dout)
        g = np.empty(param_count(), np.float32) if want_grad else None
        N.check(N.lib().lentils_unet_backward(self._h, _ptr(dout), B, float(lr),
                                              g.ctypes.data if want_grad else None, self._sp()))
        return g

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

    def set_gemm_form(self, form):
        """Convolution kernels (lentils_unet_set_gemm_form): 0 persistent TMA GEMMs with the
        first and output layers fused, 1 staged GEMMs, 2 per-tile TMA / pipelined GEMMs."""
        N.check(N.lib().lentils_unet_set_gemm_form(self._h, int(form)))

    def set_jacobi_weight(self, gamma):
        N.check(N.lib().lentils_unet_set_jacobi_weight(self._h, float(gamma)))

    def error_flag(self):
        f = ctypes.c_int()
        N.check(N.lib().lentils_unet_error_flag(self._h, ctypes.byref(f)))
        return f.value


# ------------------------------------------------------------------------------------------------
# Training data: (residual, correction) pairs from Jacobi-CG and Jacobi flexible-CG trajectories
# ------------------------------------------------------------------------------------------------
def lens_draw(rng, centre=(0.0, 0.0), jitter=0.05):
    """A PEMD + external shear drawn from the sweep priors: b in [0.8, 1.6], axis ratio q in
    [0.5, 0.95], slope gamma in [1.8, 2.3] (qh = (gamma - 1) / 2), shear strength in [0, 0.1];
    position angles uniform; centre jittered by +-jitter arcsec."""
    from .lens_models import ExternalPotential, GlobalLensModel, PowerLawEllipsoid
    b = rng.uniform(0.8, 1.6)
    q = rng.uniform(0.5, 0.95)
    gamma = rng.uniform(1.8, 2.3)
    th = rng.uniform(0.0, 180.0)
    ss = rng.uniform(0.0, 0.1)
    sa = rng.uniform(0.0, 180.0)
    x0, y0 = np.asarray(centre, float) + rng.uniform(-jitter, jitter, 2)
    return GlobalLensModel([
        PowerLawEllipsoid(z=0.5, b=b, th=th, f=q, x=x0, y=y0, rc=0.0, qh=0.5 * (gamma - 1.0)),
        ExternalPotential(z=0.5, x=x0, y=y0, ss=ss, sa=sa)])


def random_source(rng, source_space, nblobs=(1, 5)):
    """Sum of a few Gaussian blobs (widths 0.02-0.08 arcsec) inside the inner 60% of the
    source grid, x-major (nx, ny) float64."""
    sp = source_space
    xs = (sp.xmin + sp.dx * np.arange(sp.nx))[:, None]
    ys = (sp.ymin + sp.dy * np.arange(sp.ny))[None, :]
    hx, hy = 0.3 * (sp.xmax - sp.xmin), 0.3 * (sp.ymax - sp.ymin)
    cx, cy = 0.5 * (sp.xmin + sp.xmax), 0.5 * (sp.ymin + sp.ymax)
    s = np.zeros((sp.nx, sp.ny))
    for _ in range(rng.integers(nblobs[0], nblobs[1] + 1)):
        x0, y0 = cx + rng.uniform(-hx, hx), cy + rng.uniform(-hy, hy)
        w = rng.uniform(0.02, 0.08)
        s += rng.uniform(0.3, 1.0) * np.exp(-((xs - x0) ** 2 + (ys - y0) ** 2) / (2 * w * w))
    return s


def jacobi_cg_trajectory(inv, max_iter=8000, rtol=1e-6, check_every=50):
    """Plain Jacobi-preconditioned CG on inv's normal equations from x = 0 with the FP32
    operator (FP64-accumulated dot products), recording every iterate. Returns the iterates
    (K, n) float32 CUDA tensor, including x_0 = 0."""
    import ctypes as _ct
    n = inv.nsrc
    L = N.lib()
    xs = torch.zeros((max_iter + 1, n), dtype=torch.float32, device="cuda")
    b = inv.b.float()
    dinv = inv.inv_diag32
    bn = float(torch.linalg.vector_norm(inv.b))
    sp = _ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    x = torch.zeros(n, dtype=torch.float32, device="cuda")
    r = b.clone()
    z = dinv * r
    p = z.clone()
    ap = torch.empty_like(p)
    rz = torch.dot(r.double(), z.double())
    k = 0
    while k < max_iter:
        N.check(L.lentils_normal_op_apply(inv.handle, _ptr(p), _ptr(ap), sp))
        alpha = (rz / torch.dot(p.double(), ap.double())).float()
        x.add_(alpha * p)
        r.sub_(alpha * ap)
        k += 1
        xs[k] = x
        z = dinv * r
        rz_new = torch.dot(r.double(), z.double())
        p = z + (rz_new / rz).float() * p
        rz = rz_new
        if k % check_every == 0 and float(torch.linalg.vector_norm(r.double())) <= rtol * bn:
            break
    return xs[:k + 1]


def fcg_trajectory(inv, window=8, net=None, max_iter=4000, rtol=1e-6, check_every=25):
    """Truncated flexible CG on inv's normal equations from x = 0: the inner iteration of
    lentils_fcg_solve without its restarts (FP32 operator and vectors, FP64 dot products). Each
    direction p_k = d_k - sum_j (d_k . A p_j / p_j . A p_j) p_j over the last `window`
    directions; d_k = net.precondition(r_k) where that is a descent direction (d.r > 0), else
    the Jacobi direction dinv r_k (always, without a network). Returns the iterates xs
    (K + 1, n), x_0 = 0, and the normalised A-directions q_k = A p_k / sqrt(p_k . A p_k)
    (K, n): the direction taken after step k is made A-orthogonal to q_{k-m}, ..., q_{k-1},
    m = min(k, window)."""
    import ctypes as _ct
    n = inv.nsrc
    L = N.lib()
    xs = torch.zeros((max_iter + 1, n), dtype=torch.float32, device="cuda")
    qs = torch.zeros((max_iter, n), dtype=torch.float32, device="cuda")
    b = inv.b.float()
    dinv = inv.inv_diag32
    bn = float(torch.linalg.vector_norm(inv.b))
    sp = _ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    x = torch.zeros(n, dtype=torch.float32, device="cuda")
    r = b.clone()
    p = dinv * r
    ring = []  # (p_j, A p_j, p_j . A p_j)
    feat = features(dinv) if net is not None else None
    k = 0
    while k < max_iter:
        ap = torch.empty_like(p)
        N.check(L.lentils_normal_op_apply(inv.handle, _ptr(p), _ptr(ap), sp))
        pap = torch.dot(p.double(), ap.double())
        alpha = (torch.dot(p.double(), r.double()) / pap).float()
        x.add_(alpha * p)
        r.sub_(alpha * ap)
        qs[k] = ap / pap.sqrt().float()
        k += 1
        xs[k] = x
        ring.append((p, ap, pap))
        if len(ring) > window:
            ring.pop(0)
        if k % check_every == 0 and float(torch.linalg.vector_norm(r.double())) <= rtol * bn:
            break
        d = dinv * r
        if net is not None:
            z = net.precondition(r, dinv, feat)
            if float(torch.dot(z.double(), r.double())) > 0.0:
                d = z
        p = d.clone()
        for pj, apj, papj in ring:
            p.add_((-torch.dot(d.double(), apj.double()) / papj).float() * pj)
    return xs[:k + 1], qs[:k]


def window_pairs(inv, npairs, rng, window=8, net=None, max_iter=4000, tol_star=1e-9):
    """(residual, correction, window) triples of one inversion along its flexible-CG trajectory
    (fcg_trajectory, Jacobi or with `net`) at iterations drawn uniformly: the true FP64 residual
    r_k = b - A x_k, the correction e_k = x* - x_k to the FP64-refined solution x*, and the
    normalised A-directions the solver's next direction is made A-orthogonal to, zero-padded
    to `window` rows. Returns float32 CUDA tensors (npairs, n), (npairs, n),
    (npairs, window, n) and the trajectory length."""
    import ctypes as _ct
    x_star, _ = inv.solve(tol=tol_star, max_outer=60)
    xs, qs = fcg_trajectory(inv, window=window, net=net, max_iter=max_iter)
    K = xs.shape[0] - 1
    idx = np.sort(rng.choice(K, size=min(npairs, K), replace=False))
    L = N.lib()
    sp = _ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    rs, es = [], []
    Q = torch.zeros((idx.size, window, inv.nsrc), dtype=torch.float32, device="cuda")
    ax = torch.empty(inv.nsrc, dtype=torch.float64, device="cuda")
    for i, k in enumerate(idx.tolist()):
        xk = xs[k].double()
        N.check(L.lentils_normal_op_apply64(inv.handle, _ptr(xk), _ptr(ax), sp))
        rs.append((inv.b - ax).float())
        es.append((x_star - xk).float())
        m = min(k, window)
        if m:
            Q[i, :m] = qs[k - m:k]
    return torch.stack(rs), torch.stack(es), Q, K


def trajectory_pairs(inv, npairs, rng, max_iter=8000, tol_star=1e-9):
    """(residual, correction) pairs of one inversion: iterates x_k of plain Jacobi-CG at
    geometrically spaced iterations, the true FP64 residual r_k = b - A x_k and the correction
    e_k = x* - x_k to the FP64-refined solution x*. Returns float32 CUDA tensors (npairs, n)."""
    import ctypes as _ct
    x_star, info = inv.solve(tol=tol_star, max_outer=60)
    xs = jacobi_cg_trajectory(inv, max_iter=max_iter)
    K = xs.shape[0]
    idx = np.unique(np.clip(np.round(np.geomspace(1, K, npairs * 2)).astype(int) - 1, 0, K - 1))
    idx = np.sort(rng.choice(idx, size=min(npairs, idx.size), replace=False))
    L = N.lib()
    sp = _ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    rs, es = [], []
    ax = torch.empty(inv.nsrc, dtype=torch.float64, device="cuda")
    for k in idx:
        xk = xs[int(k)].double()
        N.check(L.lentils_normal_op_apply64(inv.handle, _ptr(xk), _ptr(ax), sp))
        rs.append((inv.b - ax).float())
        es.append((x_star - xk).float())
    return torch.stack(rs), torch.stack(es), K - 1, info
