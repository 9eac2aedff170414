"""GPU source inversion: solve (L^T F^T C^-1 F L + lambda R^T R) s = L^T F^T C^-1 d.

Restates the reference's CG source-inversion pattern (lentils/tests/solver_tests.py:77-114:
lhs = lensop.T * uvdata.covariance-weighted NUFFT normal operator * lensop + reg_op,
rhs = lensop.T * dirty image, solved by CG) with the explicit-visibility normal operator
F^T C^-1 F (nufft.T * cov * nufft, lentils/tests/nufft_tests.py:87), a bilinear lens operator
and the 'gradient' prior, as one device-resident operator solved by mixed-precision iterative
refinement (lentils_cg_solve): FP32 Jacobi-PCG inner solves, FP64 true residuals outside.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as N
from .gridding import _ptr
from .operators import (BilinearLensOperator, BlurredCovarianceOperator, ManifoldLensOperator,
                        NUFFTOperator)


class SourceInversion:
    def __init__(self, vis_space, data, sigma, image_space, source_space, lensmodel, z_src,
                 strength, kernel_support=4, pad_factor=2, kb_beta=None, data_mask=None,
                 nufft=None, data_term="visibilities", lens_operator="bilinear"):
        """nufft: an existing NUFFTOperator for vis_space and image_space to share (lens-model
        sweeps over one visibility set); built here when None. data_term: "visibilities"
        (F^T C^-1 F through the gridder every matvec) or "bcb" (the dirty-beam convolution,
        RadioDataset.blurred_covariance_operator, data_base.py:115-129, with the right-hand
        side L^T times the dirty image F^T C^-1 d)."""
        if data_term not in ("visibilities", "bcb"):
            raise ValueError("data_term: 'visibilities' or 'bcb'")
        if lens_operator not in ("bilinear", "manifold"):
            raise ValueError("lens_operator: 'bilinear' or 'manifold'")
        self.data_term = data_term
        self.stream = torch.cuda.Stream()
        with torch.cuda.stream(self.stream):
            self.nufft = nufft if nufft is not None else NUFFTOperator(
                vis_space, image_space, pad_factor, kernel_support, kb_beta)
            lens_cls = ManifoldLensOperator if lens_operator == "manifold" else \
                BilinearLensOperator
            self.lens = lens_cls(image_space, source_space, lensmodel, z_src)
            self.source_space = source_space
            self.image_space = image_space
            plan = self.nufft.plan
            self.plan = plan
            nvis = plan.nvis
            sig = np.broadcast_to(np.asarray(sigma, dtype=np.float64), (nvis,)).reshape(-1)
            mask = np.ones(nvis, bool) if data_mask is None else np.asarray(data_mask).reshape(-1)
            w_user = np.zeros(nvis)
            w_user[mask] = sig[mask] ** -2.0  # RadioDataset.covariance_operator, data_base.py:36-44
            wu = torch.as_tensor(w_user).cuda()
            self.weights = torch.empty(nvis, dtype=torch.float64, device="cuda")
            sp = ctypes.c_void_p(self.stream.cuda_stream)
            L = N.lib()
            N.check(L.lentils_plan_gather_real(plan.handle, _ptr(wu), _ptr(self.weights), sp))
            self._normal = ctypes.c_void_p()
            self.nsrc = source_space.nx * source_space.ny
            self.b = torch.empty(self.nsrc, dtype=torch.float64, device="cuda")
            nimg = image_space.nx * image_space.ny
            if data_term == "bcb":
                self.bcb = BlurredCovarianceOperator(vis_space, image_space, w_user,
                                                     kernel_support, pad_factor, kb_beta)
                N.check(L.lentils_normal_op_create_bcb(
                    ctypes.byref(self._normal), self.lens.handle, self.bcb.handle, nimg,
                    source_space.nx, source_space.ny, source_space.dx, source_space.dy,
                    float(strength), sp))
                dv = np.ascontiguousarray(data, dtype=np.complex128).reshape(-1)
                dirty = self.nufft.T * (w_user * dv)   # dirty image, FP64 on the GPU
                self.dirty_image = np.asarray(dirty, dtype=np.float64).reshape(-1)
                di = torch.as_tensor(self.dirty_image).cuda()
                N.check(L.lentils_normal_op_rhs_image64(self._normal, _ptr(di), _ptr(self.b),
                                                        sp))
            else:
                N.check(L.lentils_normal_op_create(
                    ctypes.byref(self._normal), self.lens.handle, self.nufft.handle,
                    _ptr(self.weights), nvis, nimg, source_space.nx, source_space.ny,
                    source_space.dx, source_space.dy, float(strength), sp))
                d = torch.as_tensor(np.ascontiguousarray(data, dtype=np.complex128)
                                    .reshape(-1)).cuda()
                dp = torch.empty(nvis, dtype=torch.complex128, device="cuda")
                N.check(L.lentils_vis_to_plan64(plan.handle, _ptr(d), _ptr(dp), sp))
                N.check(L.lentils_normal_op_rhs64(self._normal, _ptr(dp), _ptr(self.b), sp))
            self.inv_diag = torch.empty(self.nsrc, dtype=torch.float64, device="cuda")
            self.inv_diag32 = torch.empty(self.nsrc, dtype=torch.float32, device="cuda")
            N.check(L.lentils_normal_op_jacobi(self._normal, _ptr(self.inv_diag),
                                               _ptr(self.inv_diag32), sp))
        self.stream.synchronize()
        self.strength = float(strength)
        # the problem as given (reference row order), for residual checks by callers
        self.data_user = np.ascontiguousarray(data, dtype=np.complex128).reshape(-1)
        self.weights_user = w_user

    @property
    def handle(self):
        return self._normal

    def __del__(self):
        try:
            if self._normal.value:
                N.lib().lentils_normal_op_destroy(self._normal)
        except Exception:
            pass

    def apply(self, s):
        """A s: float32 CUDA tensor -> FP32 operator, float64 tensor or numpy -> FP64."""
        host = not isinstance(s, torch.Tensor)
        x = torch.as_tensor(np.ascontiguousarray(s, dtype=np.float64).reshape(-1)).cuda() if host \
            else s.contiguous().reshape(-1)
        out = torch.empty_like(x)
        sp = ctypes.c_void_p(self.stream.cuda_stream)
        torch.cuda.current_stream().synchronize()
        fn = N.lib().lentils_normal_op_apply if x.dtype == torch.float32 else \
            N.lib().lentils_normal_op_apply64
        N.check(fn(self._normal, _ptr(x), _ptr(out), sp))
        self.stream.synchronize()
        return out.cpu().numpy() if host else out

    def solve(self, tol=1e-6, inner_tol=1e-2, max_outer=30, max_inner=5000, check_every=10,
              use_graph=True, x0=None, precondition=True):
        """Solve to a true FP64 relative residual `tol`. Returns (x float64 CUDA tensor, info)."""
        x = torch.zeros(self.nsrc, dtype=torch.float64, device="cuda") if x0 is None else \
            torch.as_tensor(x0, dtype=torch.float64).reshape(-1).cuda().clone()
        opt = N.CGOptionsC(float(tol), float(inner_tol), int(max_outer), int(max_inner),
                           int(check_every), 1 if use_graph else 0)
        res = N.CGResultC()
        torch.cuda.synchronize()
        N.check(N.lib().lentils_cg_solve(
            self._normal, _ptr(self.b), _ptr(x),
            _ptr(self.inv_diag32) if precondition else None, ctypes.byref(opt),
            ctypes.byref(res), ctypes.c_void_p(self.stream.cuda_stream)))
        self.stream.synchronize()
        info = {f: getattr(res, f) for f, _ in res._fields_}
        return x, info

    def solve_flexible(self, net=None, tol=1e-6, inner_tol=1e-2, max_outer=30, max_inner=5000,
                       check_every=10, use_graph=True, x0=None, window=1, net_every=1):
        """Flexible CG with the learned preconditioner `net` (learned.UNet on the source grid;
        None: the same iteration with Jacobi directions only), inside the same FP64 iterative
        refinement as solve(); the network proposes every `net_every`-th direction. Returns
        (x float64 CUDA tensor, info)."""
        x = torch.zeros(self.nsrc, dtype=torch.float64, device="cuda") if x0 is None else \
            torch.as_tensor(x0, dtype=torch.float64).reshape(-1).cuda().clone()
        opt = N.CGOptionsC(float(tol), float(inner_tol), int(max_outer), int(max_inner),
                           int(check_every), 1 if use_graph else 0, int(window), int(net_every))
        res = N.CGResultC()
        torch.cuda.synchronize()
        N.check(N.lib().lentils_fcg_solve(
            self._normal, _ptr(self.b), _ptr(x), _ptr(self.inv_diag32),
            net.handle if net is not None else None, ctypes.byref(opt), ctypes.byref(res),
            ctypes.c_void_p(self.stream.cuda_stream)))
        self.stream.synchronize()
        info = {f: getattr(res, f) for f, _ in res._fields_}
        return x, info
