"""Operator algebra and the GPU operators of the visibility-space chain, mirroring
lentils/operators/operator_base.py and fourier_operators.py (same class names, constructor
arguments, `op * x`, `op.T`, `op1 + op2`, `op1 * op2`).

Vectors follow the reference: numpy arrays shaped like the spaces (image (1,1,nx,ny) float64,
visibilities (nchannels,1,nrows) complex128 in row order, grids (1,1,nu,nv//2+1) complex128).
numpy vectors run through the FP64 device operators and come back as numpy. CUDA tensors stay on
the device: float64/complex128 tensors use the FP64 operators and float32/complex64 tensors
the FP32 operators; visibility tensors are then in plan order and plan frame (see
GriddingPlan).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as N
from .gridding import GriddingPlan, _ptr, _stream_ptr
from .spaces import DelaunaySpace, FourierSpace, ImageSpace


def _is_tensor(x):
    return isinstance(x, torch.Tensor)


class Operator:
    """Base class: space_left <- space_right (operator_base.py:46-113)."""

    def __init__(self, space_left, space_right):
        self.space_left = space_left
        self.space_right = space_right

    def _forward(self, x):
        raise NotImplementedError

    def _transpose(self, x):
        raise NotImplementedError

    @property
    def T(self):
        t = getattr(self, "_T", None)
        if t is None:
            t = _Transposed(self)
            self._T = t
        return t

    def apply(self, other):
        if isinstance(other, Operator):
            return CompositeOperatorProduct([self, other])
        return self._forward(other)

    def __mul__(self, other):
        return self.apply(other)

    def __add__(self, other):
        return CompositeOperatorSum([self, other])

    def __repr__(self):
        return f"<{type(self).__name__}: {self.space_right} -> {self.space_left}>"


class _Transposed(Operator):
    def __init__(self, op):
        super().__init__(op.space_right, op.space_left)
        self._op = op
        self._T = op

    def _forward(self, x):
        return self._op._transpose(x)

    def _transpose(self, x):
        return self._op._forward(x)


class CompositeOperatorProduct(Operator):
    """Right-to-left product (operator_base.py:116-143)."""

    def __init__(self, oplist):
        self.subops = []
        for op in oplist:
            self.subops += op.subops if isinstance(op, CompositeOperatorProduct) else [op]
        super().__init__(self.subops[0].space_left, self.subops[-1].space_right)

    def _forward(self, x):
        for op in self.subops[::-1]:
            x = op * x
        return x

    def _transpose(self, x):
        for op in self.subops:
            x = op.T * x
        return x


class CompositeOperatorSum(Operator):
    """Sum of operators with the same spaces (operator_base.py:146-175)."""

    def __init__(self, oplist):
        self.subops = []
        for op in oplist:
            self.subops += op.subops if isinstance(op, CompositeOperatorSum) else [op]
        super().__init__(self.subops[0].space_left, self.subops[-1].space_right)

    def _forward(self, x):
        out = self.subops[0] * x
        for op in self.subops[1:]:
            out = out + op * x
        return out

    def _transpose(self, x):
        out = self.subops[0].T * x
        for op in self.subops[1:]:
            out = out + op.T * x
        return out


class DiagonalOperator(Operator):
    """Elementwise scaling by `data` (operator_base.py:178-197); symmetric."""

    def __init__(self, space, data):
        super().__init__(space, space)
        self._data = np.asarray(data)

    def _forward(self, x):
        host = not _is_tensor(x)
        t = torch.as_tensor(np.asarray(x)).cuda() if host else x
        d = torch.as_tensor(self._data.reshape(t.shape), device=t.device).to(t.dtype)
        out = t * d
        return out.cpu().numpy() if host else out

    _transpose = _forward


class GriddingOperator(Operator):
    """Visibilities <- half-plane grid (fourier_operators.py:71-93); the Nyquist guard of
    :77-80 raises ValueError as in the reference."""

    def __init__(self, space_vis, space_fourier, kb_beta, kernel_support, tile=0):
        self.kernel_support = int(kernel_support)
        self.kb_beta = float(kb_beta)
        iumax = np.max(space_vis.channels) * np.max(np.abs(space_vis.uvw[:, 0])) / space_fourier.du
        ivmax = np.max(space_vis.channels) * np.max(np.abs(space_vis.uvw[:, 1])) / space_fourier.dv
        if (iumax + self.kernel_support + 1 > 0.5 * space_fourier.nu
                or ivmax + self.kernel_support + 1 > 0.5 * space_fourier.nv):
            raise ValueError("Visibility space contains points higher than the Nyquist "
                             "frequency of the grid.")
        super().__init__(space_vis, space_fourier)
        self.plan = GriddingPlan(space_vis.uvw, space_vis.channels, space_fourier.nu,
                                 space_fourier.nv, space_fourier.du, space_fourier.dv,
                                 space_fourier.gcx, space_fourier.gcy, self.kernel_support,
                                 self.kb_beta, tile=tile)

    def _forward(self, grid):
        p = self.plan
        if _is_tensor(grid):
            if grid.dtype == torch.complex64:
                return p.degrid(grid)
            g = grid.to(torch.complex128).contiguous()
            out = torch.empty(p.nvis, dtype=torch.complex128, device=g.device)
            N.check(N.lib().lentils_degrid64(p.handle, _ptr(g), _ptr(out), _stream_ptr()))
            return out
        g = torch.as_tensor(np.ascontiguousarray(grid, dtype=np.complex128)).cuda()
        y = self._forward(g)
        out = torch.zeros(p.nvis, dtype=torch.complex128, device="cuda")
        N.check(N.lib().lentils_vis_from_plan64(p.handle, _ptr(y), _ptr(out), 0, _stream_ptr()))
        return out.cpu().numpy().reshape(self.space_left.shape)

    def _transpose(self, vis):
        p = self.plan
        if _is_tensor(vis):
            if vis.dtype == torch.complex64:
                return p.grid(vis)
            v = vis.to(torch.complex128).contiguous()
            out = torch.zeros((p.nu, p.half_nv), dtype=torch.complex128, device=v.device)
            N.check(N.lib().lentils_grid64(p.handle, _ptr(v), _ptr(out), _stream_ptr()))
            return out
        v = torch.as_tensor(np.ascontiguousarray(vis, dtype=np.complex128).reshape(-1)).cuda()
        vp = torch.empty(p.nvis, dtype=torch.complex128, device="cuda")
        N.check(N.lib().lentils_vis_to_plan64(p.handle, _ptr(v), _ptr(vp), _stream_ptr()))
        return self._transpose(vp).cpu().numpy().reshape(self.space_right.shape)


def kb_beta_beatty(kernel_support, pad_factor):
    """NUFFTOperator's shape parameter (fourier_operators.py:104-108)."""
    return np.pi * np.sqrt((2.0 * kernel_support / pad_factor) ** 2 * (pad_factor - 0.5) ** 2 - 0.8)


class NUFFTOperator(Operator):
    """F = Gridder . rFFT2 . ZeroPad . Apod (fourier_operators.py:96-126): image -> visibilities.

    kb_beta defaults to the reference's Beatty value; pass it explicitly to use another."""

    def __init__(self, vis_space, image_space, pad_factor=2, kernel_support=4, kb_beta=None,
                 tile=0, precisions=3):
        self.image_space = image_space
        self.pad_factor = int(pad_factor)
        self.kernel_support = int(kernel_support)
        self.kb_beta = (kb_beta_beatty(self.kernel_support, self.pad_factor) if kb_beta is None
                        else float(kb_beta))
        # zero padding (ZeroPaddingOperator, fourier_operators.py:29-42)
        p = self.pad_factor
        self.padx = ((p - 1) * image_space.nx + 1) // 2
        self.pady = ((p - 1) * image_space.ny + 1) // 2
        dx, dy = image_space.dx, image_space.dy
        bounds = image_space.bounds + np.array([-self.padx * dx, self.padx * dx,
                                                -self.pady * dy, self.pady * dy])
        self.padded_space = ImageSpace(shape=(image_space.nx + 2 * self.padx,
                                              image_space.ny + 2 * self.pady),
                                       bounds=[(bounds[0], bounds[1]), (bounds[2], bounds[3])])
        self.fourier_space = FourierSpace(self.padded_space)
        # apodisation factors (ApodizationCorrectionOperator, fourier_operators.py:54-68)
        w = self.kernel_support
        cx = (np.arange(image_space.nx) - 0.5 * image_space.nx) / self.padded_space.nx
        cy = (np.arange(image_space.ny) - 0.5 * image_space.ny) / self.padded_space.ny
        ax = np.sqrt(self.kb_beta ** 2 - (2 * np.pi * w * cx) ** 2)
        ay = np.sqrt(self.kb_beta ** 2 - (2 * np.pi * w * cy) ** 2)
        self.apod_x = np.ascontiguousarray(ax / np.sinh(ax))
        self.apod_y = np.ascontiguousarray(ay / np.sinh(ay))
        self.gridder = GriddingOperator(vis_space, self.fourier_space, self.kb_beta,
                                        self.kernel_support, tile=tile)
        self.plan = self.gridder.plan
        self._handle = ctypes.c_void_p()
        N.check(N.lib().lentils_nufft_create(
            ctypes.byref(self._handle), self.plan.handle, image_space.nx, image_space.ny,
            self.padx, self.pady, ctypes.c_void_p(self.apod_x.ctypes.data),
            ctypes.c_void_p(self.apod_y.ctypes.data), int(precisions), _stream_ptr()))
        super().__init__(vis_space, image_space)

    @property
    def handle(self):
        return self._handle

    def close(self):
        if getattr(self, "_handle", None) is not None and self._handle.value:
            N.lib().lentils_nufft_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _forward(self, image):
        L, p = N.lib(), self.plan
        if _is_tensor(image):
            x = image.contiguous().reshape(-1)
            if x.dtype == torch.float32:
                out = torch.empty(p.nvis, dtype=torch.complex64, device=x.device)
                N.check(L.lentils_nufft_forward(self._handle, _ptr(x), _ptr(out), _stream_ptr()))
            else:
                x = x.to(torch.float64)
                out = torch.empty(p.nvis, dtype=torch.complex128, device=x.device)
                N.check(L.lentils_nufft_forward64(self._handle, _ptr(x), _ptr(out), _stream_ptr()))
            return out
        x = torch.as_tensor(np.ascontiguousarray(image, dtype=np.float64).reshape(-1)).cuda()
        y = self._forward(x)
        out = torch.zeros(p.nvis, dtype=torch.complex128, device="cuda")
        N.check(L.lentils_vis_from_plan64(p.handle, _ptr(y), _ptr(out), 0, _stream_ptr()))
        return out.cpu().numpy().reshape(self.space_left.shape)

    def _transpose(self, vis):
        L, p = N.lib(), self.plan
        n = self.image_space.nx * self.image_space.ny
        if _is_tensor(vis):
            v = vis.contiguous().reshape(-1)
            if v.dtype == torch.complex64:
                out = torch.empty(n, dtype=torch.float32, device=v.device)
                N.check(L.lentils_nufft_adjoint(self._handle, _ptr(v), _ptr(out), _stream_ptr()))
            else:
                v = v.to(torch.complex128)
                out = torch.empty(n, dtype=torch.float64, device=v.device)
                N.check(L.lentils_nufft_adjoint64(self._handle, _ptr(v), _ptr(out), _stream_ptr()))
            return out.reshape(self.image_space.nx, self.image_space.ny)
        v = torch.as_tensor(np.ascontiguousarray(vis, dtype=np.complex128).reshape(-1)).cuda()
        vp = torch.empty(p.nvis, dtype=torch.complex128, device="cuda")
        N.check(L.lentils_vis_to_plan64(p.handle, _ptr(v), _ptr(vp), _stream_ptr()))
        return self._transpose(vp).cpu().numpy().reshape(self.image_space.shape)


class BilinearLensOperator(Operator):
    """Image pixels <- regular source grid by bilinear interpolation at the deflected pixel
    positions (no reference counterpart; see include/lentils_gb300.h). `lensmodel` is a
    GlobalLensModel; image-plane positions are ImageSpace.points (pixel corners)."""

    def __init__(self, image_space, source_space, lensmodel, z_src):
        from .lens_models import deflect_points
        lenses = lensmodel.setup_raytracing(z_src)
        pts = torch.as_tensor(np.ascontiguousarray(image_space.points.reshape(-1, 2))).cuda()
        self.source_points = deflect_points(lenses, pts)
        mask = torch.as_tensor(np.ascontiguousarray(image_space.mask.reshape(-1)).astype(np.uint8)).cuda()
        self._handle = ctypes.c_void_p()
        N.check(N.lib().lentils_lensop_create(
            ctypes.byref(self._handle), _ptr(self.source_points), _ptr(mask),
            image_space.nx * image_space.ny, source_space.nx, source_space.ny, source_space.xmin,
            source_space.ymin, source_space.dx, source_space.dy, _stream_ptr()))
        self._mask = mask
        super().__init__(image_space, source_space)

    @property
    def handle(self):
        return self._handle

    def __del__(self):
        try:
            if self._handle.value:
                N.lib().lentils_lensop_destroy(self._handle)
        except Exception:
            pass

    def _run(self, x, fwd):
        L = N.lib()
        nout = (self.space_left.nx * self.space_left.ny if fwd
                else self.space_right.nx * self.space_right.ny)
        host = not _is_tensor(x)
        t = torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64).reshape(-1)).cuda() if host \
            else x.contiguous().reshape(-1)
        out = torch.empty(nout, dtype=t.dtype, device=t.device)
        if t.dtype == torch.float32:
            fn = L.lentils_lensop_apply if fwd else L.lentils_lensop_apply_t
        else:
            fn = L.lentils_lensop_apply64 if fwd else L.lentils_lensop_apply_t64
        N.check(fn(self._handle, _ptr(t), _ptr(out), _stream_ptr()))
        sp = self.space_left if fwd else self.space_right
        return out.cpu().numpy().reshape(sp.shape) if host else out.reshape(sp.nx, sp.ny)

    def _forward(self, src):
        return self._run(src, True)

    def _transpose(self, img):
        return self._run(img, False)


class ManifoldLensOperator(BilinearLensOperator):
    """The reference's ManifoldLensOperator (lentils/operators/lens_operators.py:21-38,
    manifold_lens_matrix_csr of lentils/backend/raster.c:272-395): image pixels <- source
    pixels weighted by the rasterised overlap of each pixel's 8 deflected triangles, built on
    the GPU in FP64 (lentils_manifold_lens_matrix) and applied as CSR / transposed CSR.
    `matrix` holds a scipy copy of the CSR."""

    def __init__(self, image_space, source_space, lensmodel, z_src):
        lenses = lensmodel.setup_raytracing(z_src)
        mask = torch.as_tensor(np.ascontiguousarray(image_space.mask.reshape(-1))
                               .astype(np.uint8)).cuda()
        L = N.lib()
        rows, cols, vals = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        nnz = ctypes.c_longlong()
        torch.cuda.current_stream().synchronize()
        N.check(L.lentils_manifold_lens_matrix(
            ctypes.byref(image_space), ctypes.byref(source_space),
            ctypes.c_void_p(lenses.ctypes.data), len(lenses), _ptr(mask), ctypes.byref(rows),
            ctypes.byref(cols), ctypes.byref(vals), ctypes.byref(nnz), _stream_ptr()))
        nimg, nsrc = image_space.nx * image_space.ny, source_space.nx * source_space.ny
        self._handle, self.matrix = _csr_lensop(rows, cols, vals, nnz.value, nimg, nsrc)
        self._mask = mask
        Operator.__init__(self, image_space, source_space)


def _csr_lensop(rows, cols, vals, nnz, nimg, nsrc):
    """lensop handle and scipy copy of a device CSR an entry point returned (freed here)."""
    import scipy.sparse as sps
    L = N.lib()
    n = int(nnz)
    try:
        h = ctypes.c_void_p()
        N.check(L.lentils_lensop_create_csr(ctypes.byref(h), rows, cols, vals, nimg, nsrc, n,
                                            _stream_ptr()))
        h_rows = np.empty(nimg + 1, np.int32)
        h_cols = np.empty(max(1, n), np.int32)
        h_vals = np.empty(max(1, n), np.float64)
        for dst, src, nb in ((h_rows, rows, 4 * (nimg + 1)), (h_cols, cols, 4 * n),
                             (h_vals, vals, 8 * n)):
            N.check(L.lentils_copy_to_host(ctypes.c_void_p(dst.ctypes.data), src, nb))
    finally:
        for ptr in (rows, cols, vals):
            if ptr.value:
                L.lentils_device_free(ptr)
    return h, sps.csr_matrix((h_vals[:n], h_cols[:n], h_rows), shape=(nimg, nsrc))


def deflect64(lenses, points):
    """FP64 deflection with the reference's formulas (lentils_deflect64): numpy (..., 2) in and
    out."""
    p = torch.as_tensor(np.ascontiguousarray(points, dtype=np.float64)).cuda()
    out = torch.empty_like(p)
    lenses = np.ascontiguousarray(lenses)
    N.check(N.lib().lentils_deflect64(ctypes.c_void_p(lenses.ctypes.data), len(lenses),
                                      _ptr(p), _ptr(out), p.numel() // 2, _stream_ptr()))
    return out.cpu().numpy()


class DelaunayLensOperator(BilinearLensOperator):
    """The reference's DelaunayLensOperator (lentils/operators/lens_operators.py:43-80): image
    pixels on the `ncasted` lattice are the source vertices, deflected in FP64 on the GPU;
    scipy triangulates them and locates the other deflected pixels, as the reference does; the
    barycentric CSR (delaunay_lens_matrix_csr, triangles.c:105-140) is assembled on the GPU.
    `source_space` is the DelaunaySpace of the casted points; `matrix` a scipy copy."""

    def __init__(self, image_space, lensmodel, z_src, ncasted=1):
        lenses = lensmodel.setup_raytracing(z_src)
        mask = image_space.mask
        pts = image_space.points
        cmask = np.zeros_like(mask)
        cmask[::ncasted, ::ncasted] = True
        umask = ~cmask
        cmask = cmask & mask
        umask = umask & mask
        self.casted_points = deflect64(lenses, pts[cmask])
        self.uncasted_points = deflect64(lenses, pts[umask])
        self.source_space = DelaunaySpace(self.casted_points)
        tind = self.source_space.delaunay.find_simplex(self.uncasted_points)
        nimg = image_space.nx * image_space.ny
        dev = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a, dtype=dt)).cuda()
        mask_d = dev(mask.reshape(-1).astype(np.uint8), np.uint8)
        up = dev(self.uncasted_points.reshape(-1, 2), np.float64)
        ti = dev(tind, np.int32)
        tr = dev(self.source_space.triangles, np.int32)
        tp = dev(self.casted_points.reshape(-1, 2), np.float64)
        rows, cols, vals = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        nnz = ctypes.c_longlong()
        N.check(N.lib().lentils_delaunay_lens_matrix(
            _ptr(mask_d), image_space.nx, image_space.ny, int(ncasted), _ptr(up), _ptr(ti),
            _ptr(tr), _ptr(tp), ctypes.byref(rows), ctypes.byref(cols), ctypes.byref(vals),
            ctypes.byref(nnz), _stream_ptr()))
        self._nsrc = self.source_space.num_points
        self._handle, self.matrix = _csr_lensop(rows, cols, vals, nnz.value, nimg, self._nsrc)
        self._mask = mask_d
        Operator.__init__(self, image_space, self.source_space)

    def _run(self, x, fwd):
        L = N.lib()
        nout = self.space_left.nx * self.space_left.ny if fwd else self._nsrc
        host = not _is_tensor(x)
        t = torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64).reshape(-1)).cuda() if host \
            else x.contiguous().reshape(-1)
        out = torch.empty(nout, dtype=t.dtype, device=t.device)
        if t.dtype == torch.float32:
            fn = L.lentils_lensop_apply if fwd else L.lentils_lensop_apply_t
        else:
            fn = L.lentils_lensop_apply64 if fwd else L.lentils_lensop_apply_t64
        N.check(fn(self._handle, _ptr(t), _ptr(out), _stream_ptr()))
        if fwd:
            sp = self.space_left
            return out.cpu().numpy().reshape(sp.shape) if host else out.reshape(sp.nx, sp.ny)
        return out.cpu().numpy() if host else out


class DFTOperator(Operator):
    """The direct Fourier sum (DFTOperator, lentils/operators/fourier_operators.py:130-145)
    in FP64 on the GPU (lentils_dft_forward / lentils_dft_adjoint): image (nx, ny) ->
    visibilities (nrows,) complex128 and the real transpose back. A validator of the NUFFT;
    numpy in, numpy out."""

    def __init__(self, vis_space, image_space):
        self._uvw = torch.as_tensor(np.ascontiguousarray(vis_space.uvw, dtype=np.float64)
                                    .reshape(-1, 3)).cuda()
        self._ch = torch.as_tensor(np.ascontiguousarray(vis_space.channels, dtype=np.float64)
                                   .reshape(-1)).cuda()
        self._mask = torch.as_tensor(np.ascontiguousarray(image_space.mask.reshape(-1))
                                     .astype(np.uint8)).cuda()
        self._nrows = self._uvw.shape[0]
        super().__init__(vis_space, image_space)

    def _forward(self, image):
        sp = self.space_right
        x = torch.as_tensor(np.ascontiguousarray(image, dtype=np.float64).reshape(-1)).cuda()
        out = torch.empty(self._nrows, dtype=torch.complex128, device="cuda")
        N.check(N.lib().lentils_dft_forward(_ptr(self._uvw), self._nrows, _ptr(self._ch),
                                            ctypes.byref(sp), _ptr(self._mask), _ptr(x),
                                            _ptr(out), _stream_ptr()))
        return out.cpu().numpy()

    def _transpose(self, vis):
        sp = self.space_right
        v = torch.as_tensor(np.ascontiguousarray(vis, dtype=np.complex128).reshape(-1)).cuda()
        out = torch.empty(sp.nx * sp.ny, dtype=torch.float64, device="cuda")
        N.check(N.lib().lentils_dft_adjoint(_ptr(self._uvw), self._nrows, _ptr(self._ch),
                                            ctypes.byref(sp), _ptr(self._mask), _ptr(v),
                                            _ptr(out), _stream_ptr()))
        return out.cpu().numpy().reshape(sp.nx, sp.ny)


class PriorCovarianceOperator(Operator):
    """lambda * R^T R with R the forward-difference gradient of grad_matrix_findiff_csr
    ('gradient' prior of operator_base.py:200-251), matrix-free; symmetric."""

    def __init__(self, space, type="gradient", strength=1.0):
        if type != "gradient":
            raise NotImplementedError("only the 'gradient' prior is built")
        self._lambda = float(strength)
        super().__init__(space, space)
        self._T = self

    def _forward(self, s):
        host = not _is_tensor(s)
        sp = self.space_left
        x = torch.as_tensor(np.ascontiguousarray(s, dtype=np.float64).reshape(-1)).cuda() if host \
            else s.contiguous().reshape(-1)
        out = torch.empty_like(x)
        L = N.lib()
        fn = L.lentils_prior_gradient_apply if x.dtype == torch.float32 else \
            L.lentils_prior_gradient_apply64
        N.check(fn(_ptr(x), _ptr(out), sp.nx, sp.ny, sp.dx, sp.dy, self._lambda, _stream_ptr()))
        return out.cpu().numpy().reshape(sp.shape) if host else out.reshape(sp.nx, sp.ny)

    _transpose = _forward


class BlurredCovarianceOperator(Operator):
    """F^T C^-1 F as a convolution with the dirty beam (RadioDataset.blurred_covariance_operator,
    lentils/common/data_base.py:115-129): the beam NUFFT_beam^T C^-1 1 is computed once on the
    beam space (2nx x 2ny pixels, bounds +-(nx dx, ny dy), data_base.py:147-172) by the FP64
    NUFFT adjoint on the GPU; each application is pad, rFFT, multiply, inverse rFFT, crop
    (lentils_bcb). `weights` are C^-1 per visibility in the reference's row order. Symmetric.
    numpy in -> FP64 on the GPU -> numpy out; a float32 CUDA tensor -> FP32."""

    def __init__(self, vis_space, image_space, weights, kernel_support=4, pad_factor=2,
                 kb_beta=None):
        nx, ny = image_space.nx, image_space.ny
        if nx % 2 or ny % 2:
            raise ValueError("the dirty-beam form needs even image sizes")
        rx, ry = image_space.dx * nx, image_space.dy * ny
        self.beam_space = ImageSpace(shape=(2 * nx, 2 * ny), bounds=[(-rx, rx), (-ry, ry)])
        nufft_beam = NUFFTOperator(vis_space, self.beam_space, pad_factor, kernel_support,
                                   kb_beta)
        w = np.asarray(weights, dtype=np.float64).reshape(-1)
        self.dirty_beam = np.ascontiguousarray(
            (nufft_beam.T * (w + 0.0j)).reshape(2 * nx, 2 * ny), dtype=np.float64)
        nufft_beam.close()
        beam_d = torch.as_tensor(self.dirty_beam).cuda()
        self._h = ctypes.c_void_p()
        N.check(N.lib().lentils_bcb_create(ctypes.byref(self._h), _ptr(beam_d), nx, ny,
                                           _stream_ptr()))
        torch.cuda.current_stream().synchronize()
        super().__init__(image_space, image_space)
        self._T = self

    @property
    def handle(self):
        return self._h

    @property
    def centre(self):
        return N.lib().lentils_bcb_centre(self._h)

    def __del__(self):
        try:
            if self._h.value:
                N.lib().lentils_bcb_destroy(self._h)
        except Exception:
            pass

    def _forward(self, x):
        host = not _is_tensor(x)
        sp = self.space_left
        v = torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64).reshape(-1)).cuda() if host \
            else x.contiguous().reshape(-1)
        out = torch.empty_like(v)
        fn = N.lib().lentils_bcb_apply if v.dtype == torch.float32 else N.lib().lentils_bcb_apply64
        N.check(fn(self._h, _ptr(v), _ptr(out), _stream_ptr()))
        return out.cpu().numpy().reshape(sp.nx, sp.ny) if host else out.reshape(sp.nx, sp.ny)

    _transpose = _forward
