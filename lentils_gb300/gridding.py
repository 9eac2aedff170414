"""Device-resident Kaiser-Bessel gridding plan (PyTorch tensors over the C ABI).

A :class:`GriddingPlan` bins one uv set once (``lentils_plan_create``) and then applies
degridding (grid -> visibilities, the FORWARD direction of the reference's ``grid_cpu``,
lentils/backend/nufft.c:42-105) and gridding (the ADJOINT direction, nufft.c:106-118) on
complex64 CUDA tensors. Visibilities inside the plan are in plan order and plan frame;
:meth:`to_plan` / :meth:`from_plan` convert from/to the reference's row order.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as N


def _stream_ptr(stream=None):
    s = torch.cuda.current_stream() if stream is None else stream
    return ctypes.c_void_p(s.cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class GriddingPlan:
    """Binned visibility set for one uv grid.

    Parameters mirror the reference's Fourier / visibility spaces: (nu, nv) full grid size,
    (du, dv) cell size in wavelengths, (gcx, gcy) phase centre in radians, `wsup` the kernel
    half-width w and `kb_beta` the Kaiser-Bessel shape. `uvw` is (nrows, 3) float64 (numpy or
    a CUDA tensor), `channels` the per-channel scale factors.
    """

    def __init__(self, uvw, channels, nu, nv, du, dv, gcx=0.0, gcy=0.0, wsup=4, kb_beta=None,
                 tile=0, chunk=0, nyquist_guard=False, stream=None):
        L = N.lib()
        if kb_beta is None:
            kb_beta = np.pi * np.sqrt((2.0 * wsup / 2) ** 2 * 1.5 ** 2 - 0.8)
        self.nu, self.nv = int(nu), int(nv)
        self.half_nv = self.nv // 2 + 1
        self.wsup, self.kb_beta = int(wsup), float(kb_beta)
        self.du, self.dv, self.gcx, self.gcy = float(du), float(dv), float(gcx), float(gcy)
        desc = N.GridDescC(self.nu, self.nv, float(du), float(dv), float(gcx), float(gcy),
                           self.wsup, self.kb_beta, int(tile), int(chunk))
        flags = N.PLAN_NYQUIST_GUARD if nyquist_guard else 0
        if isinstance(uvw, torch.Tensor):
            uvw_t = uvw.to(dtype=torch.float64).contiguous()
            ch_t = torch.as_tensor(np.asarray(channels, dtype=np.float64).reshape(-1),
                                   device=uvw_t.device)
            nrows, nch = uvw_t.shape[0], ch_t.numel()
            uptr, cptr = _ptr(uvw_t), _ptr(ch_t)
            flags |= N.PLAN_UVW_ON_DEVICE
            keep = (uvw_t, ch_t)
        else:
            uvw_n = np.ascontiguousarray(np.asarray(uvw, dtype=np.float64).reshape(-1, 3))
            ch_n = np.ascontiguousarray(np.asarray(channels, dtype=np.float64).reshape(-1))
            nrows, nch = uvw_n.shape[0], ch_n.size
            uptr, cptr = ctypes.c_void_p(uvw_n.ctypes.data), ctypes.c_void_p(ch_n.ctypes.data)
            keep = (uvw_n, ch_n)
        self._handle = ctypes.c_void_p()
        N.check(L.lentils_plan_create(ctypes.byref(self._handle), ctypes.byref(desc), uptr,
                                      int(nrows), cptr, int(nch), flags, _stream_ptr(stream)))
        del keep
        self.nrows, self.nchannels = int(nrows), int(nch)
        self.nvis = self.nrows * self.nchannels

    # --- lifetime ----------------------------------------------------------------------
    def close(self):
        if getattr(self, "_handle", None) is not None and self._handle.value:
            N.lib().lentils_plan_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._handle

    def set_grid_variant(self, variant):
        """Work split of the gridding kernel (lentils_plan_set_grid_variant, 0-11); tuning only,
        equal results up to FP32 summation order."""
        N.check(N.lib().lentils_plan_set_grid_variant(self._handle, int(variant)))

    def set_degrid_variant(self, variant):
        """Form of the degridding kernel (lentils_plan_set_degrid_variant, 0-2); tuning only,
        identical results."""
        N.check(N.lib().lentils_plan_set_degrid_variant(self._handle, int(variant)))

    @property
    def stats(self):
        s = N.PlanStatsC()
        N.check(N.lib().lentils_plan_get_stats(self._handle, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    # --- operators (plan order, complex64 CUDA tensors) ----------------------------------
    def new_grid(self, device="cuda"):
        return torch.zeros((self.nu, self.half_nv), dtype=torch.complex64, device=device)

    def new_vis(self, device="cuda"):
        return torch.zeros(self.nvis, dtype=torch.complex64, device=device)

    def degrid(self, grid, out=None, stream=None):
        """Half-plane grid (nu, nv//2+1) complex64 -> plan-order visibilities (overwrites)."""
        assert grid.dtype == torch.complex64 and grid.numel() == self.nu * self.half_nv
        grid = grid.contiguous()
        if out is None:
            out = torch.empty(self.nvis, dtype=torch.complex64, device=grid.device)
        N.check(N.lib().lentils_degrid(self._handle, _ptr(grid), _ptr(out), _stream_ptr(stream)))
        return out

    def grid(self, vis, out=None, accumulate=False, stream=None):
        """Plan-order visibilities complex64 -> half-plane grid (accumulates into `out` when
        accumulate=True, else returns a fresh grid)."""
        assert vis.dtype == torch.complex64 and vis.numel() == self.nvis
        vis = vis.contiguous()
        if out is None:
            out = torch.zeros((self.nu, self.half_nv), dtype=torch.complex64, device=vis.device)
        elif not accumulate:
            out.zero_()
        N.check(N.lib().lentils_grid(self._handle, _ptr(vis), _ptr(out), _stream_ptr(stream)))
        return out

    def degrid64(self, grid, out=None, stream=None):
        """FP64 degridding (the double-precision operator): half-plane grid complex128 ->
        plan-order visibilities complex128 (overwrites)."""
        assert grid.dtype == torch.complex128 and grid.numel() == self.nu * self.half_nv
        grid = grid.contiguous()
        if out is None:
            out = torch.empty(self.nvis, dtype=torch.complex128, device=grid.device)
        N.check(N.lib().lentils_degrid64(self._handle, _ptr(grid), _ptr(out),
                                         _stream_ptr(stream)))
        return out

    def grid64(self, vis, out=None, stream=None):
        """FP64 gridding: plan-order visibilities complex128 -> a fresh half-plane grid
        complex128 (or accumulated into `out`)."""
        assert vis.dtype == torch.complex128 and vis.numel() == self.nvis
        vis = vis.contiguous()
        if out is None:
            out = torch.zeros((self.nu, self.half_nv), dtype=torch.complex128, device=vis.device)
        N.check(N.lib().lentils_grid64(self._handle, _ptr(vis), _ptr(out), _stream_ptr(stream)))
        return out

    def to_plan(self, vis_user, out=None, stream=None):
        """Reference row order (complex128 or complex64 CUDA tensor) -> plan order c64."""
        v = vis_user.contiguous().reshape(-1)
        assert v.numel() == self.nvis
        c128 = 1 if v.dtype == torch.complex128 else 0
        if not c128:
            assert v.dtype == torch.complex64
        if out is None:
            out = torch.empty(self.nvis, dtype=torch.complex64, device=v.device)
        N.check(N.lib().lentils_vis_to_plan(self._handle, _ptr(v), c128, _ptr(out),
                                            _stream_ptr(stream)))
        return out

    def from_plan(self, vis_plan, out=None, dtype=torch.complex128, accumulate=False,
                  stream=None):
        """Plan order c64 -> reference row order (complex128 by default)."""
        if out is None:
            out = torch.zeros(self.nvis, dtype=dtype, device=vis_plan.device)
        c128 = 1 if out.dtype == torch.complex128 else 0
        N.check(N.lib().lentils_vis_from_plan(self._handle, _ptr(vis_plan), _ptr(out), c128,
                                              1 if accumulate else 0, _stream_ptr(stream)))
        return out

    # --- host-buffer forms (numpy complex128, reference row order) ------------------------
    @staticmethod
    def _host(a, n, name):
        """Pointer of a contiguous complex128 host buffer: a numpy array or a CPU tensor
        (page-locked tensors take the direct path, pageable memory the staging copies)."""
        if isinstance(a, torch.Tensor):
            assert not a.is_cuda and a.dtype == torch.complex128 and a.is_contiguous(), name
            assert a.numel() == n, name
            return a, ctypes.c_void_p(a.data_ptr())
        a = np.ascontiguousarray(a, dtype=np.complex128)
        assert a.size == n, name
        return a, ctypes.c_void_p(a.ctypes.data)

    def degrid_host(self, grid, vis_out=None, accumulate=False, stream=None):
        """Reference-layout host buffers (numpy or CPU tensors, complex128): half-plane grid ->
        row-order visibilities, accumulated into vis_out when accumulate=True."""
        g, gp = self._host(grid, self.nu * self.half_nv, "grid")
        if vis_out is None:
            vis_out = np.zeros(self.nvis, dtype=np.complex128)
        if isinstance(vis_out, np.ndarray):
            assert vis_out.dtype == np.complex128 and vis_out.flags.c_contiguous
        vis_out, vp = self._host(vis_out, self.nvis, "vis_out")
        N.check(N.lib().lentils_degrid_host(self._handle, gp, vp, 1 if accumulate else 0,
                                            _stream_ptr(stream)))
        return vis_out

    def grid_host(self, vis, grid_out=None, accumulate=False, stream=None):
        """Row-order host visibilities -> half-plane host grid (accumulated when
        accumulate=True); buffers as for degrid_host."""
        v, vp = self._host(vis, self.nvis, "vis")
        if grid_out is None:
            grid_out = np.zeros((self.nu, self.half_nv), dtype=np.complex128)
        if isinstance(grid_out, np.ndarray):
            assert grid_out.dtype == np.complex128 and grid_out.flags.c_contiguous
        grid_out, gp = self._host(grid_out, self.nu * self.half_nv, "grid_out")
        N.check(N.lib().lentils_grid_host(self._handle, vp, gp, 1 if accumulate else 0,
                                          _stream_ptr(stream)))
        return grid_out


def grid_cpu(visspace, vis, gspace, grid, wsup, kb_beta, direction):
    """The drop-in ``grid_cpu`` (reference signature, numpy complex128 buffers, accumulate),
    executed on the GPU by liblentils_gb300. Raises LentilsError on failure."""
    assert vis.dtype == np.complex128 and vis.flags.c_contiguous
    assert grid.dtype == np.complex128 and grid.flags.c_contiguous
    N.lib().grid_cpu(visspace, ctypes.c_void_p(vis.ctypes.data), gspace,
                     ctypes.c_void_p(grid.ctypes.data), int(wsup), float(kb_beta),
                     int(direction))
    N.check_last()
