"""Lens models, mirroring lentils/models/lens_models.py: the same classes, constructor
arguments and C parameter packing (get_cpars, 320-byte generic_mass_model records), with the
deflection evaluated on the GPU through lentils_deflect_f64io.

Angular-diameter distances (GlobalLensModel.setup_raytracing, lens_models.py:38-48) do not
enter the PEMD, shear or multipole deflection formulas; they are left zero here (no astropy).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as N

# lentils/backend/load_backend.py:55-56
MASS_MODEL_DTYPE = np.dtype([("type", "u4"), ("_pad", "u4"), ("z_l", "f8"), ("z_s", "f8"),
                             ("d_l", "f8"), ("d_s", "f8"), ("d_ls", "f8"), ("sigma_c", "f8"),
                             ("beta", "f8"), ("fpars", "f8", 24), ("ipars", "i4", 8),
                             ("flags", "u1", 32)])


class MassModel:
    def get_cpars(self):
        raise NotImplementedError


class PowerLawEllipsoid(MassModel):
    """PEMD (type 0): lens_models.py:92-116. qh = (gamma - 1) / 2; th in degrees; f = q."""

    _my_ctype = 0

    def __init__(self, z=0.881000, b=0.463544, th=-14.278754, f=0.799362, x=-0.046847,
                 y=-0.105357, rc=0.000571, qh=0.506730):
        self.z, self.x, self.y, self.f, self.th, self.b, self.qh, self.rc = z, x, y, f, th, b, qh, rc

    def get_cpars(self):
        c = np.zeros(1, dtype=MASS_MODEL_DTYPE)[0]
        c["type"] = self._my_ctype
        c["z_l"] = self.z
        fp = c["fpars"]
        fp[0], fp[1], fp[2], fp[3] = self.x, self.y, self.f, self.th
        fp[4] = np.sin((self.th + 90) * np.pi / 180)
        fp[5] = np.cos((self.th + 90) * np.pi / 180)
        fp[6], fp[7], fp[8] = self.b, self.qh, self.rc
        return c


class ExternalPotential(MassModel):
    """External shear and convergence/shear gradients (type 1): lens_models.py:119-147."""

    _my_ctype = 1

    def __init__(self, z=0.881000, x=-0.046847, y=-0.105357, ss=-0.046500, sa=7.921300,
                 gks=0.0, gka=0.0, gss=0.0, gsa=0.0):
        self.z, self.x, self.y, self.ss, self.sa = z, x, y, ss, sa
        self.gks, self.gka, self.gss, self.gsa = gks, gka, gss, gsa

    def get_cpars(self):
        c = np.zeros(1, dtype=MASS_MODEL_DTYPE)[0]
        c["type"] = self._my_ctype
        c["z_l"] = self.z
        fp = c["fpars"]
        fp[0], fp[1], fp[2], fp[3] = self.x, self.y, self.ss, self.sa
        fp[4] = np.sin((self.sa + 90) * np.pi / 180)
        fp[5] = np.cos((self.sa + 90) * np.pi / 180)
        fp[6], fp[7] = self.gks, self.gka
        fp[8] = np.sin((self.gka + 90) * np.pi / 180)
        fp[9] = np.cos((self.gka + 90) * np.pi / 180)
        fp[10], fp[11] = self.gss, self.gsa
        fp[12] = np.sin((self.gsa + 90) * np.pi / 180)
        fp[13] = np.cos((self.gsa + 90) * np.pi / 180)
        return c


class InternalMultipoles(MassModel):
    """Internal multipoles of orders 3..order (type 2): lens_models.py:151-172."""

    _my_ctype = 2

    def __init__(self, z=0.881000, x=-0.046847, y=-0.105357, qh=0.5, order=4,
                 coefficients=((0.0, 0.0), (0.0, 0.0))):
        self.z, self.x, self.y, self.qh, self.order = z, x, y, qh, int(order)
        self.coefficients = np.array(coefficients, dtype=np.float64).reshape((order - 2, 2))

    def get_cpars(self):
        c = np.zeros(1, dtype=MASS_MODEL_DTYPE)[0]
        c["type"] = self._my_ctype
        c["z_l"] = self.z
        fp = c["fpars"]
        fp[0], fp[1], fp[2] = self.x, self.y, self.qh
        for i, v in enumerate(self.coefficients.flatten()):
            fp[3 + i] = v
        c["ipars"][0] = self.order
        return c


class GlobalLensModel:
    """A set of mass components deflecting a single source plane (lens_models.py:13-77)."""

    def __init__(self, components=None):
        self.components = []
        for comp in components or []:
            self.add_component(comp)
        self.lenses = np.zeros(0, dtype=MASS_MODEL_DTYPE)

    def add_component(self, component):
        self.components.append(component)

    def setup_raytracing(self, z_s):
        """Pack, sort by z_l and keep z_l < z_s (lens_models.py:31-35)."""
        lenses = np.zeros(len(self.components), dtype=MASS_MODEL_DTYPE)
        for i, comp in enumerate(self.components):
            lenses[i] = comp.get_cpars()
        lenses.sort(order="z_l")
        lenses = lenses[lenses["z_l"] < z_s]
        lenses["z_s"] = z_s
        self.lenses = np.ascontiguousarray(lenses)
        return self.lenses

    def deflect(self, points, z_s, deriv=False):
        """Source-plane positions of `points` (..., 2): numpy float64 in -> numpy out, or a CUDA
        tensor (float64 or float32) in -> CUDA tensor out. deriv=True also returns the
        per-point parameter derivatives d alpha / d (b, qh, q, x, y, th, ss, sa) summed over
        the lenses, shaped (8,) + points.shape like the reference allocates them
        (lens_models.py:71-73), in FP64 (lentils_deflect_grad)."""
        lenses = self.setup_raytracing(z_s)
        out = deflect_points(lenses, points)
        if not deriv:
            return out
        host = not isinstance(points, torch.Tensor)
        p = torch.as_tensor(np.ascontiguousarray(points, dtype=np.float64)).cuda() if host \
            else points.to(torch.float64).contiguous()
        g = torch.empty((8,) + tuple(p.shape), dtype=torch.float64, device=p.device)
        s = torch.cuda.current_stream()
        N.check(N.lib().lentils_deflect_grad(ctypes.c_void_p(lenses.ctypes.data), len(lenses),
                                             ctypes.c_void_p(p.data_ptr()),
                                             ctypes.c_void_p(g.data_ptr()), p.numel() // 2,
                                             ctypes.c_void_p(s.cuda_stream)))
        return out, (g.cpu().numpy() if host else g)


def deflect_points(lenses, points, stream=None):
    lenses = np.ascontiguousarray(lenses, dtype=MASS_MODEL_DTYPE)
    L = N.lib()
    host = not isinstance(points, torch.Tensor)
    p = torch.as_tensor(np.ascontiguousarray(points, dtype=np.float64)).cuda() if host else points.contiguous()
    out = torch.empty_like(p)
    s = torch.cuda.current_stream() if stream is None else stream
    fn = L.lentils_deflect_f32 if p.dtype == torch.float32 else L.lentils_deflect_f64io
    N.check(fn(ctypes.c_void_p(lenses.ctypes.data), len(lenses), ctypes.c_void_p(p.data_ptr()),
               ctypes.c_void_p(out.data_ptr()), p.numel() // 2, ctypes.c_void_p(s.cuda_stream)))
    return out.cpu().numpy() if host else out
