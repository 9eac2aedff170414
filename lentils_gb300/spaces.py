"""Data spaces of the lensed visibility operator chain, mirroring the reference's
``lentils/common/space_base.py`` (same class names, constructor arguments, attributes and
array layouts). Each space *is* its C struct (a ctypes Structure subclass), as in the
reference, so it passes by value to the drop-in entry points.

Layouts (reference shapes):
  ImageSpace        (nchannels=1, nstokes=1, nx, ny)   float64, x-major     space_base.py:221-247
  FourierSpace      (1, 1, nu, nv//2 + 1)              complex128 r2c half  space_base.py:62-84
  VisibilitySpace   (nchannels, nstokes=1, nrows)      complex128           space_base.py:41-58
"""
from __future__ import annotations

from copy import deepcopy
from ctypes import POINTER, c_char, c_double

import numpy as np

from ._native import FourierSpaceC, ImageSpaceC, VisibilitySpaceC

ARCSEC_TO_RAD = 4.8481368111e-6  # lentils/common/space_base.py:82


class Space:
    """Base class: a shape and dtype (space_base.py:17-38)."""

    def __init__(self, shape=(0,), dtype=np.float64):
        self.shape = tuple(shape)
        self.dtype = dtype

    def new_vector(self, value=0.0):
        return np.full(self.shape, value, dtype=self.dtype)

    def copy(self):
        return deepcopy(self)

    @property
    def size(self):
        return int(np.prod(self.shape))

    @property
    def points(self):
        raise NotImplementedError

    def __repr__(self):
        return f"{type(self).__name__}{self.shape}"


class VisibilitySpace(Space, VisibilitySpaceC):
    """uv coordinates (rows of u, v, w in wavelengths) and channel scale factors."""

    def __init__(self, channels=(0.0,), uvcoords=np.array([0.0, 0.0, 0.0]), stokes=("I",)):
        VisibilitySpaceC.__init__(self)
        self.channels = np.array(channels, dtype=np.float64, order="C").flatten()
        self._c_channels = self.channels.ctypes.data_as(POINTER(c_double))
        self.num_channels = self.channels.shape[0]
        self.uvw = np.ascontiguousarray(np.array(uvcoords, dtype=np.float64).reshape((-1, 3)))
        self._c_uvw = self.uvw.ctypes.data_as(POINTER(c_double))
        self.num_rows = self.uvw.shape[0]
        self.num_stokes = len(stokes)
        if self.num_stokes != 1 or stokes[0] != "I":
            raise ValueError("Only stokes 'I' is allowed for now.")
        Space.__init__(self, shape=(self.num_channels, self.num_stokes, self.num_rows),
                       dtype=np.complex128)

    @property
    def points(self):
        return self.uvw


class FourierSpace(Space, FourierSpaceC):
    """r2c half-plane uv grid of an image space: du = 1/FOV_rad, phase centre at the image
    centre (space_base.py:62-84)."""

    def __init__(self, image_space, channels=(0.0,), stokes=("I",)):
        FourierSpaceC.__init__(self)
        self.nu, self.nv = image_space.nx, image_space.ny
        self.half_nv = self.nv // 2 + 1
        lx = ARCSEC_TO_RAD * (image_space.xmax - image_space.xmin)
        ly = ARCSEC_TO_RAD * (image_space.ymax - image_space.ymin)
        self.du = 1.0 / lx
        self.dv = 1.0 / ly
        self.gcx = ARCSEC_TO_RAD * 0.5 * (image_space.xmax + image_space.xmin)
        self.gcy = ARCSEC_TO_RAD * 0.5 * (image_space.ymax + image_space.ymin)
        self.channels = np.array(channels, dtype=np.float64, order="C").flatten()
        self._c_channels = self.channels.ctypes.data_as(POINTER(c_double))
        self.num_channels = 1
        self.num_stokes = 1
        Space.__init__(self, shape=(self.num_channels, self.num_stokes, self.nu, self.half_nv),
                       dtype=np.complex128)


class ImageSpace(Space, ImageSpaceC):
    """Regular pixel grid with bounds in arcsec; pixel positions at the lower-left corners
    (space_base.py:221-266). `mask` is a boolean array (the reference reads it from FITS;
    no FITS reader is bundled)."""

    def __init__(self, shape=(128, 128), bounds=((-1.0, 1.0), (-1.0, 1.0)), channels=(0.0,),
                 stokes=("I",), mask=None):
        ImageSpaceC.__init__(self)
        self.nx, self.ny = int(shape[0]), int(shape[1])
        self.num_channels = 1
        self.num_stokes = 1
        self.bounds = np.array(bounds, dtype=np.float64, order="C").flatten()
        self.xmin, self.xmax = self.bounds[0], self.bounds[1]
        self.ymin, self.ymax = self.bounds[2], self.bounds[3]
        self.dx = (self.xmax - self.xmin) / self.nx
        self.dy = (self.ymax - self.ymin) / self.ny
        self.channels = np.array(channels, dtype=np.float64, order="C").flatten()
        self._c_channels = self.channels.ctypes.data_as(POINTER(c_double))
        if mask is None:
            self.mask = np.ones((self.nx, self.ny), dtype=np.bool_)
        else:
            m = np.asarray(mask)
            if m.shape != (self.nx, self.ny):
                raise ValueError(f"mask shape {m.shape} != {(self.nx, self.ny)}")
            self.mask = np.ascontiguousarray(m.astype(np.bool_))
        self._c_mask = self.mask.ctypes.data_as(POINTER(c_char))
        Space.__init__(self, shape=(self.num_channels, self.num_stokes, self.nx, self.ny),
                       dtype=np.float64)

    @property
    def points(self):
        centers = np.zeros(self.shape[-2:] + (2,))
        centers[:, :, 0] = (self.xmin + self.dx * np.arange(self.nx))[:, None]
        centers[:, :, 1] = (self.ymin + self.dy * np.arange(self.ny))[None, :]
        return centers


class DelaunaySpace(Space):
    """Source space of Delaunay-triangulated points (lentils/common/space_base.py:139-158):
    `points` (N, 2), `triangles` (M, 3) and the scipy triangulation `delaunay`."""

    def __init__(self, points, channels=(0.0,), stokes=("I",)):
        from scipy.spatial import Delaunay
        self.num_channels, self.num_stokes = 1, 1
        self.delaunay = Delaunay(np.asarray(points, dtype=np.float64))
        self.edge = np.unique(self.delaunay.convex_hull.flatten())
        self.vertices = self.delaunay.points
        self.num_points = self.vertices.shape[0]
        self.triangles = self.delaunay.simplices
        self.num_triangles = self.triangles.shape[0]
        super().__init__(shape=(self.num_channels, self.num_stokes, self.num_points))

    @property
    def points(self):
        return self.vertices

