"""CPU oracle for the lensed visibility-operator chain.

TEST INFRASTRUCTURE ONLY. Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline / reference arm import this module, and only to compare results against or as the
timed CPU baseline. The product package ``lentils_gb300`` never imports it.

Two layers:

* ``liblentils_oracle.so`` (``oracle/lentils_oracle.c``): a plain-C restatement of the
  reference's FP64 C routines (``grid_cpu``, ``deflect_points``, ``grad_matrix_findiff_csr``,
  ``dft_matrix_csr``), pinned bit-for-bit against the reference's own sources compiled by
  ``oracle/Makefile`` into ``oracle/_ref/`` and against the committed fixtures in
  ``tests/golden/``.
* A numpy/scipy restatement of the reference's Python glue around them (spaces, zero padding,
  apodisation, r2c FFTs, operator composition, dataset weights), each function citing the
  reference file and lines it follows.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, Structure, c_char, c_double, c_int, c_void_p

import numpy as np
import scipy.fft as sfft
import scipy.sparse as sps

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)

# Constants as the reference defines them (lentils/backend/common.h:8-11,
# lentils/common/space_base.py:82).
ARCSEC_TO_RAD = 4.8481368111e-6
TWO_PI_TRUNC = 6.28318530718


# ---------------------------------------------------------------------------------------------
# ctypes mirrors of the by-value structs (lentils/backend/load_backend.py:27-57)
# ---------------------------------------------------------------------------------------------
class CImageSpace(Structure):
    _fields_ = [("nx", c_int), ("ny", c_int), ("nchannels", c_int), ("nstokes", c_int),
                ("xmin", c_double), ("xmax", c_double), ("ymin", c_double), ("ymax", c_double),
                ("dx", c_double), ("dy", c_double), ("channels", POINTER(c_double)),
                ("mask", POINTER(c_char))]


class CFourierSpace(Structure):
    _fields_ = [("nu", c_int), ("nv", c_int), ("half_nv", c_int), ("nchannels", c_int),
                ("nstokes", c_int), ("du", c_double), ("dv", c_double), ("gcx", c_double),
                ("gcy", c_double), ("channels", POINTER(c_double))]


class CVisibilitySpace(Structure):
    _fields_ = [("nrows", c_int), ("nchannels", c_int), ("nstokes", c_int),
                ("uv", POINTER(c_double)), ("channels", POINTER(c_double))]


class CDelaunaySpace(Structure):
    """delaunay_space, lentils/backend/common.h:24-35."""
    _fields_ = [("num_points", c_int), ("num_tris", c_int), ("nchannels", c_int),
                ("nstokes", c_int), ("channels", POINTER(c_double)), ("points", c_void_p),
                ("triangles", c_void_p)]


class CGlobalLensModel(Structure):
    _fields_ = [("num_lenses", c_int), ("num_zplanes", c_int), ("lenses", c_void_p)]


# lentils/backend/load_backend.py:55-56 (320 bytes per model)
MASS_MODEL_DTYPE = np.dtype([("type", "u4"), ("_pad", "u4"), ("z_l", "f8"), ("z_s", "f8"),
                             ("d_l", "f8"), ("d_s", "f8"), ("d_ls", "f8"), ("sigma_c", "f8"),
                             ("beta", "f8"), ("fpars", "f8", 24), ("ipars", "i4", 8),
                             ("flags", "u1", 32)])
assert MASS_MODEL_DTYPE.itemsize == 320


def _dp(a):
    return a.ctypes.data_as(POINTER(c_double))


# ---------------------------------------------------------------------------------------------
# library loading / building
# ---------------------------------------------------------------------------------------------
_PORT = None
_REF = {}


def build_port(quiet=True):
    """Compile oracle/lentils_oracle.c with oracle/Makefile (gcc, no GPU needed)."""
    out = subprocess.run(["make", "-C", HERE, "port"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


def reference_root():
    """Root of a Lentils checkout (the directory holding lentils/backend): the environment
    variable LENTILS_REFERENCE, else a checkout named ``reference`` beside this repository;
    None when neither exists."""
    for cand in (os.environ.get("LENTILS_REFERENCE"),
                 os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")):
        if cand and os.path.isdir(os.path.join(cand, "lentils", "backend")):
            return cand
    return None


def build_ref(ref_root=None):
    """Compile the reference's own nufft.c / deflect.c into oracle/_ref (only where the
    reference sources exist). Returns True when both libraries are present afterwards."""
    ref_root = ref_root or reference_root()
    if ref_root:
        subprocess.run(["make", "-C", HERE, "ref", f"REF={ref_root}"], capture_output=True,
                       text=True)
    return ref_available()


def ref_available():
    return all(os.path.exists(os.path.join(HERE, "_ref", n))
               for n in ("libref_nufft.so", "libref_deflect.so"))


def port_lib():
    global _PORT
    if _PORT is None:
        path = os.path.join(HERE, "liblentils_oracle.so")
        if not os.path.exists(path):
            build_port()
        lib = ctypes.CDLL(path)
        lib.oracle_grid.restype = None
        lib.oracle_grid.argtypes = [CVisibilitySpace, c_void_p, CFourierSpace, c_void_p, c_int,
                                    c_double, c_int]
        lib.oracle_deflect_points.restype = None
        lib.oracle_deflect_points.argtypes = [CGlobalLensModel, c_void_p, c_int, c_void_p]
        lib.oracle_grad_findiff_csr.restype = None
        lib.oracle_grad_findiff_csr.argtypes = [CImageSpace, c_void_p, c_void_p, c_void_p]
        lib.oracle_dft_dense.restype = None
        lib.oracle_dft_dense.argtypes = [CVisibilitySpace, CImageSpace, c_void_p]
        lib.oracle_bessel_i0.restype = c_double
        lib.oracle_bessel_i0.argtypes = [c_double]
        lib.oracle_kb_beta.restype = c_double
        lib.oracle_kb_beta.argtypes = [c_double, c_double]
        _PORT = lib
    return _PORT


def ref_lib(name):
    """The reference's compiled nufft / deflect library from oracle/_ref (None if absent)."""
    if name in _REF:
        return _REF[name]
    path = os.path.join(HERE, "_ref", f"libref_{name}.so")
    if not os.path.exists(path):
        return None
    lib = ctypes.CDLL(path)
    if name == "triangles":
        pass
    elif name == "nufft":
        lib.grid_cpu.restype = None
        lib.grid_cpu.argtypes = [CVisibilitySpace, c_void_p, CFourierSpace, c_void_p, c_int,
                                 c_double, c_int]
        lib.grad_matrix_findiff_csr.restype = None
        lib.grad_matrix_findiff_csr.argtypes = [CImageSpace, c_void_p, c_void_p, c_void_p]
    else:
        lib.deflect_points.restype = None
        lib.deflect_points.argtypes = [CGlobalLensModel, c_void_p, c_int, c_void_p, c_int,
                                       c_void_p]
    if name == "triangles":
        lib.delaunay_lens_matrix_csr.restype = None
        lib.delaunay_lens_matrix_csr.argtypes = [CImageSpace, CDelaunaySpace, c_int, c_void_p,
                                                 c_void_p, c_void_p, c_void_p, c_void_p]
    if name == "raster":
        lib.manifold_lens_matrix_csr.restype = None
        lib.manifold_lens_matrix_csr.argtypes = [CImageSpace, CImageSpace, CGlobalLensModel,
                                                 c_void_p, c_void_p, c_void_p]
    _REF[name] = lib
    return lib


# ---------------------------------------------------------------------------------------------
# Spaces (lentils/common/space_base.py)
# ---------------------------------------------------------------------------------------------
class ImageGeom:
    """Image-plane pixel grid; restates ImageSpace, space_base.py:221-247 (points are pixel
    lower-left corners, space_base.py:258-266)."""

    def __init__(self, shape, bounds, mask=None):
        self.nx, self.ny = int(shape[0]), int(shape[1])
        b = np.asarray(bounds, dtype=np.float64).reshape(-1)
        self.bounds = b.copy()
        self.xmin, self.xmax, self.ymin, self.ymax = b
        self.dx = (self.xmax - self.xmin) / self.nx
        self.dy = (self.ymax - self.ymin) / self.ny
        self.mask = (np.ones((self.nx, self.ny), dtype=np.bool_) if mask is None
                     else np.ascontiguousarray(mask, dtype=np.bool_))
        self._chan = np.zeros(1)

    @property
    def shape(self):
        return (self.nx, self.ny)

    def points(self):
        pts = np.zeros((self.nx, self.ny, 2))
        pts[:, :, 0] = (self.xmin + self.dx * np.arange(self.nx))[:, None]
        pts[:, :, 1] = (self.ymin + self.dy * np.arange(self.ny))[None, :]
        return pts

    def cstruct(self):
        s = CImageSpace()
        s.nx, s.ny, s.nchannels, s.nstokes = self.nx, self.ny, 1, 1
        s.xmin, s.xmax, s.ymin, s.ymax = self.xmin, self.xmax, self.ymin, self.ymax
        s.dx, s.dy = self.dx, self.dy
        s.channels = _dp(self._chan)
        self._maskbytes = np.ascontiguousarray(self.mask.astype(np.uint8))
        s.mask = self._maskbytes.ctypes.data_as(POINTER(c_char))
        return s


class FourierGeom:
    """r2c half-plane uv grid of an image space; restates FourierSpace, space_base.py:62-84."""

    def __init__(self, img: ImageGeom):
        self.nu, self.nv = img.nx, img.ny
        self.half_nv = self.nv // 2 + 1
        self.du = 1.0 / (ARCSEC_TO_RAD * (img.xmax - img.xmin))
        self.dv = 1.0 / (ARCSEC_TO_RAD * (img.ymax - img.ymin))
        self.gcx = ARCSEC_TO_RAD * 0.5 * (img.xmax + img.xmin)
        self.gcy = ARCSEC_TO_RAD * 0.5 * (img.ymax + img.ymin)
        self._chan = np.zeros(1)

    @property
    def shape(self):
        return (self.nu, self.half_nv)

    def cstruct(self):
        s = CFourierSpace()
        s.nu, s.nv, s.half_nv, s.nchannels, s.nstokes = self.nu, self.nv, self.half_nv, 1, 1
        s.du, s.dv, s.gcx, s.gcy = self.du, self.dv, self.gcx, self.gcy
        s.channels = _dp(self._chan)
        return s


class VisGeom:
    """uv coordinates and channel scale factors; restates VisibilitySpace,
    space_base.py:41-58. Visibility vectors are (nchannels * nrows) complex, row index fastest
    (nufft.c:97)."""

    def __init__(self, uvw, channels=(1.0,)):
        self.uvw = np.ascontiguousarray(np.asarray(uvw, dtype=np.float64).reshape(-1, 3))
        self.channels = np.ascontiguousarray(np.asarray(channels, dtype=np.float64).reshape(-1))
        self.nrows = self.uvw.shape[0]
        self.nchannels = self.channels.shape[0]

    @property
    def nvis(self):
        return self.nrows * self.nchannels

    def cstruct(self):
        s = CVisibilitySpace()
        s.nrows, s.nchannels, s.nstokes = self.nrows, self.nchannels, 1
        s.uv = _dp(self.uvw)
        s.channels = _dp(self.channels)
        return s


def padded_geom(img: ImageGeom, pad_factor=2):
    """Zero-padded image space; restates ZeroPaddingOperator.__init__,
    fourier_operators.py:29-42. Returns (padded geometry, padx, pady)."""
    p = int(pad_factor)
    padx = ((p - 1) * img.nx + 1) // 2
    pady = ((p - 1) * img.ny + 1) // 2
    bounds = img.bounds + np.array([-padx * img.dx, padx * img.dx, -pady * img.dy,
                                    pady * img.dy])
    return ImageGeom((img.nx + 2 * padx, img.ny + 2 * pady), bounds), padx, pady


def kb_beta(wsup, pad_factor=2):
    """Beatty et al. shape parameter as NUFFTOperator computes it (fourier_operators.py:104-108,
    exact pi)."""
    return np.pi * np.sqrt((2.0 * wsup / pad_factor) ** 2 * (pad_factor - 0.5) ** 2 - 0.8)


def apodization(img: ImageGeom, padded: ImageGeom, beta, wsup):
    """Grid-correction diagonal 1/(sinhc_x outer sinhc_y); restates
    ApodizationCorrectionOperator, fourier_operators.py:54-68."""
    cx = (np.arange(img.nx) - 0.5 * img.nx) / padded.nx
    cy = (np.arange(img.ny) - 0.5 * img.ny) / padded.ny
    ax = np.sqrt(beta ** 2 - (2 * np.pi * wsup * cx) ** 2)
    ay = np.sqrt(beta ** 2 - (2 * np.pi * wsup * cy) ** 2)
    return 1.0 / np.outer(np.sinh(ax) / ax, np.sinh(ay) / ay)


def nyquist_ok(vis: VisGeom, four: FourierGeom, wsup):
    """The guard of GriddingOperator.__init__, fourier_operators.py:77-80."""
    iumax = np.max(vis.channels) * np.max(np.abs(vis.uvw[:, 0])) / four.du
    ivmax = np.max(vis.channels) * np.max(np.abs(vis.uvw[:, 1])) / four.dv
    return not (iumax + wsup + 1 > 0.5 * four.nu or ivmax + wsup + 1 > 0.5 * four.nv)


# ---------------------------------------------------------------------------------------------
# Gridder wrappers (port by default, compiled reference on request)
# ---------------------------------------------------------------------------------------------
def grid_cpu(vis: VisGeom, visbuf, four: FourierGeom, gridbuf, wsup, beta, direction,
             use_ref=False):
    """Call grid_cpu (reference) or oracle_grid (port) on complex128 buffers in place
    (accumulating, nufft.c:42-122)."""
    assert visbuf.dtype == np.complex128 and visbuf.flags.c_contiguous
    assert gridbuf.dtype == np.complex128 and gridbuf.flags.c_contiguous
    assert visbuf.size == vis.nvis and gridbuf.size == four.nu * four.half_nv
    vs, gs = vis.cstruct(), four.cstruct()
    if use_ref:
        lib = ref_lib("nufft")
        if lib is None:
            raise RuntimeError("compiled reference not available (oracle/_ref)")
        lib.grid_cpu(vs, visbuf.ctypes.data, gs, gridbuf.ctypes.data, int(wsup), float(beta),
                     int(direction))
    else:
        port_lib().oracle_grid(vs, visbuf.ctypes.data, gs, gridbuf.ctypes.data, int(wsup),
                               float(beta), int(direction))


def degrid(vis: VisGeom, four: FourierGeom, grid, wsup, beta, use_ref=False):
    """GriddingOperator._matrixfree_forward (fourier_operators.py:85-88): fresh zeros, FORWARD."""
    out = np.zeros(vis.nvis, dtype=np.complex128)
    g = np.ascontiguousarray(grid, dtype=np.complex128)
    grid_cpu(vis, out, four, g, wsup, beta, 0, use_ref)
    return out


def grid(vis: VisGeom, four: FourierGeom, visdata, wsup, beta, use_ref=False):
    """GriddingOperator._matrixfree_transpose (fourier_operators.py:90-93): fresh zeros,
    ADJOINT."""
    out = np.zeros((four.nu, four.half_nv), dtype=np.complex128)
    v = np.ascontiguousarray(visdata, dtype=np.complex128)
    grid_cpu(vis, v, four, out, wsup, beta, 1, use_ref)
    return out


class NufftOracle:
    """NUFFT = Gridder . rFFT2 . ZeroPad . Apod and its transpose; restates NUFFTOperator,
    fourier_operators.py:96-126, with FFTOperator (:12-24, rfft2 norm='backward', irfft2
    norm='forward') and ZeroPaddingOperator (:44-52)."""

    def __init__(self, vis: VisGeom, img: ImageGeom, pad_factor=2, wsup=4, beta=None,
                 use_ref=False):
        self.vis, self.img = vis, img
        self.wsup = int(wsup)
        self.beta = kb_beta(self.wsup, pad_factor) if beta is None else float(beta)
        self.padded, self.padx, self.pady = padded_geom(img, pad_factor)
        self.four = FourierGeom(self.padded)
        self.apod = apodization(img, self.padded, self.beta, self.wsup)
        self.use_ref = use_ref

    def zpad(self, x):
        out = np.zeros(self.padded.shape)
        out[self.padx:self.padx + self.img.nx, self.pady:self.pady + self.img.ny] = x
        return out

    def crop(self, x):
        return x[self.padx:self.padx + self.img.nx, self.pady:self.pady + self.img.ny].copy()

    def forward_grid(self, image):
        """Image -> half-plane grid (everything but the gridder)."""
        x = self.apod * np.asarray(image, dtype=np.float64).reshape(self.img.shape)
        return sfft.rfft2(self.zpad(x), s=self.padded.shape, norm="backward")

    def forward(self, image):
        return degrid(self.vis, self.four, self.forward_grid(image), self.wsup, self.beta,
                      self.use_ref)

    def adjoint_from_grid(self, g):
        x = sfft.irfft2(g, s=self.padded.shape, norm="forward")
        return self.apod * self.crop(x)

    def adjoint(self, visdata):
        return self.adjoint_from_grid(grid(self.vis, self.four, visdata, self.wsup, self.beta,
                                           self.use_ref))


def beam_geom(img: ImageGeom):
    """Beam space of an image: 2nx x 2ny pixels, bounds +-(nx dx, ny dy); restates
    RadioDataset._make_beam_space, data_base.py:147-158."""
    rx, ry = img.dx * img.nx, img.dy * img.ny
    return ImageGeom((2 * img.nx, 2 * img.ny), [(-rx, rx), (-ry, ry)])


def dirty_beam(vis: VisGeom, img: ImageGeom, weights, wsup=4, beta=None):
    """NUFFT_beam^T C^-1 1 on the beam space; restates RadioDataset.dirty_beam,
    data_base.py:160-172."""
    nb = NufftOracle(vis, beam_geom(img), 2, wsup, beta)
    return nb.adjoint(np.asarray(weights, dtype=np.float64) + 0.0j)


def bcb_apply(beam, img: ImageGeom, x):
    """Blurred covariance F^T C^-1 F x as the dirty-beam convolution; restates
    RadioDataset.blurred_covariance_operator, data_base.py:115-129: zero padding by
    ((p-1)n+1)//2 per side (fourier_operators.py:33-47), rfft2 (norm 'backward'), the spectrum
    of the beam rolled by half the padded size over the padded pixel count, irfft2 (norm
    'forward'), crop."""
    nx, ny = img.nx, img.ny
    padx, pady = (nx + 1) // 2, (ny + 1) // 2
    shape = (nx + 2 * padx, ny + 2 * pady)
    z = np.zeros(shape)
    z[padx:padx + nx, pady:pady + ny] = np.asarray(x, dtype=np.float64).reshape(nx, ny)
    db = np.roll(np.asarray(beam, dtype=np.float64).reshape(shape),
                 [shape[0] // 2, shape[1] // 2], axis=[-2, -1])
    dbfft = sfft.rfft2(db, norm="backward") / np.prod(db.shape)
    y = sfft.irfft2(dbfft * sfft.rfft2(z, norm="backward"), s=shape, norm="forward")
    return y[padx:padx + nx, pady:pady + ny].copy()


def dft_matrix(vis: VisGeom, img: ImageGeom):
    """Dense DFT matrix (2*nrows x npix, rows cos/sin interleaved); restates dft_matrix_csr,
    nufft.c:128-161, densely (masked columns zero)."""
    mat = np.zeros((2 * vis.nrows, img.nx * img.ny))
    port_lib().oracle_dft_dense(vis.cstruct(), img.cstruct(), mat.ctypes.data)
    return mat


def dft_forward(mat, image):
    """DFTOperator * image, viewed as complex (operator_base.py:96-101)."""
    return (mat @ np.asarray(image, dtype=np.float64).reshape(-1)).view(np.complex128)


def dft_adjoint(mat, visdata):
    """DFTOperator.T * vis: the real transpose applied to the interleaved vector."""
    v = np.ascontiguousarray(visdata, dtype=np.complex128).view(np.float64)
    return mat.T @ v


def grad_csr(img: ImageGeom, use_ref=False):
    """Gradient CSR (2*npix x npix); restates grad_matrix_findiff_csr and its allocation in
    PriorCovarianceOperator, operator_base.py:225-230."""
    n = img.nx * img.ny
    rows = np.zeros(2 * n + 1, dtype=np.int32)
    cols = np.zeros(4 * n, dtype=np.int32)
    vals = np.zeros(4 * n, dtype=np.float64)
    if use_ref:
        ref_lib("nufft").grad_matrix_findiff_csr(img.cstruct(), rows.ctypes.data,
                                                 cols.ctypes.data, vals.ctypes.data)
    else:
        port_lib().oracle_grad_findiff_csr(img.cstruct(), rows.ctypes.data, cols.ctypes.data,
                                           vals.ctypes.data)
    return rows, cols, vals


def regulariser(img: ImageGeom, strength):
    """lambda * R^T R for the 'gradient' prior; restates PriorCovarianceOperator,
    operator_base.py:225-242."""
    rows, cols, vals = grad_csr(img)
    n = img.nx * img.ny
    r = sps.csr_matrix((vals, cols, rows), shape=(2 * n, n))
    return (strength * (r.T @ r)).tocsr()


# ---------------------------------------------------------------------------------------------
# Lens models (lentils/models/lens_models.py)
# ---------------------------------------------------------------------------------------------
def pemd_cpars(b, th, f, x, y, qh, rc=0.0, z=0.5):
    """PowerLawEllipsoid.get_cpars, lens_models.py:102-116."""
    m = np.zeros(1, dtype=MASS_MODEL_DTYPE)[0]
    m["type"] = 0
    m["z_l"] = z
    fp = m["fpars"]
    fp[0], fp[1], fp[2], fp[3] = x, y, f, th
    fp[4] = np.sin((th + 90) * np.pi / 180)
    fp[5] = np.cos((th + 90) * np.pi / 180)
    fp[6], fp[7], fp[8] = b, qh, rc
    return m


def shear_cpars(x, y, ss, sa, gks=0.0, gka=0.0, gss=0.0, gsa=0.0, z=0.5):
    """ExternalPotential.get_cpars, lens_models.py:129-147."""
    m = np.zeros(1, dtype=MASS_MODEL_DTYPE)[0]
    m["type"] = 1
    m["z_l"] = z
    fp = m["fpars"]
    fp[0], fp[1], fp[2], fp[3] = x, y, ss, sa
    fp[4] = np.sin((sa + 90) * np.pi / 180)
    fp[5] = np.cos((sa + 90) * np.pi / 180)
    fp[6], fp[7] = gks, gka
    fp[8] = np.sin((gka + 90) * np.pi / 180)
    fp[9] = np.cos((gka + 90) * np.pi / 180)
    fp[10], fp[11] = gss, gsa
    fp[12] = np.sin((gsa + 90) * np.pi / 180)
    fp[13] = np.cos((gsa + 90) * np.pi / 180)
    return m


def multipole_cpars(x, y, qh, order, coefficients, z=0.5):
    """InternalMultipoles.get_cpars, lens_models.py:161-172."""
    m = np.zeros(1, dtype=MASS_MODEL_DTYPE)[0]
    m["type"] = 2
    m["z_l"] = z
    fp = m["fpars"]
    fp[0], fp[1], fp[2] = x, y, qh
    c = np.asarray(coefficients, dtype=np.float64).reshape(-1)
    fp[3:3 + c.size] = c
    m["ipars"][0] = order
    return m


def lens_array(models, z_s=None):
    """Structured array of mass models, sorted by z_l and cut to z_l < z_s as
    GlobalLensModel.setup_raytracing does (lens_models.py:31-35). Distances are not filled:
    they do not enter the deflection formulas."""
    arr = np.array(list(models), dtype=MASS_MODEL_DTYPE)
    arr.sort(order="z_l")
    if z_s is not None:
        arr = arr[arr["z_l"] < z_s]
    return np.ascontiguousarray(arr)


def deflect(lenses, points, use_ref=False):
    """GlobalLensModel.deflect (lens_models.py:64-77) through deflect_points (reference) or
    oracle_deflect_points (port). points: (..., 2) float64."""
    lenses = np.ascontiguousarray(lenses, dtype=MASS_MODEL_DTYPE)
    pts = np.ascontiguousarray(points, dtype=np.float64)
    n = pts.size // 2
    out = np.zeros_like(pts)
    glm = CGlobalLensModel()
    glm.num_lenses = lenses.shape[0]
    glm.num_zplanes = 1
    glm.lenses = lenses.ctypes.data
    if use_ref:
        lib = ref_lib("deflect")
        if lib is None:
            raise RuntimeError("compiled reference not available (oracle/_ref)")
        dummy = np.zeros(1)
        lib.deflect_points(glm, pts.ctypes.data, n, out.ctypes.data, 0, dummy.ctypes.data)
    else:
        port_lib().oracle_deflect_points(glm, pts.ctypes.data, n, out.ctypes.data)
    return out


def manifold_lens_matrix_ref(img: ImageGeom, src: ImageGeom, lenses):
    """The compiled reference's ManifoldLensOperator matrix (manifold_lens_matrix_csr,
    raster.c:272-395, called as lens_operators.py:21-38 does): (row_inds, cols, vals) with
    nnz = row_inds[-1]. Needs oracle/_ref."""
    lib = ref_lib("raster")
    if lib is None:
        raise RuntimeError("compiled reference not available (oracle/_ref)")
    lenses = np.ascontiguousarray(lenses, dtype=MASS_MODEL_DTYPE)
    glm = CGlobalLensModel()
    glm.num_lenses = lenses.shape[0]
    glm.num_zplanes = 1
    glm.lenses = lenses.ctypes.data
    nrows = img.nx * img.ny
    rows = np.zeros(nrows + 1, dtype=np.int32)
    cols = np.zeros(50 * nrows, dtype=np.int32)
    vals = np.zeros(50 * nrows, dtype=np.float64)
    ic, sc = img.cstruct(), src.cstruct()
    lib.manifold_lens_matrix_csr(ic, sc, glm, rows.ctypes.data, cols.ctypes.data,
                                 vals.ctypes.data)
    nnz = int(rows[-1])
    return rows, cols[:nnz].copy(), vals[:nnz].copy()


def delaunay_lens_matrix_ref(img: ImageGeom, ncast, casted_points, uncasted_points,
                             triangles, tri_inds):
    """The compiled reference's delaunay_lens_matrix_csr (triangles.c:105-140) for a given
    triangulation of the casted points and point location of the uncasted ones (the reference
    takes both from scipy's Delaunay, lens_operators.py:67-70): (row_inds, cols, vals)."""
    lib = ref_lib("triangles")
    if lib is None:
        raise RuntimeError("compiled reference not available (oracle/_ref)")
    cp = np.ascontiguousarray(casted_points, dtype=np.float64).reshape(-1, 2)
    up = np.ascontiguousarray(uncasted_points, dtype=np.float64).reshape(-1, 2)
    tr = np.ascontiguousarray(triangles, dtype=np.int32).reshape(-1, 3)
    ti = np.ascontiguousarray(tri_inds, dtype=np.int32).reshape(-1)
    ds = CDelaunaySpace()
    ds.num_points, ds.num_tris, ds.nchannels, ds.nstokes = cp.shape[0], tr.shape[0], 1, 1
    ds.points, ds.triangles = cp.ctypes.data, tr.ctypes.data
    n = img.nx * img.ny
    rows = np.zeros(n + 1, np.int32)
    cols = np.zeros(cp.shape[0] + 3 * up.shape[0] + 1, np.int32)
    vals = np.zeros(cols.size)
    lib.delaunay_lens_matrix_csr(img.cstruct(), ds, int(ncast), up.ctypes.data, ti.ctypes.data,
                                 rows.ctypes.data, cols.ctypes.data, vals.ctypes.data)
    nnz = int(rows[-1])
    return rows, cols[:nnz].copy(), vals[:nnz].copy()


def deflect_derivatives_ref(lenses, points):
    """The compiled reference's want_deriv output (deflect_points, deflect.c:26-66,243-339):
    (the 12 numbers it accumulates over all points in one call, and the same 12 numbers per
    point from one-point calls). Needs oracle/_ref."""
    lenses = np.ascontiguousarray(lenses, dtype=MASS_MODEL_DTYPE)
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 2)
    lib = ref_lib("deflect")
    if lib is None:
        raise RuntimeError("compiled reference not available (oracle/_ref)")
    glm = CGlobalLensModel()
    glm.num_lenses = lenses.shape[0]
    glm.num_zplanes = 1
    glm.lenses = lenses.ctypes.data
    out = np.zeros_like(pts)
    total = np.zeros(16)
    lib.deflect_points(glm, pts.ctypes.data, pts.shape[0], out.ctypes.data, 1, total.ctypes.data)
    per = np.zeros((pts.shape[0], 12))
    one = np.zeros(2)
    for p in range(pts.shape[0]):
        d = np.zeros(16)
        lib.deflect_points(glm, pts[p].ctypes.data, 1, one.ctypes.data, 1, d.ctypes.data)
        per[p] = d[:12]
    assert not np.any(total[12:])
    return total[:12], per


# ---------------------------------------------------------------------------------------------
# Bilinear lens operator and the CG normal equations (no reference counterpart for the
# bilinear interpolation; the CG pattern follows lentils/tests/solver_tests.py:77-114)
# ---------------------------------------------------------------------------------------------
def bilinear_lens_matrix(src_points, img_mask, src: ImageGeom):
    """Sparse L (npix_image x npix_source): each unmasked image pixel whose deflected position
    falls inside the source node lattice interpolates bilinearly from the four surrounding
    source nodes (nodes at the pixel corners xmin + j*dx, as ImageSpace.points places them).
    Pixels outside the lattice or masked give empty rows."""
    p = np.asarray(src_points, dtype=np.float64).reshape(-1, 2)
    m = np.asarray(img_mask, dtype=np.bool_).reshape(-1)
    fx = (p[:, 0] - src.xmin) / src.dx
    fy = (p[:, 1] - src.ymin) / src.dy
    with np.errstate(invalid="ignore"):
        j0 = np.floor(fx)
        k0 = np.floor(fy)
    ok = m & np.isfinite(fx) & np.isfinite(fy) & (j0 >= 0) & (j0 <= src.nx - 2) & \
        (k0 >= 0) & (k0 <= src.ny - 2)
    rows = np.nonzero(ok)[0]
    j0 = j0[ok].astype(np.int64)
    k0 = k0[ok].astype(np.int64)
    tx = fx[ok] - j0
    ty = fy[ok] - k0
    cols = np.stack([j0 * src.ny + k0, (j0 + 1) * src.ny + k0, j0 * src.ny + k0 + 1,
                     (j0 + 1) * src.ny + k0 + 1], axis=1)
    vals = np.stack([(1 - tx) * (1 - ty), tx * (1 - ty), (1 - tx) * ty, tx * ty], axis=1)
    mat = sps.csr_matrix((vals.reshape(-1), (np.repeat(rows, 4), cols.reshape(-1))),
                         shape=(p.shape[0], src.nx * src.ny))
    return mat


def normal_operator(img: ImageGeom, src: ImageGeom, uvw, src_points, weights, lam, wsup=4,
                    beta=None):
    """The FP64 normal equations of the CG source inversion, visibility form:
    A s = M^T F^T C^-1 F M s + lam R^T R s and rhs(d) = M^T F^T C^-1 d, with M the bilinear
    lens matrix, F the NUFFT (NufftOracle) and C^-1 = diag(weights); restates
    lhs = lensop.T * (nufft.T * C^-1 * nufft) * lensop + reg_op (solver_tests.py:97-99,
    operator_base.py:116-175, data_base.py:36-44). Returns (A, rhs, M, R)."""
    vis = VisGeom(uvw, [1.0])
    ora = NufftOracle(vis, img, 2, wsup, beta)
    M = bilinear_lens_matrix(src_points, img.mask, src)
    R = regulariser(src, lam)
    w = np.asarray(weights, dtype=np.float64)

    def A(s):
        return M.T @ ora.adjoint(w * ora.forward((M @ s).reshape(img.shape))).reshape(-1) + R @ s

    def rhs(d):
        return M.T @ ora.adjoint(w * d).reshape(-1)
    return A, rhs, M, R


def normal_operator_bcb(img: ImageGeom, src: ImageGeom, uvw, src_points, weights, lam,
                        wsup=4, beta=None):
    """The same normal equations with the dirty-beam data term, the reference's production
    form: A s = M^T BCB(M s) + lam R^T R s with BCB the blurred covariance (bcb_apply of the
    dirty beam), rhs(d) = M^T (dirty image F^T C^-1 d) (data_base.py:115-172,
    solver_tests.py:97-99). Returns (A, rhs, M, R)."""
    vis = VisGeom(uvw, [1.0])
    w = np.asarray(weights, dtype=np.float64)
    beam = dirty_beam(vis, img, w, wsup, beta)
    ora = NufftOracle(vis, img, 2, wsup, beta)
    M = bilinear_lens_matrix(src_points, img.mask, src)
    R = regulariser(src, lam)

    def A(s):
        return M.T @ bcb_apply(beam, img, (M @ s).reshape(img.shape)).reshape(-1) + R @ s

    def rhs(d):
        return M.T @ ora.adjoint(w * d).reshape(-1)
    return A, rhs, M, R


def jacobi_inverse_diagonal(M, R, weights):
    """1 / diag(wsum M^T M + R^T R) with wsum the sum of the data weights (the dirty beam's
    peak): the diagonal of the matrix whose factorisation the reference's radio CG uses as its
    preconditioner, reg_op + wtsum * L^T L (solver_tests.py:103-106)."""
    wsum = float(np.sum(np.abs(weights)))
    d = wsum * np.asarray(M.multiply(M).sum(axis=0)).reshape(-1) + R.diagonal()
    out = np.zeros_like(d)
    out[d > 0] = 1.0 / d[d > 0]
    return out


def max_relative_error(a, b):
    """lentils/tests/test_utils.py:12-19 (relative to max |b|)."""
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128).reshape(-1)
    b = np.asarray(b, dtype=np.complex128).reshape(-1)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


# ---------------------------------------------------------------------------------------------
# Seeded synthetic inputs with the benchmark shapes
# ---------------------------------------------------------------------------------------------
def synth_uv(rng, nvis, four: FourierGeom, frac, wsup):
    """uv points with areal density ~ 1/|uv| (radius uniform, angle uniform) out to
    `frac` of the grid's Nyquist extent, clipped inside the Nyquist guard of
    fourier_operators.py:77-80. Returns (nvis, 3) with w = 0; channel scale 1."""
    rmax_u = frac * 0.5 * four.nu * four.du
    rmax_v = frac * 0.5 * four.nv * four.dv
    r = rng.uniform(0.0, 1.0, nvis)
    th = rng.uniform(0.0, 2 * np.pi, nvis)
    uvw = np.zeros((nvis, 3))
    uvw[:, 0] = r * np.cos(th) * rmax_u
    uvw[:, 1] = r * np.sin(th) * rmax_v
    return _clip_guard(uvw, four, wsup)


def _clip_guard(uvw, four, wsup):
    lim_u = (0.5 * four.nu - wsup - 1.0 - 1e-6) * four.du
    lim_v = (0.5 * four.nv - wsup - 1.0 - 1e-6) * four.dv
    uvw[:, 0] = np.clip(uvw[:, 0], -lim_u, lim_u)
    uvw[:, 1] = np.clip(uvw[:, 1], -lim_v, lim_v)
    return uvw


def synth_uv_blobs(rng, nvis, four: FourierGeom, frac, wsup, nblobs=50, blob_frac=0.1,
                   blob_width=0.005):
    """As synth_uv, with `blob_frac` of the points in `nblobs` Gaussian blobs of standard
    deviation blob_width * (nu/2) cells, centres drawn by the same radial law."""
    nb = int(round(blob_frac * nvis))
    base = synth_uv(rng, nvis - nb, four, frac, wsup)
    centres = synth_uv(rng, nblobs, four, frac, wsup)
    which = rng.integers(0, nblobs, nb)
    blobs = np.zeros((nb, 3))
    blobs[:, 0] = centres[which, 0] + rng.normal(0, blob_width * 0.5 * four.nu * four.du, nb)
    blobs[:, 1] = centres[which, 1] + rng.normal(0, blob_width * 0.5 * four.nv * four.dv, nb)
    out = np.concatenate([base, _clip_guard(blobs, four, wsup)])
    return np.ascontiguousarray(out[rng.permutation(out.shape[0])])


def complex_normal(rng, n, sigma=1.0):
    return (rng.normal(0, sigma, n) + 1j * rng.normal(0, sigma, n)).astype(np.complex128)
