"""The CG source-inversion workload: a 512^2 image plane (0.01 arcsec pixels) lensed by a PEMD
(b = 1.2, q = 0.7, gamma = 2.0) plus external shear (0.05, 20 deg) onto a 128^2 regular source
grid (+-0.64 arcsec) with bilinear interpolation, 2e6 visibilities (density ~ 1/|uv| to 0.45 of
Nyquist) with complex Gaussian noise sigma = 1 and a 'gradient' regulariser lambda = 1e-2.
Mirrors the reference's solver-test pattern (lentils/tests/solver_tests.py:77-114) at
benchmark size, on seeded synthetic data.
"""
from __future__ import annotations

import numpy as np

IMG, PIX, SRC, SRC_HALF, NVIS, LAMBDA = 512, 0.01, 128, 0.64, 2_000_000, 1e-2
Z_LENS, Z_SRC = 0.5, 2.0
SEED = 1241
DESCRIPTION = ("CG source inversion: 512^2 image (0.01\"), 128^2 source, 2e6 vis, PEMD b=1.2 "
               "q=0.7 gamma=2 + shear (0.05, 20 deg), lambda=1e-2")


def geometry(seed=SEED, nvis=NVIS):
    """(visibility space, image space, source space, uvw) of the workload."""
    from .spaces import ImageSpace, VisibilitySpace
    from .synthetic import padded_fourier_space, synth_uv
    rng = np.random.default_rng(seed)
    half = 0.5 * IMG * PIX
    ims = ImageSpace((IMG, IMG), [(-half, half), (-half, half)])
    srcs = ImageSpace((SRC, SRC), [(-SRC_HALF, SRC_HALF), (-SRC_HALF, SRC_HALF)])
    four = padded_fourier_space(ims, 2)
    uvw = synth_uv(rng, nvis, four, 0.45, 4)
    vs = VisibilitySpace(channels=[1.0], uvcoords=uvw)
    return vs, ims, srcs, uvw, rng


def lens_model():
    """The workload's lens, centred a quarter pixel off the pixel corners (the PEMD deflection
    is singular at its centre)."""
    from .lens_models import ExternalPotential, GlobalLensModel, PowerLawEllipsoid
    c = 0.25 * PIX
    return GlobalLensModel([PowerLawEllipsoid(z=Z_LENS, b=1.2, th=0.0, f=0.7, x=c, y=c, rc=0.0,
                                              qh=0.5),
                            ExternalPotential(z=Z_LENS, x=c, y=c, ss=0.05, sa=20.0)])


def two_blob_source(srcs):
    xs = (srcs.xmin + srcs.dx * np.arange(srcs.nx))[:, None]
    ys = (srcs.ymin + srcs.dy * np.arange(srcs.ny))[None, :]
    return (np.exp(-((xs - 0.05) ** 2 + (ys - 0.02) ** 2) / (2 * 0.06 ** 2))
            + 0.5 * np.exp(-((xs + 0.1) ** 2 + (ys + 0.08) ** 2) / (2 * 0.04 ** 2)))


def simulate(nufft, ims, srcs, glm, s_true, rng, sigma=1.0, z_src=Z_SRC):
    """Visibilities F L s_true + CN(0, sigma^2) noise (FP64 operators on the GPU)."""
    from .operators import BilinearLensOperator
    from .synthetic import complex_normal
    L = BilinearLensOperator(ims, srcs, glm, z_src=z_src)
    model = nufft * (L * s_true)
    del L
    return model.reshape(-1) + complex_normal(rng, model.size, sigma)


def inversion(seed=SEED, nufft=None, data_term="visibilities"):
    """(SourceInversion of the workload, shared NUFFT operator, geometry tuple); data_term
    "bcb" uses the dirty-beam form of F^T C^-1 F."""
    from .inversion import SourceInversion
    from .operators import NUFFTOperator
    vs, ims, srcs, uvw, rng = geometry(seed)
    F = nufft if nufft is not None else NUFFTOperator(vs, ims)
    glm = lens_model()
    d = simulate(F, ims, srcs, glm, two_blob_source(srcs), rng)
    inv = SourceInversion(vs, d, 1.0, ims, srcs, glm, Z_SRC, LAMBDA, nufft=F,
                          data_term=data_term)
    return inv, F, (vs, ims, srcs, uvw)
