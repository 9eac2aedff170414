"""Seeded synthetic visibility sets for benchmarks, training data and examples.

uv points have areal density proportional to 1/|uv| (radius and angle uniform) out to a
fraction of the grid's Nyquist extent, optionally with a share of the points in dense Gaussian
blobs, and are clipped inside the Nyquist guard of the gridding operator
(lentils/operators/fourier_operators.py:77-80: |u|/du + w + 1 <= nu/2). w = 0, one channel
of scale 1.0.
"""
from __future__ import annotations

import numpy as np

from .spaces import FourierSpace, ImageSpace


def padded_fourier_space(image_space, pad_factor=2):
    """The Fourier space of the zero-padded image (ZeroPaddingOperator + FourierSpace,
    lentils/operators/fourier_operators.py:29-42, lentils/common/space_base.py:62-84), as the
    NUFFT operator builds it."""
    p = int(pad_factor)
    padx = ((p - 1) * image_space.nx + 1) // 2
    pady = ((p - 1) * image_space.ny + 1) // 2
    dx, dy = image_space.dx, image_space.dy
    b = image_space.bounds + np.array([-padx * dx, padx * dx, -pady * dy, pady * dy])
    padded = ImageSpace(shape=(image_space.nx + 2 * padx, image_space.ny + 2 * pady),
                        bounds=[(b[0], b[1]), (b[2], b[3])])
    return FourierSpace(padded)


def _clip_guard(uvw, four, wsup):
    lim_u = (0.5 * four.nu - wsup - 1.0 - 1e-6) * four.du
    lim_v = (0.5 * four.nv - wsup - 1.0 - 1e-6) * four.dv
    uvw[:, 0] = np.clip(uvw[:, 0], -lim_u, lim_u)
    uvw[:, 1] = np.clip(uvw[:, 1], -lim_v, lim_v)
    return uvw


def synth_uv(rng, nvis, four, frac, wsup):
    """(nvis, 3) uv points out to `frac` of the Nyquist extent of `four` (any object with nu,
    nv, du, dv)."""
    rmax_u = frac * 0.5 * four.nu * four.du
    rmax_v = frac * 0.5 * four.nv * four.dv
    r = rng.uniform(0.0, 1.0, nvis)
    th = rng.uniform(0.0, 2 * np.pi, nvis)
    uvw = np.zeros((nvis, 3))
    uvw[:, 0] = r * np.cos(th) * rmax_u
    uvw[:, 1] = r * np.sin(th) * rmax_v
    return _clip_guard(uvw, four, wsup)


def synth_uv_blobs(rng, nvis, four, frac, wsup, nblobs=50, blob_frac=0.1, blob_width=0.005):
    """As synth_uv, with `blob_frac` of the points in `nblobs` Gaussian blobs of standard
    deviation blob_width * (nu/2) cells whose centres follow the same radial law."""
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
