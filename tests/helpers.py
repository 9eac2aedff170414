"""Shared helpers for the test-suite (seeded inputs, fixture loading, tolerances)."""
import os

import numpy as np

import oracle as O

# Tolerances. FP32 kernels against the FP64 oracle: relative L2 <= 1e-5 (the stated target of
# the FP32 path); max-relative error of the reference's own tests: errtol = 1e-6
# (lentils/tests/test_utils.py:9).
REL_L2_FP32 = 1e-5
ERRTOL = 1e-6

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_nufft_golden(name):
    d = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    vis = O.VisGeom(d["uvw"], d["channels"])
    four = O.FourierGeom.__new__(O.FourierGeom)
    four.nu, four.nv = int(d["nu"]), int(d["nv"])
    four.half_nv = four.nv // 2 + 1
    four.du, four.dv = float(d["du"]), float(d["dv"])
    four.gcx, four.gcy = float(d["gcx"]), float(d["gcy"])
    four._chan = np.zeros(1)
    return d, vis, four


def nufft_setup(rng, shape, bounds, chans, wsup, nvis, frac, blobs=False):
    img = O.ImageGeom(shape, bounds)
    padded, _, _ = O.padded_geom(img, 2)
    four = O.FourierGeom(padded)
    if blobs:
        uvw = O.synth_uv_blobs(rng, nvis, four, frac, wsup)
    else:
        uvw = O.synth_uv(rng, nvis, four, frac, wsup)
    uvw = uvw / max(chans)
    return img, four, O.VisGeom(uvw, chans)


def lens_problem(rng, n_img=128, pix=0.02, n_src=48, src_half=0.6, nvis=20000, b=0.8,
                 wsup=4, frac=0.45):
    """A small CG source-inversion problem: PEMD (q=0.7, gamma=2) + shear (0.05, 20 deg)
    centred off the pixel corners, bilinear source grid, nvis visibilities with sigma = 1.
    Returns geometry, uv, lens array, a true source and seeded noisy data is left to callers."""
    half = 0.5 * n_img * pix
    img = O.ImageGeom((n_img, n_img), [(-half, half), (-half, half)])
    src = O.ImageGeom((n_src, n_src), [(-src_half, src_half), (-src_half, src_half)])
    padded, _, _ = O.padded_geom(img, 2)
    four = O.FourierGeom(padded)
    uvw = O.synth_uv(rng, nvis, four, frac, wsup)
    lenses = O.lens_array([O.pemd_cpars(b, 0.0, 0.7, 0.5 * pix * 0.5, 0.5 * pix * 0.5, 0.5),
                           O.shear_cpars(0.5 * pix * 0.5, 0.5 * pix * 0.5, 0.05, 20.0)])
    xs = (src.xmin + src.dx * np.arange(src.nx))[:, None]
    ys = (src.ymin + src.dy * np.arange(src.ny))[None, :]
    s_true = (np.exp(-((xs - 0.05) ** 2 + (ys - 0.02) ** 2) / (2 * 0.06 ** 2))
              + 0.5 * np.exp(-((xs + 0.1) ** 2 + (ys + 0.08) ** 2) / (2 * 0.04 ** 2)))
    return img, src, four, uvw, lenses, s_true
