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
