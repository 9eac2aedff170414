"""The autotuner's accuracy model: its KB-width error bounds hold against the direct Fourier
sum (the oracle's dft_matrix, restating dft_matrix_csr, lentils/backend/nufft.c:128-161) for
the oracle NUFFT at beta = 2.34 W, and the narrower width is really less accurate."""
import numpy as np

import oracle as O
from lentils_gb300 import autotune


def _kb_error(W, n=32, seed=5):
    rng = np.random.default_rng(seed)
    half = 0.5 * n * 0.02
    img = O.ImageGeom((n, n), [(-half, half), (-half, half)])
    four = O.FourierGeom(O.padded_geom(img, 2)[0])
    uvw = O.synth_uv(rng, 3000, four, 0.45, W // 2)
    vis = O.VisGeom(uvw, [1.0])
    x = rng.normal(size=(n, n))
    exact = O.dft_forward(O.dft_matrix(vis, img), x)
    approx = O.NufftOracle(vis, img, 2, W // 2, beta=autotune.kb_beta(W)).forward(x)
    return np.linalg.norm(approx - exact) / np.linalg.norm(exact)


def test_width_error_bounds_hold():
    e6, e8 = _kb_error(6), _kb_error(8)
    assert e6 <= autotune.KB_ERROR[6]
    assert e8 <= autotune.KB_ERROR[8]
    assert e6 > autotune.KB_ERROR[8]


def test_width_for():
    assert autotune.width_for(1e-4) == 6
    assert autotune.width_for(autotune.KB_ERROR[6]) == 6
    assert autotune.width_for(1e-6) == 8
    assert autotune.width_for(1e-12) == 8
