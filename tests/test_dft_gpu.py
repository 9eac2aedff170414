"""The direct Fourier sum on the GPU (DFTOperator) against the oracle's dense restatement of
dft_matrix_csr (nufft.c:128-161), and the reference's NUFFT-vs-DFT known-answer test
(test_gridder_and_apodization, lentils/tests/nufft_tests.py:43-66) at the 128^2 / 2e4
visibility size, run entirely on the GPU."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _spaces(rng, shape, bounds, nvis, frac, wsup, mask=None):
    from lentils_gb300.spaces import ImageSpace, VisibilitySpace
    img = O.ImageGeom(shape, bounds, mask=mask)
    four = O.FourierGeom(O.padded_geom(img, 2)[0])
    uvw = O.synth_uv(rng, nvis, four, frac, wsup)
    ims = ImageSpace(shape, [(bounds[0][0], bounds[0][1]), (bounds[1][0], bounds[1][1])])
    if mask is not None:
        ims.mask[...] = mask
    return img, uvw, VisibilitySpace(channels=[1.0], uvcoords=uvw), ims


def test_dft_vs_oracle_matrix(native):
    from lentils_gb300.operators import DFTOperator
    rng = np.random.default_rng(61)
    mask = np.ones((20, 24), bool)
    mask[3:7, 5:9] = False
    img, uvw, vs, ims = _spaces(rng, (20, 24), [(-0.3, 0.5), (-0.4, 0.56)], 500, 0.45, 3, mask)
    D = DFTOperator(vs, ims)
    mat = O.dft_matrix(O.VisGeom(uvw, [1.0]), img)
    x = rng.normal(size=img.shape)
    assert O.rel_l2(D * x, O.dft_forward(mat, x)) < 1e-12
    y = O.complex_normal(rng, uvw.shape[0])
    assert O.rel_l2(D.T * y, O.dft_adjoint(mat, y).reshape(img.shape)) < 1e-12


@pytest.mark.parametrize("wsup,bar", [(3, 1e-5), (4, 1e-6)])
def test_nufft_vs_dft_known_answer(native, wsup, bar):
    """NUFFT (GPU, FP64 path) against the direct sum (GPU) on a 128^2 image with 2e4
    visibilities; bar 1e-6 at W = 8 as in the reference's test."""
    from lentils_gb300.operators import DFTOperator, NUFFTOperator
    rng = np.random.default_rng(67)
    img, uvw, vs, ims = _spaces(rng, (128, 128), [(-1.28, 1.28), (-1.28, 1.28)], 20000, 0.45,
                                wsup)
    F = NUFFTOperator(vs, ims, kernel_support=wsup, kb_beta=2.34 * 2 * wsup)
    D = DFTOperator(vs, ims)
    x = rng.normal(size=img.shape)
    assert O.max_relative_error(F * x, D * x) < bar
    y = O.complex_normal(rng, uvw.shape[0])
    assert O.rel_l2(F.T * y, D.T * y) < bar
