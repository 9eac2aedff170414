"""Dirty-beam (blurred covariance) form of F^T C^-1 F on the GPU against the oracle's
restatement of RadioDataset.blurred_covariance_operator (data_base.py:115-129), against the
explicit visibility form, and inside the CG source inversion."""
import numpy as np
import pytest
import torch

import oracle as O
from helpers import REL_L2_FP32, lens_problem

pytestmark = pytest.mark.gpu


def _setup(rng, n=(48, 40), nvis=6000):
    from lentils_gb300.spaces import ImageSpace, VisibilitySpace
    half = (0.5 * n[0] * 0.02, 0.5 * n[1] * 0.02)
    img = O.ImageGeom(n, [(-half[0], half[0]), (-half[1], half[1])])
    four = O.FourierGeom(O.padded_geom(img, 2)[0])
    uvw = O.synth_uv(rng, nvis, four, 0.45, 4)
    vis = O.VisGeom(uvw, [1.0])
    vs = VisibilitySpace(channels=[1.0], uvcoords=uvw)
    ims = ImageSpace(n, [(-half[0], half[0]), (-half[1], half[1])])
    return img, vis, vs, ims


def test_bcb_operator_vs_oracle(native):
    from lentils_gb300.operators import BlurredCovarianceOperator
    rng = np.random.default_rng(41)
    img, vis, vs, ims = _setup(rng)
    w = rng.uniform(0.5, 2.0, vis.nvis)
    B = BlurredCovarianceOperator(vs, ims, w)
    beam_or = O.dirty_beam(vis, img, w, 4)
    assert O.rel_l2(B.dirty_beam, beam_or) < 1e-9
    assert abs(B.centre - beam_or[img.nx, img.ny]) <= 1e-9 * abs(beam_or[img.nx, img.ny])
    x = rng.normal(size=img.shape)
    ref = O.bcb_apply(beam_or, img, x)
    assert O.rel_l2(B * x, ref) < 1e-9
    got32 = (B * torch.as_tensor(x, dtype=torch.float32).cuda()).double().cpu().numpy()
    assert O.rel_l2(got32, ref) < REL_L2_FP32


def test_bcb_matches_visibility_form(native):
    from lentils_gb300.operators import BlurredCovarianceOperator, NUFFTOperator
    rng = np.random.default_rng(43)
    img, vis, vs, ims = _setup(rng, n=(40, 40))
    w = rng.uniform(0.5, 2.0, vis.nvis)
    B = BlurredCovarianceOperator(vs, ims, w)
    F = NUFFTOperator(vs, ims)
    x = rng.normal(size=img.shape)
    explicit = F.T * (w * (F * x))
    assert O.rel_l2(B * x, explicit) < 1e-6


@pytest.mark.parametrize("flexible", [False, True])
def test_cg_with_dirty_beam_form(native, flexible):
    """The inversion with the dirty-beam data term reaches a true relative residual of 1e-6,
    checked with the oracle's FP64 operator L^T B L + lambda R^T R and b = L^T F^T C^-1 d."""
    from lentils_gb300.inversion import SourceInversion
    from lentils_gb300.lens_models import ExternalPotential, GlobalLensModel, PowerLawEllipsoid
    from lentils_gb300.operators import BilinearLensOperator, NUFFTOperator
    from lentils_gb300.spaces import ImageSpace, VisibilitySpace
    rng = np.random.default_rng(47)
    img, src, four, uvw, _, s_true = lens_problem(rng, n_img=96, n_src=40, nvis=8000)
    pix = img.dx
    glm = GlobalLensModel([PowerLawEllipsoid(z=0.5, b=0.8, th=0.0, f=0.7, x=0.25 * pix,
                                             y=0.25 * pix, rc=0.0, qh=0.5),
                           ExternalPotential(z=0.5, x=0.25 * pix, y=0.25 * pix, ss=0.05,
                                             sa=20.0)])
    vs = VisibilitySpace(channels=[1.0], uvcoords=uvw)
    ims = ImageSpace(img.shape, [(img.xmin, img.xmax), (img.ymin, img.ymax)])
    srcs = ImageSpace(src.shape, [(src.xmin, src.xmax), (src.ymin, src.ymax)])
    F = NUFFTOperator(vs, ims)
    L = BilinearLensOperator(ims, srcs, glm, z_src=2.0)
    d = (F * (L * s_true)).reshape(-1) + O.complex_normal(rng, uvw.shape[0])
    inv = SourceInversion(vs, d, 1.0, ims, srcs, glm, 2.0, 1e-2, data_term="bcb")
    if flexible:
        x, info = inv.solve_flexible(None, tol=1e-6, inner_tol=1e-3, window=8)
    else:
        x, info = inv.solve(tol=1e-6)
    assert info["converged"] == 1, info
    vis = O.VisGeom(uvw, [1.0])
    beam = O.dirty_beam(vis, img, np.ones(uvw.shape[0]), 4)
    M = O.bilinear_lens_matrix(inv.lens.source_points.cpu().numpy(), img.mask, src)
    R = O.regulariser(src, 1e-2)
    ora = O.NufftOracle(vis, img, 2, 4)
    b = M.T @ ora.adjoint(d).reshape(-1)
    xs = x.cpu().numpy()
    r = b - (M.T @ O.bcb_apply(beam, img, (M @ xs).reshape(img.shape)).reshape(-1) + R @ xs)
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1.5e-6
