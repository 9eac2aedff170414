"""GPU NUFFT operator (apodise, pad, cuFFT, degrid and the transpose), bilinear lens operator,
gradient prior and the normal-equation operator, against the FP64 oracle: the reference's
NUFFT composition (lentils/operators/fourier_operators.py:96-126) restated in oracle/oracle.py,
its known-answer test against the direct Fourier transform (lentils/tests/nufft_tests.py:43-66)
and the 'gradient' prior (lentils/operators/operator_base.py:225-242)."""
import numpy as np
import pytest
import scipy.sparse as sps
import torch

import oracle as O
from helpers import ERRTOL, REL_L2_FP32, lens_problem

pytestmark = pytest.mark.gpu


def _spaces(vis, img):
    from lentils_gb300.spaces import ImageSpace, VisibilitySpace
    vs = VisibilitySpace(channels=vis.channels, uvcoords=vis.uvw)
    ims = ImageSpace(img.shape, [(img.xmin, img.xmax), (img.ymin, img.ymax)])
    return vs, ims


def test_nufft_known_answer_against_dft(native):
    """nufft_tests.py:43-66 through the GPU NUFFTOperator (FP64 path), max-relative < 1e-6."""
    from lentils_gb300.operators import NUFFTOperator
    rng = np.random.default_rng(7)
    all_uv = np.concatenate([rng.normal(scale=1e5 * s, size=(4, 3))
                             for s in np.linspace(0.0, 55.0, 20)])
    vis = O.VisGeom(all_uv, [0.5])
    img = O.ImageGeom((236, 257), [(-0.5, 0.7), (-0.7, 0.5)])
    vs, ims = _spaces(vis, img)
    nufft = NUFFTOperator(vs, ims)
    vdata = rng.normal(size=(vis.nrows, 2)).view(np.complex128).reshape(-1)
    mat = O.dft_matrix(vis, img)
    dftvec = O.dft_adjoint(mat, vdata).reshape(img.shape)
    assert O.max_relative_error((nufft.T * vdata).reshape(img.shape), dftvec) < ERRTOL
    assert O.max_relative_error((nufft * dftvec).reshape(-1), O.dft_forward(mat, dftvec)) < ERRTOL


@pytest.mark.parametrize("centred", [True, False])
def test_nufft_vs_oracle(native, centred):
    from lentils_gb300.operators import NUFFTOperator
    rng = np.random.default_rng(11)
    bounds = [(-0.64, 0.64), (-0.64, 0.64)] if centred else [(-0.5, 0.78), (-0.7, 0.58)]
    img = O.ImageGeom((64, 70), bounds)
    four = O.FourierGeom(O.padded_geom(img)[0])
    vis = O.VisGeom(O.synth_uv(rng, 3000, four, 0.45, 4), [1.0])
    vs, ims = _spaces(vis, img)
    nufft = NUFFTOperator(vs, ims, kernel_support=4)
    ora = O.NufftOracle(vis, img, 2, 4)
    x = rng.normal(size=img.shape)
    y = O.complex_normal(rng, vis.nvis)
    tol64 = 1e-9 if centred else 1e-6   # the phase-centre factor is stored in FP32
    assert O.rel_l2((nufft * x).reshape(-1), ora.forward(x)) < tol64
    assert O.rel_l2((nufft.T * y).reshape(-1), ora.adjoint(y).reshape(-1)) < tol64
    # FP32 path on device tensors (plan order)
    xt = torch.as_tensor(x, dtype=torch.float32).cuda()
    yp = nufft * xt
    got = nufft.plan.from_plan(yp).cpu().numpy()
    assert O.rel_l2(got, ora.forward(x)) < REL_L2_FP32
    yt = nufft.plan.to_plan(torch.as_tensor(y).cuda())
    assert O.rel_l2((nufft.T * yt).cpu().numpy().reshape(-1), ora.adjoint(y).reshape(-1)) < REL_L2_FP32


def test_lens_and_prior_vs_oracle(native):
    from lentils_gb300.lens_models import deflect_points
    from lentils_gb300.operators import BilinearLensOperator, PriorCovarianceOperator
    from lentils_gb300.lens_models import GlobalLensModel, PowerLawEllipsoid, ExternalPotential
    from lentils_gb300.spaces import ImageSpace
    rng = np.random.default_rng(3)
    img, src, four, uvw, lenses, s_true = lens_problem(rng, n_img=96, n_src=40)
    ims = ImageSpace(img.shape, [(img.xmin, img.xmax), (img.ymin, img.ymax)])
    srcs = ImageSpace(src.shape, [(src.xmin, src.xmax), (src.ymin, src.ymax)])
    glm = GlobalLensModel([PowerLawEllipsoid(z=0.5, b=0.8, th=0.0, f=0.7, x=0.005, y=0.005,
                                             rc=0.0, qh=0.5),
                           ExternalPotential(z=0.5, x=0.005, y=0.005, ss=0.05, sa=20.0)])
    L = BilinearLensOperator(ims, srcs, glm, z_src=2.0)
    pts = L.source_points.cpu().numpy()
    ref_pts = O.deflect(lenses, img.points().reshape(-1, 2))
    assert np.max(np.abs(pts - ref_pts)) < 2e-6
    M = O.bilinear_lens_matrix(pts, img.mask, src)
    assert M.nnz > 100
    s = rng.normal(size=src.shape)
    r = rng.normal(size=img.shape)
    assert O.rel_l2((L * s).reshape(-1), M @ s.reshape(-1)) < 1e-12
    assert O.rel_l2((L.T * r).reshape(-1), M.T @ r.reshape(-1)) < 1e-12
    st = torch.as_tensor(s, dtype=torch.float32).cuda()
    assert O.rel_l2((L * st).cpu().numpy().reshape(-1), M @ s.reshape(-1)) < 1e-6
    P = PriorCovarianceOperator(srcs, "gradient", 1e-2)
    R = O.regulariser(src, 1e-2)
    assert O.rel_l2((P * s).reshape(-1), R @ s.reshape(-1)) < 1e-12


def _oracle_normal(img, src, four, uvw, pts, w, lam, wsup=4):
    A, rhs, _, _ = O.normal_operator(img, src, uvw, pts, w, lam, wsup)
    return A, rhs


def _inversion(rng, **kw):
    from lentils_gb300.inversion import SourceInversion
    from lentils_gb300.lens_models import GlobalLensModel, PowerLawEllipsoid, ExternalPotential
    from lentils_gb300.spaces import ImageSpace, VisibilitySpace
    img, src, four, uvw, lenses, s_true = lens_problem(rng, **kw)
    pix = img.dx
    glm = GlobalLensModel([PowerLawEllipsoid(z=0.5, b=kw.get("b", 0.8), th=0.0, f=0.7,
                                             x=0.25 * pix, y=0.25 * pix, rc=0.0, qh=0.5),
                           ExternalPotential(z=0.5, x=0.25 * pix, y=0.25 * pix, ss=0.05, sa=20.0)])
    vs = VisibilitySpace(channels=[1.0], uvcoords=uvw)
    ims = ImageSpace(img.shape, [(img.xmin, img.xmax), (img.ymin, img.ymax)])
    srcs = ImageSpace(src.shape, [(src.xmin, src.xmax), (src.ymin, src.ymax)])
    from lentils_gb300.operators import BilinearLensOperator, NUFFTOperator
    F = NUFFTOperator(vs, ims)
    L = BilinearLensOperator(ims, srcs, glm, z_src=2.0)
    model = F * (L * s_true)
    d = model.reshape(-1) + O.complex_normal(rng, uvw.shape[0])
    inv = SourceInversion(vs, d, 1.0, ims, srcs, glm, 2.0, 1e-2)
    return inv, img, src, four, uvw, d


def test_normal_operator_vs_oracle(native):
    rng = np.random.default_rng(17)
    inv, img, src, four, uvw, d = _inversion(rng, n_img=96, n_src=40, nvis=8000)
    pts = inv.lens.source_points.cpu().numpy()
    A, rhs = _oracle_normal(img, src, four, uvw, pts, np.ones(uvw.shape[0]), 1e-2)
    s = rng.normal(size=src.nx * src.ny)
    assert O.rel_l2(inv.apply(s), A(s)) < 1e-9
    got32 = inv.apply(torch.as_tensor(s, dtype=torch.float32).cuda()).double().cpu().numpy()
    assert O.rel_l2(got32, A(s)) < REL_L2_FP32
    assert O.rel_l2(inv.b.cpu().numpy(), rhs(d)) < 1e-9


@pytest.mark.parametrize("use_graph", [True, False])
def test_cg_reaches_true_residual(native, use_graph):
    """Jacobi-PCG with FP32 operator and FP64 refinement reaches a true relative residual of
    1e-6, measured again with the oracle's FP64 operator (exact Kaiser-Bessel weights and
    scipy FFTs), which decides convergence."""
    rng = np.random.default_rng(23)
    inv, img, src, four, uvw, d = _inversion(rng, n_img=96, n_src=40, nvis=8000)
    x, info = inv.solve(tol=1e-6, use_graph=use_graph)
    assert info["converged"] == 1, info
    assert info["rel_residual"] <= 1e-6
    pts = inv.lens.source_points.cpu().numpy()
    A, rhs = _oracle_normal(img, src, four, uvw, pts, np.ones(uvw.shape[0]), 1e-2)
    b = rhs(d)
    xs = x.cpu().numpy()
    assert np.linalg.norm(b - A(xs)) / np.linalg.norm(b) < 1.5e-6


def test_cg_warm_start(native):
    """A nonzero initial guess takes the FP64 residual matvec path (a zero guess skips it):
    from half the solution both solvers converge to the zero-start solution, and from the
    converged solution they stop after the first residual check."""
    rng = np.random.default_rng(41)
    inv, img, src, four, uvw, d = _inversion(rng, n_img=96, n_src=40, nvis=8000)
    x_ref, info = inv.solve(tol=1e-8)
    assert info["converged"] == 1
    scale = float(torch.linalg.vector_norm(x_ref))
    for solve in (inv.solve, lambda **kw: inv.solve_flexible(None, window=8, **kw)):
        x_half, info = solve(tol=1e-6, x0=0.5 * x_ref)
        assert info["converged"] == 1 and info["rel_residual"] <= 1e-6, info
        # the residual bound is the contract; the solution error also carries the condition
        # number, so this is a loose sanity bound
        assert float(torch.linalg.vector_norm(x_half - x_ref)) / scale < 1e-2
        _, info = solve(tol=1e-6, x0=x_ref)
        assert info["converged"] == 1 and info["inner_total"] == 0 and info["outer"] == 0, info


def test_workload_normal_operator_and_cg_vs_oracle(native):
    """The benchmarked CG inversion at full size (512^2 image, 128^2 source, 2e6 visibilities,
    PEMD + shear): the GPU deflection against the oracle's, the FP64 normal operator
    (lentils_normal_op_apply64) against the oracle's FP64 operator on a random source, the
    right-hand side, and the benchmarked solve's answer, whose true relative residual is
    recomputed with the oracle's operator (exact Kaiser-Bessel weights, scipy FFTs)."""
    from lentils_gb300 import workloads as WL
    inv, F, (vs, ims, srcs, uvw) = WL.inversion()
    img = O.ImageGeom((ims.nx, ims.ny), [(ims.xmin, ims.xmax), (ims.ymin, ims.ymax)])
    src = O.ImageGeom((srcs.nx, srcs.ny), [(srcs.xmin, srcs.xmax), (srcs.ymin, srcs.ymax)])
    c = 0.25 * WL.PIX
    lenses = O.lens_array([O.pemd_cpars(1.2, 0.0, 0.7, c, c, 0.5),
                           O.shear_cpars(c, c, 0.05, 20.0)])
    pts = inv.lens.source_points.cpu().numpy()
    assert np.max(np.abs(pts - O.deflect(lenses, img.points().reshape(-1, 2)))) < 2e-6
    A, rhs, _, _ = O.normal_operator(img, src, uvw, pts, inv.weights_user, WL.LAMBDA)
    rng = np.random.default_rng(5)
    s = rng.normal(size=src.nx * src.ny)
    assert O.rel_l2(inv.apply(s), A(s)) < 1e-9
    b = rhs(inv.data_user)
    assert O.rel_l2(inv.b.cpu().numpy(), b) < 1e-9
    x, info = inv.solve(tol=1e-6, inner_tol=1e-3)
    assert info["converged"] == 1 and info["rel_residual"] <= 1e-6, info
    xs = x.cpu().numpy()
    assert np.linalg.norm(b - A(xs)) / np.linalg.norm(b) < 1.5e-6
    # the learned flexible-CG solve as the benchmark runs it (committed weights and policy)
    from lentils_gb300 import learned
    from lentils_gb300 import train_preconditioner as T
    params, meta = T.load(T.DEFAULT_WEIGHTS)
    pol = T.deploy_policy(meta)
    net = learned.UNet(WL.SRC, WL.SRC, max_batch=1, params=params)
    net.set_jacobi_weight(pol["jacobi_weight"])
    x, info = inv.solve_flexible(net, tol=1e-6, inner_tol=1e-3, window=pol["window"],
                                 net_every=pol["net_every"])
    assert info["converged"] == 1 and info["rel_residual"] <= 1e-6, info
    xs = x.cpu().numpy()
    assert np.linalg.norm(b - A(xs)) / np.linalg.norm(b) < 1.5e-6
