"""The learned preconditioner's network on the tensor cores against the CPU oracle (PyTorch
FP64 autograd): forward outputs and parameter gradients, with and without BF16 emulation in
the oracle; Adam training on the GPU; the preconditioner form; flexible CG."""
import numpy as np
import pytest
import torch

import unet_oracle as U

pytestmark = pytest.mark.gpu

# BF16-emulating oracle: differences come from FP32 accumulation order only, amplified where a
# value lands on the other side of a BF16 rounding boundary (the oracle itself moves by up to
# 2e-3 relative L2 under a 1e-7 relative perturbation of its parameters)
REL_EMULATED = 6e-3
# exact FP64 network: the BF16 storage of weights and activations
REL_EXACT = 3e-2


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def _problem(seed, B, H, W):
    from lentils_gb300 import learned
    rng = np.random.default_rng(seed)
    p = learned.init_params(seed, out_scale=1.0)
    # non-zero biases exercise the bias paths
    o = 0
    for ci, co, k, _, _ in learned.LAYERS:
        o += co * k * k * ci
        p[o:o + co] = rng.normal(0, 0.05, co)
        o += co
    x = rng.normal(size=(B, H, W)).astype(np.float32)
    f = rng.normal(size=(B, H, W)).astype(np.float32)
    t = rng.normal(size=(B, H, W)).astype(np.float32)
    return p, x, f, t


def _cuda(*a):
    return [torch.as_tensor(v).cuda() for v in a]


# (1, 16, 16) ... (2, 32, 48) run every layer through the split-K form (FP32 partial slabs summed
# in order), (3, 64, 64) the full-resolution layers through the unsplit form, (1, 128, 128) is
# the 128 x 128 source at batch 1 as the solver applies it (deep layers split, top ones not),
# (5, 128, 128) has enough 4-row bands for c1's band kernel.
@pytest.mark.parametrize("B,H,W", [(1, 16, 16), (2, 32, 48), (3, 64, 64), (1, 128, 128),
                                   (5, 128, 128)])
def test_unet_forward_matches_oracle(native, B, H, W):
    from lentils_gb300 import learned
    p, x, f, _ = _problem(10 + H, B, H, W)
    net = learned.UNet(H, W, max_batch=B, params=p)
    xc, fc = _cuda(x, f)
    out = net.forward(xc, fc).cpu().numpy()
    assert net.error_flag() == 0
    ref_e = U.forward(p, x, f, emulate_bf16=True)
    ref_x = U.forward(p, x, f, emulate_bf16=False)
    assert _rel(out, ref_e) < REL_EMULATED
    assert _rel(out, ref_x) < REL_EXACT


def test_unet_forward_is_deterministic(native):
    """Split-K layers sum their partial slabs in a fixed order, and no forward kernel uses
    atomics: repeated forwards at batch 1, 4 and 5 (c1's band kernel), same weights, give
    bit-identical outputs."""
    from lentils_gb300 import learned
    p, x, f, _ = _problem(77, 5, 128, 128)
    net = learned.UNet(128, 128, max_batch=5, params=p)
    xc, fc = _cuda(x, f)
    for B in (1, 4, 5):
        outs = [net.forward(xc[:B], fc[:B]) for _ in range(4)]
        for o in outs[1:]:
            assert torch.equal(o, outs[0])
    assert net.error_flag() == 0


# (1, 16, 16), (2, 32, 32): every weight gradient on the MN-major tensor-core kernel;
# (1, 24, 40): no layer's grid fits its 64-pixel chunks, so the transposed-operand forms run
@pytest.mark.parametrize("B,H,W", [(1, 16, 16), (2, 32, 32), (1, 24, 40)])
def test_unet_gradients_match_oracle(native, B, H, W):
    from lentils_gb300 import learned
    p, x, f, t = _problem(20 + H, B, H, W)
    net = learned.UNet(H, W, max_batch=B, params=p)
    xc, fc, tc = _cuda(x, f, t)
    g, loss = net.gradients(xc, fc, tc)
    assert net.error_flag() == 0
    le, ge = U.loss_and_grads(p, x, f, t, emulate_bf16=True)
    lx, gx = U.loss_and_grads(p, x, f, t, emulate_bf16=False)
    assert abs(loss - le) <= 1e-3 * le
    o = 0
    for li, (ci, co, k, _, _) in enumerate(learned.LAYERS):
        n = co * k * k * ci
        for name, sl in (("w", slice(o, o + n)), ("b", slice(o + n, o + n + co))):
            assert _rel(g[sl], ge[sl]) < 1e-2, (li, name, _rel(g[sl], ge[sl]))
            # against the exact network only the weights: a bias gradient is a sum over pixels
            # of residuals that largely cancel, so BF16 storage moves it by its own size
            if name == "w":
                assert _rel(g[sl], gx[sl]) < 1e-1, (li, name, _rel(g[sl], gx[sl]))
        o += n + co
    assert _rel(g, ge) < 5e-3
    assert _rel(g, gx) < 1e-1


def test_unet_gemm_forms_agree(native):
    """The persistent TMA convolutions with the fused first and output layers (form 0), the
    per-tile TMA / pipelined GEMMs (form 2) and the staged ones (form 1) give the same forward
    output and gradients on the 128^2 grid, up to FP32 summation order and the BF16 rounding it
    can flip. Batch 5 gives c1 160 bands of 4 rows, enough for its band kernel (forward and
    data gradient)."""
    from lentils_gb300 import learned
    p, x, f, t = _problem(77, 5, 128, 128)
    net = learned.UNet(128, 128, max_batch=5, params=p)
    xc, fc, tc = _cuda(x, f, t)
    res = {}
    for form in (1, 2, 0):
        net.set_gemm_form(form)
        out = net.forward(xc, fc)
        g, loss = net.gradients(xc, fc, tc)
        res[form] = (out.cpu().numpy(), g, loss)
    assert net.error_flag() == 0
    for form in (0, 2):
        # the first layer and the output layer sum in another order in form 0; a wrong tile or
        # band would show as a local error of the output's size
        assert _rel(res[form][0], res[1][0]) < 2e-3, form
        err = np.max(np.abs(res[form][0] - res[1][0]))
        assert err < 0.02 * np.max(np.abs(res[1][0])), (form, err)
        o = 0
        for li, (ci, co, k, _, _) in enumerate(learned.LAYERS):
            n = co * k * k * ci
            assert _rel(res[form][1][o:o + n], res[1][1][o:o + n]) < 1e-2, (form, li)
            o += n + co
        assert abs(res[form][2] - res[1][2]) <= 1e-4 * abs(res[1][2]), form


def test_unet_adam_overfits_one_batch(native):
    from lentils_gb300 import learned
    p, x, f, _ = _problem(31, 4, 32, 32)
    # a smooth target the network can represent
    yy, xx = np.meshgrid(np.linspace(-1, 1, 32), np.linspace(-1, 1, 32), indexing="ij")
    t = np.broadcast_to(np.sin(2 * xx) * np.cos(3 * yy), (4, 32, 32)).astype(np.float32).copy()
    net = learned.UNet(32, 32, max_batch=4, params=learned.init_params(5))
    xc, fc, tc = _cuda(x, f, t)
    _, l0 = net.gradients(xc, fc, tc)
    lbuf = torch.zeros(1, device="cuda")
    for _ in range(150):
        net.train_step(xc, fc, tc, 2e-3, lbuf)
    _, l1 = net.gradients(xc, fc, tc)
    assert net.error_flag() == 0
    assert l1 < 0.1 * l0, (l0, l1)


# 32 x 32: every hidden layer split over K; 128 x 128: the first layer, c1 and the output layer
# and the combination fused (persistent GEMM epilogue)
@pytest.mark.parametrize("H", [32, 128])
def test_unet_precondition_form(native, H):
    from lentils_gb300 import learned
    W = H
    rng = np.random.default_rng(7)
    net = learned.UNet(H, W, max_batch=1, params=learned.init_params(2, out_scale=1.0))
    r = torch.as_tensor(rng.normal(size=(H, W)).astype(np.float32)).cuda()
    dinv = torch.as_tensor(np.exp(rng.normal(size=(H, W))).astype(np.float32)).cuda()
    feat = learned.features(dinv.reshape(-1)).reshape(H, W)
    ref_feat = torch.log(dinv.double()) - torch.log(dinv.double()).mean()
    assert torch.allclose(feat.double(), ref_feat, atol=1e-5)
    xs, fs = learned.scaled_inputs(r[None], dinv[None], feat[None])
    out = net.forward(xs, fs)[0]
    u = dinv * r
    s = torch.sqrt(torch.mean(u.double() ** 2)).float()
    for gamma in (0.0, 1.0):
        net.set_jacobi_weight(gamma)
        z = net.precondition(r, dinv, feat)
        assert _rel(z.cpu().numpy(), (gamma * u + s * out).cpu().numpy()) < 1e-5


@pytest.mark.parametrize("with_net,window,every",
                         [(False, 1, 1), (True, 1, 1), (False, 4, 1), (True, 8, 1), (True, 8, 3)])
@pytest.mark.parametrize("use_graph", [True, False])
def test_flexible_cg_reaches_true_residual(native, with_net, window, every, use_graph):
    """Flexible CG (Jacobi directions only, or an untrained network with the Jacobi fallback,
    proposing every direction or every third) reaches a true FP64 relative residual of 1e-6,
    checked again with the oracle operator."""
    import oracle as O
    from lentils_gb300 import learned
    from test_operators_gpu import _inversion, _oracle_normal
    rng = np.random.default_rng(29)
    inv, img, src, four, uvw, d = _inversion(rng, n_img=96, n_src=48, nvis=8000)
    net = learned.UNet(48, 48, max_batch=1, params=learned.init_params(3)) if with_net else None
    x, info = inv.solve_flexible(net, tol=1e-6, use_graph=use_graph, window=window,
                                 net_every=every)
    assert info["converged"] == 1, info
    if not with_net:
        assert info["net_iterations"] == 0 and info["fallback"] == 0
    elif every > 1 and not info["fallback"]:
        # the network is offered one direction in `every` (plus the first of each inner solve)
        assert info["net_iterations"] <= info["inner_total"] // every + 2 * info["outer"], info
    pts = inv.lens.source_points.cpu().numpy()
    A, rhs = _oracle_normal(img, src, four, uvw, pts, np.ones(uvw.shape[0]), 1e-2)
    b = rhs(d)
    assert np.linalg.norm(b - A(x.cpu().numpy())) / np.linalg.norm(b) < 1.5e-6
    if not with_net:
        _, ref = inv.solve(tol=1e-6, use_graph=use_graph)
        assert info["inner_total"] <= 1.2 * ref["inner_total"] + 10, (info, ref)


def test_unet_backward_external_gradient_matches_mse_path(native):
    """An external output gradient 2 (out - t) / n through lentils_unet_backward gives the
    same parameter gradient as the built-in mean-squared-error path."""
    from lentils_gb300 import learned
    p, x, f, t = _problem(41, 2, 32, 32)
    net = learned.UNet(32, 32, max_batch=2, params=p)
    xc, fc, tc = _cuda(x, f, t)
    g_mse, _ = net.gradients(xc, fc, tc)
    out = net.forward(xc, fc)
    g_ext = net.backward(2.0 * (out - tc) / out.numel(), want_grad=True)
    assert _rel(g_ext, g_mse) < 1e-3


def test_trained_network_in_flexible_cg(native):
    """What the trained network (the committed weights, trained on the GPU by
    train_preconditioner) gains, and does not gain, on the 128^2 source inversion, used with
    the deployment policy stored beside it. The fair comparison is flexible CG with the same
    8-direction window and Jacobi directions only: in exact arithmetic that is Jacobi-PCG, and
    it needs about the iterations of Jacobi-PCG with FP64 vectors.
    - Per step, on windowed flexible-CG pairs from lens draws it was not trained on, its
      direction (with the Jacobi share it was trained with) removes a larger share of the
      A-norm error than the Jacobi direction, after the A-orthogonalisation flexible CG applies.
    - On the workload inversion the learned solver stays within 1.5x of Jacobi flexible CG's
      iterations, and both windowed solvers need at most a third of the iterations of plain
      Jacobi-CG with FP32 inner solves (which lose conjugacy).
    - On held-out lens draws the per-step gain does not carry over: the learned solver can
      need more than twice the iterations of Jacobi flexible CG. The descent check and the
      stagnation fallback keep it within twice plain Jacobi-CG's iterations, and every solve
      reaches the true relative residual of 1e-6."""
    from lentils_gb300 import learned, workloads
    from lentils_gb300 import train_preconditioner as T
    from lentils_gb300.inversion import SourceInversion
    from lentils_gb300.operators import NUFFTOperator
    params, meta = T.load(T.DEFAULT_WEIGHTS)
    pol = T.deploy_policy(meta)
    g_train = float(meta.get("gamma", 0.0))
    vs, ims, srcs, uvw, _ = workloads.geometry()
    F = NUFFTOperator(vs, ims)
    data = T.build_training_set(F, (vs, ims, srcs, uvw), 2, 40, 90210, log=lambda m: None,
                                window=pol["window"])
    net = learned.UNet(workloads.SRC, workloads.SRC, max_batch=16, params=params)
    fr_net, fr_jac = [], []
    for i in range(0, data["r"].shape[0] - 15, 16):
        ids = torch.arange(i, i + 16, device="cuda")
        r = data["r"][ids].view(-1, 128, 128)
        di = data["draw"][ids]
        x, f = learned.scaled_inputs(r, data["dinv"][di].view(-1, 128, 128),
                                     data["feat"][di].view(-1, 128, 128))
        fr_net.append(T.window_energy_loss(data, ids, g_train * x + net.forward(x, f))[0])
        fr_jac.append(T.window_energy_loss(data, ids, x)[0])
    fn, fj = float(torch.cat(fr_net).mean()), float(torch.cat(fr_jac).mean())
    assert fn < fj - 0.03, (fn, fj)
    del data
    pnet = learned.UNet(workloads.SRC, workloads.SRC, max_batch=1, params=params)
    pnet.set_jacobi_weight(pol["jacobi_weight"])
    inv, _, _ = workloads.inversion(nufft=F)
    rng = np.random.default_rng(4242)
    problems = [inv]
    for _ in range(2):
        glm = learned.lens_draw(rng, centre=(0.25 * ims.dx, 0.25 * ims.dy))
        d = workloads.simulate(F, ims, srcs, glm, learned.random_source(rng, srcs), rng)
        problems.append(SourceInversion(vs, d, 1.0, ims, srcs, glm, workloads.Z_SRC,
                                        workloads.LAMBDA, nufft=F))
    for k, p in enumerate(problems):
        _, jac = p.solve_flexible(None, tol=1e-6, inner_tol=1e-3, window=pol["window"])
        _, lrn = p.solve_flexible(pnet, tol=1e-6, inner_tol=1e-3, window=pol["window"],
                                  net_every=pol["net_every"])
        _, plain = p.solve(tol=1e-6, inner_tol=1e-3)
        for info in (jac, lrn, plain):
            assert info["converged"] == 1 and info["rel_residual"] <= 1e-6, (k, jac, lrn, plain)
        assert lrn["net_iterations"] > 0, (k, lrn)
        if k == 0:
            assert lrn["inner_total"] <= 1.5 * jac["inner_total"], (k, lrn, jac)
            assert 3 * max(lrn["inner_total"], jac["inner_total"]) <= plain["inner_total"], \
                (lrn, jac, plain)
        else:
            assert lrn["inner_total"] <= 2 * plain["inner_total"] + 50, (k, lrn, plain)
