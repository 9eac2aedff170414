"""The batched lens-parameter sweep (one persistent launch over many samples of uneven size,
KB widths 6 and 8 side by side): against the per-sample entry points (themselves pinned to the
oracle) and, for a few samples, against the oracle directly."""
import numpy as np
import pytest
import torch

import oracle as O
from helpers import REL_L2_FP32

pytestmark = pytest.mark.gpu


def _samples(rng, k=10):
    from lentils_gb300.sweep import draw_samples
    s = draw_samples(rng, k, sizes=(32, 48, 64), nvis_range=(2000, 20000), eps=0.01)
    # accuracy targets on both sides of the KB-width threshold
    for i, x in enumerate(s):
        x.tol = 1e-4 if i % 2 else 1e-6
        x.pix = 0.04
    return s


@pytest.fixture(scope="module")
def sweep(tmp_path_factory):
    from lentils_gb300.autotune import Autotuner
    from lentils_gb300.sweep import BatchedSweep
    path = str(tmp_path_factory.mktemp("tune") / "cache.json")
    tuner = Autotuner(path=path, tiles=(8, 16), chunks=(256, 1024), reps=1, mode="batched")
    sw = BatchedSweep(_samples(np.random.default_rng(11)), tuner=tuner)
    tuner.save()
    return sw, tuner, path


def test_sweep_mixes_widths_and_tunes(sweep):
    from lentils_gb300.autotune import Autotuner
    sw, tuner, path = sweep
    widths = {s.info["w2"] for s in sw.samples}
    assert widths == {6, 8}
    assert tuner.tuned > 0
    again = Autotuner(path=path, tiles=(8, 16), chunks=(256, 1024), mode="batched")
    for s in sw.samples:
        p = sw.plans[sw.samples.index(s)]
        assert again.params(p.nu, p.nv, 0, 0, s.info["w2"], s.nvis) == (s.info["tile"],
                                                                        s.info["chunk"])
    assert again.tuned == 0
    st = sw.stats()
    assert st["nsamples"] == len(sw.samples) and st["nwork"] > 0 and st["blocks"] > 0


@pytest.mark.parametrize("use_graph", [True, False])
def test_sweep_matches_per_sample_entry_points(sweep, use_graph):
    from lentils_gb300.lens_models import GlobalLensModel
    sw, _, _ = sweep
    for go in sw.grid_out:
        go.fill_(float("nan"))
    sw.run(use_graph=use_graph)
    sw.run(use_graph=use_graph)  # a second run overwrites (grids are cleared per run)
    sw.stream.synchronize()
    for k, s in enumerate(sw.samples):
        plan = sw.plans[k]
        v_ref = plan.degrid(sw.grid_in[k])
        assert torch.equal(sw.vis_out[k], v_ref), k
        g_ref = plan.grid(sw.vis_in[k])
        rel = float((sw.grid_out[k] - g_ref).abs().norm() / g_ref.abs().norm())
        assert rel < 1e-6, (k, rel)
        pts = torch.as_tensor(sw.pixel_points(k)).cuda()
        b_ref = GlobalLensModel(s.lenses).deflect(pts, 2.0).float()
        assert torch.allclose(sw.beta_out[k], b_ref, rtol=0, atol=2e-6), k


@pytest.mark.parametrize("form", [1, 2])
def test_sweep_kernel_forms(sweep, form):
    """The other item forms of the sweep kernel (column-pair gridder; same-cell chunk or
    per-visibility degridding) on the same samples, plans and inputs: visibilities identical,
    grids within FP32 summation order, deflections identical."""
    from lentils_gb300.autotune import Autotuner
    from lentils_gb300.sweep import BatchedSweep
    sw, _, path = sweep
    sw.run(use_graph=True)
    sw.stream.synchronize()
    tuner = Autotuner(path=path, tiles=(8, 16), chunks=(256, 1024), mode="batched")
    other = BatchedSweep(_samples(np.random.default_rng(11)), tuner=tuner, form=form)
    assert tuner.tuned == 0
    other.run(use_graph=True)
    other.stream.synchronize()
    for k in range(len(sw.samples)):
        assert torch.equal(other.grid_in[k], sw.grid_in[k]) and torch.equal(other.vis_in[k], sw.vis_in[k])
        assert torch.equal(other.vis_out[k], sw.vis_out[k]), k
        rel = float((other.grid_out[k] - sw.grid_out[k]).abs().norm() / sw.grid_out[k].abs().norm())
        assert rel < 1e-6, (k, rel)
        assert torch.equal(other.beta_out[k], sw.beta_out[k]), k


def test_sweep_against_oracle(sweep):
    """Two samples (one per KB width) in user row order against the FP64 CPU oracle."""
    from lentils_gb300.lens_models import GlobalLensModel
    sw, _, _ = sweep
    rng = np.random.default_rng(3)
    ks = [0, 1]
    ys = {}
    for k in ks:
        plan = sw.plans[k]
        y = O.complex_normal(rng, plan.nvis)
        sw.vis_in[k].copy_(plan.to_plan(torch.as_tensor(y).cuda()))
        ys[k] = y
    sw.run()
    sw.stream.synchronize()
    for k in ks:
        s, plan = sw.samples[k], sw.plans[k]
        four = O.FourierGeom.__new__(O.FourierGeom)
        four.nu, four.nv, four.half_nv = plan.nu, plan.nv, plan.half_nv
        four.du, four.dv = plan.du, plan.dv
        four.gcx = four.gcy = 0.0
        four._chan = np.zeros(1)
        vis = O.VisGeom(sw.uvw[k], [1.0])
        w, beta = plan.wsup, plan.kb_beta
        g_in = sw.grid_in[k].cpu().numpy().astype(np.complex128)
        v_or = O.degrid(vis, four, g_in, w, beta)
        v_us = plan.from_plan(sw.vis_out[k]).cpu().numpy()
        assert O.rel_l2(v_us, v_or) < REL_L2_FP32
        g_or = O.grid(vis, four, ys[k], w, beta)
        assert O.rel_l2(sw.grid_out[k].cpu().numpy(), g_or) < REL_L2_FP32
        lenses = GlobalLensModel(s.lenses).setup_raytracing(2.0)
        b_or = O.deflect(lenses, sw.pixel_points(k))
        assert np.max(np.abs(sw.beta_out[k].cpu().numpy() - b_or)) < 2e-6


def test_single_plan_tuning(tmp_path):
    """Single-plan mode: every (tile, chunk) candidate timed on its own plan; the cache
    answers the same class without tuning again."""
    from lentils_gb300.autotune import Autotuner
    path = str(tmp_path / "single.json")
    t = Autotuner(path=path, tiles=(8, 16), chunks=(256, 1024), reps=1)
    p = t.params(128, 128, 2e4, 2e4, 8, 5000)
    assert p in {(8, 256), (8, 1024), (16, 256), (16, 1024)} and t.tuned == 1
    assert len(t.cache[t.key(128, 128, 8, 5000)]["candidates"]) == 4
    t.save()
    assert Autotuner(path=path).params(128, 128, 0, 0, 8, 5000) == p

