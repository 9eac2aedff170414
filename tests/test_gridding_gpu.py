"""GPU degridding / gridding through the C ABI, against the FP64 oracle.

Bar: relative L2 <= 1e-5 (FP32 kernels vs the FP64 reference arithmetic), on the committed
golden fixtures (generated by the reference's own grid_cpu), on seeded synthetic inputs with
the benchmark geometries, and on the edge cases the reference's gridder handles: empty input,
points exactly on grid cells, the origin, points beyond the Nyquist guard (wrap), odd and
non-square grids, several channels, an off-centre phase centre, every kernel width 1..8, and
heavy bins. At the full 1e7-visibility size the checks are size-independent: the adjoint
identity and an oracle comparison on sampled visibilities."""
import numpy as np
import pytest
import torch

import oracle as O
from helpers import REL_L2_FP32, load_nufft_golden, nufft_setup

pytestmark = pytest.mark.gpu


def make_plan(vis, four, w, beta, **kw):
    from lentils_gb300.gridding import GriddingPlan
    return GriddingPlan(vis.uvw, vis.channels, four.nu, four.nv, four.du, four.dv, four.gcx,
                        four.gcy, w, beta, **kw)


def gpu_degrid(plan, grid_c128):
    g = torch.as_tensor(grid_c128.astype(np.complex64)).cuda()
    yp = plan.degrid(g)
    return plan.from_plan(yp).cpu().numpy()


def gpu_grid(plan, vis_c128):
    v = torch.as_tensor(vis_c128).cuda()
    gp = plan.grid(plan.to_plan(v))
    return gp.cpu().numpy().astype(np.complex128)


@pytest.mark.parametrize("name", ["nufft_cfg0_w3", "nufft_odd_w4", "nufft_tiny_w1"])
@pytest.mark.parametrize("tile,variant", [(0, 0), (8, 0), (64, 0), (0, 1), (32, 1), (0, 2),
                                          (0, 5), (0, 6), (0, 7), (0, 8), (8, 8), (64, 8),
                                          (16, 2), (0, 3), (32, 3), (0, 4), (8, 4), (64, 4),
                                          (0, 9), (8, 9), (64, 9), (0, 10), (32, 10),
                                          (0, 11), (8, 11), (64, 11), (0, 12), (8, 12)])
def test_plan_api_vs_golden(native, name, tile, variant):
    d, vis, four = load_nufft_golden(name)
    w, beta = int(d["wsup"]), float(d["beta"])
    plan = make_plan(vis, four, w, beta, tile=tile)
    plan.set_grid_variant(variant)
    v = gpu_degrid(plan, d["grid_in"])
    assert O.rel_l2(v, d["vis_out"] - d["vis_acc0"]) < REL_L2_FP32
    g = gpu_grid(plan, d["vis_in"])
    assert O.rel_l2(g, d["grid_out"] - d["grid_acc0"]) < REL_L2_FP32


@pytest.mark.parametrize("name", ["nufft_cfg0_w3", "nufft_odd_w4", "nufft_tiny_w1"])
@pytest.mark.parametrize("tile", [0, 8, 64])
def test_degrid_layouts_vs_golden(native, name, tile):
    """Every form of the degridding kernel (same-cell chunks, the paired-column shared tile,
    one visibility per thread) gives the same bits."""
    d, vis, four = load_nufft_golden(name)
    w, beta = int(d["wsup"]), float(d["beta"])
    plan = make_plan(vis, four, w, beta, tile=tile)
    plan.set_degrid_variant(0)
    v0 = gpu_degrid(plan, d["grid_in"])
    for variant in (1, 2):
        plan.set_degrid_variant(variant)
        v1 = gpu_degrid(plan, d["grid_in"])
        assert np.array_equal(v0, v1), variant
        assert O.rel_l2(v1, d["vis_out"] - d["vis_acc0"]) < REL_L2_FP32


@pytest.mark.parametrize("name", ["nufft_cfg0_w3", "nufft_odd_w4", "nufft_tiny_w1"])
def test_dropin_grid_cpu_vs_golden(native, name):
    """grid_cpu with the reference's signature, host complex128 buffers, += semantics."""
    from lentils_gb300.gridding import grid_cpu
    from lentils_gb300.spaces import VisibilitySpace
    d, vis, four = load_nufft_golden(name)
    from lentils_gb300._native import FourierSpaceC
    vs = VisibilitySpace(channels=d["channels"], uvcoords=d["uvw"])
    gsc = FourierSpaceC(four.nu, four.nv, four.half_nv, 1, 1, four.du, four.dv, four.gcx,
                        four.gcy, None)
    w, beta = int(d["wsup"]), float(d["beta"])
    v = d["vis_acc0"].copy()
    grid_cpu(vs, v, gsc, d["grid_in"].copy(), w, beta, 0)
    assert O.rel_l2(v - d["vis_acc0"], d["vis_out"] - d["vis_acc0"]) < REL_L2_FP32
    g = d["grid_acc0"].copy()
    grid_cpu(vs, d["vis_in"].copy(), gsc, g, w, beta, 1)
    assert O.rel_l2(g - d["grid_acc0"], d["grid_out"] - d["grid_acc0"]) < REL_L2_FP32


def test_dropin_grid_cpu_plan_cache(native):
    """Repeated grid_cpu calls on one visibility space reuse one cached plan and give the
    reference's results every time; rewriting the uv buffer in place replaces the cached plan
    (mode 1 digests sampled rows, mode 2 every row); mode 0 bins on every call."""
    from lentils_gb300 import _native as N
    from lentils_gb300.gridding import grid_cpu
    from lentils_gb300.spaces import VisibilitySpace
    from lentils_gb300._native import FourierSpaceC
    L = N.lib()
    d, vis, four = load_nufft_golden("nufft_odd_w4")
    w, beta = int(d["wsup"]), float(d["beta"])
    gsc = FourierSpaceC(four.nu, four.nv, four.half_nv, 1, 1, four.du, four.dv, four.gcx,
                        four.gcy, None)
    try:
        for mode in (1, 2, 0):
            N.check(L.lentils_dropin_cache_mode(mode))
            N.check(L.lentils_dropin_cache_clear())
            vs = VisibilitySpace(channels=d["channels"], uvcoords=d["uvw"])
            for _ in range(3):
                v = np.zeros_like(d["vis_acc0"])
                grid_cpu(vs, v, gsc, d["grid_in"].copy(), w, beta, 0)
                assert O.rel_l2(v, d["vis_out"] - d["vis_acc0"]) < REL_L2_FP32
                g = np.zeros_like(d["grid_acc0"])
                grid_cpu(vs, d["vis_in"].copy(), gsc, g, w, beta, 1)
                assert O.rel_l2(g, d["grid_out"] - d["grid_acc0"]) < REL_L2_FP32
                assert L.lentils_dropin_cache_size() == (1 if mode else 0)
            # the same buffer rewritten in place: new uv, same address
            vs.uvw[:] *= 0.9
            nv = O.VisGeom(vs.uvw.copy(), d["channels"])
            v = np.zeros_like(d["vis_acc0"])
            grid_cpu(vs, v, gsc, d["grid_in"].copy(), w, beta, 0)
            assert O.rel_l2(v, O.degrid(nv, four, d["grid_in"], w, beta)) < REL_L2_FP32
            assert L.lentils_dropin_cache_size() == (1 if mode else 0)
    finally:
        N.check(L.lentils_dropin_cache_mode(1))
        N.check(L.lentils_dropin_cache_clear())


@pytest.mark.parametrize("w", [1, 2, 3, 4, 5, 6, 7, 8])
def test_every_kernel_width(native, w):
    rng = np.random.default_rng(100 + w)
    img, four, vis = nufft_setup(rng, (48, 52), [(-0.4, 0.6), (-0.5, 0.5)], [1.0], w, 700, 0.4)
    beta = O.kb_beta(w)
    plan = make_plan(vis, four, w, beta)
    g = rng.normal(size=four.shape) + 1j * rng.normal(size=four.shape)
    assert O.rel_l2(gpu_degrid(plan, g), O.degrid(vis, four, g, w, beta)) < REL_L2_FP32
    y = O.complex_normal(rng, vis.nvis)
    assert O.rel_l2(gpu_grid(plan, y), O.grid(vis, four, y, w, beta)) < REL_L2_FP32


def test_special_points(native):
    """Points on grid cells (the reference's extra edge tap), the origin, wrapped points
    beyond the Nyquist guard, several channels, odd grid, phase centre off the origin."""
    rng = np.random.default_rng(21)
    img = O.ImageGeom((45, 38), [(-0.35, 0.55), (-0.1, 0.66)])
    padded, _, _ = O.padded_geom(img, 2)
    four = O.FourierGeom(padded)
    pts = [[0, 0, 0], [5 * four.du, -3 * four.dv, 0],
           [-2 * four.du, 0, 0], [0, 7 * four.dv, 0], [0.2 * four.du, -11 * four.dv, 0],
           [0.7 * four.nu * four.du, 0.2 * four.nv * four.dv, 0],
           [-1.3 * four.nu * four.du, -0.9 * four.nv * four.dv, 0],
           [0.5 * four.nu * four.du, 0.5 * four.nv * four.dv, 0]]
    uvw = np.concatenate([np.array(pts, float), rng.normal(size=(200, 3)) * 6 * four.du])
    for chans in ([1.0], [1.0, 0.5, -0.25]):
        vis = O.VisGeom(uvw, chans)
        for w in (2, 4):
            beta = O.kb_beta(w)
            plan = make_plan(vis, four, w, beta, tile=8)
            g = rng.normal(size=four.shape) + 1j * rng.normal(size=four.shape)
            assert O.rel_l2(gpu_degrid(plan, g), O.degrid(vis, four, g, w, beta)) < REL_L2_FP32
            y = O.complex_normal(rng, vis.nvis)
            assert O.rel_l2(gpu_grid(plan, y), O.grid(vis, four, y, w, beta)) < REL_L2_FP32


def test_heavy_bins_and_seams(native):
    """All points in one cell; points strung along tile seams and the v = 0 fold."""
    rng = np.random.default_rng(31)
    img = O.ImageGeom((128, 128), [(-1.28, 1.28), (-1.28, 1.28)])
    four = O.FourierGeom(O.padded_geom(img)[0])
    w, beta = 4, O.kb_beta(4)
    one_cell = np.zeros((5000, 3))
    one_cell[:, 0] = (17.3 + rng.uniform(0, 0.4, 5000)) * four.du
    one_cell[:, 1] = (-3.6 + rng.uniform(0, 0.4, 5000)) * four.dv
    seams = np.zeros((3000, 3))
    seams[:, 0] = (rng.integers(-4, 4, 3000) * 16 + rng.uniform(-0.5, 0.5, 3000)) * four.du
    seams[:, 1] = (rng.uniform(-1.0, 1.0, 3000) * 4) * four.dv
    for uvw, variant in ((one_cell, 0), (seams, 0), (one_cell, 1), (seams, 1), (one_cell, 2),
                         (seams, 2), (one_cell, 3), (seams, 3), (one_cell, 4), (seams, 4),
                         (one_cell, 9), (seams, 9), (one_cell, 10), (seams, 10),
                         (one_cell, 11), (seams, 11), (one_cell, 12), (seams, 12)):
        vis = O.VisGeom(uvw, [1.0])
        plan = make_plan(vis, four, w, beta, tile=16, chunk=512)
        plan.set_grid_variant(variant)
        g = rng.normal(size=four.shape) + 1j * rng.normal(size=four.shape)
        assert O.rel_l2(gpu_degrid(plan, g), O.degrid(vis, four, g, w, beta)) < REL_L2_FP32
        y = O.complex_normal(rng, vis.nvis)
        assert O.rel_l2(gpu_grid(plan, y), O.grid(vis, four, y, w, beta)) < REL_L2_FP32


def test_empty_and_single(native):
    rng = np.random.default_rng(41)
    img = O.ImageGeom((32, 32), [(-0.32, 0.32), (-0.32, 0.32)])
    four = O.FourierGeom(O.padded_geom(img)[0])
    from lentils_gb300.gridding import GriddingPlan
    p = GriddingPlan(np.zeros((0, 3)), [1.0], four.nu, four.nv, four.du, four.dv, wsup=3)
    assert p.nvis == 0
    g = torch.zeros((four.nu, four.half_nv), dtype=torch.complex64, device="cuda")
    assert p.degrid(g).numel() == 0
    assert float(p.grid(torch.zeros(0, dtype=torch.complex64, device="cuda")).abs().sum()) == 0.0
    vis = O.VisGeom(np.array([[3.3 * four.du, -2.2 * four.dv, 0.0]]), [1.0])
    plan = make_plan(vis, four, 3, O.kb_beta(3))
    g = rng.normal(size=four.shape) + 1j * rng.normal(size=four.shape)
    assert O.rel_l2(gpu_degrid(plan, g), O.degrid(vis, four, g, 3, O.kb_beta(3))) < REL_L2_FP32


def test_plan_errors(native):
    from lentils_gb300._native import LentilsError
    from lentils_gb300.gridding import GriddingPlan
    img = O.ImageGeom((32, 32), [(-0.32, 0.32), (-0.32, 0.32)])
    four = O.FourierGeom(O.padded_geom(img)[0])
    far = np.array([[0.49 * four.nu * four.du, 0.0, 0.0]])
    with pytest.raises(LentilsError) as e:
        GriddingPlan(far, [1.0], four.nu, four.nv, four.du, four.dv, wsup=3, nyquist_guard=True)
    assert e.value.code == 2
    bad = np.array([[np.nan, 0.0, 0.0]])
    with pytest.raises(LentilsError) as e:
        GriddingPlan(bad, [1.0], four.nu, four.nv, four.du, four.dv, wsup=3)
    assert e.value.code == 7
    with pytest.raises(LentilsError) as e:
        GriddingPlan(far * 0.1, [1.0], four.nu, four.nv, four.du, four.dv, wsup=9)
    assert e.value.code == 5


def test_host_forms_accumulate(native):
    d, vis, four = load_nufft_golden("nufft_odd_w4")
    w, beta = int(d["wsup"]), float(d["beta"])
    plan = make_plan(vis, four, w, beta)
    v = d["vis_acc0"].copy()
    plan.degrid_host(d["grid_in"], v, accumulate=True)
    assert O.rel_l2(v - d["vis_acc0"], d["vis_out"] - d["vis_acc0"]) < REL_L2_FP32
    v2 = plan.degrid_host(d["grid_in"], np.full_like(v, 5.0), accumulate=False)
    assert O.rel_l2(v2, d["vis_out"] - d["vis_acc0"]) < REL_L2_FP32
    g = d["grid_acc0"].copy()
    plan.grid_host(d["vis_in"], g, accumulate=True)
    assert O.rel_l2(g - d["grid_acc0"], d["grid_out"] - d["grid_acc0"]) < REL_L2_FP32


def test_host_forms_page_locked(native):
    """Page-locked host buffers take the direct path (the kernels read and write host memory);
    same results as the staging path, with and without accumulation."""
    d, vis, four = load_nufft_golden("nufft_odd_w4")
    w, beta = int(d["wsup"]), float(d["beta"])
    plan = make_plan(vis, four, w, beta)

    def pinned(a):
        return torch.as_tensor(np.ascontiguousarray(a, dtype=np.complex128)).pin_memory()

    v = pinned(d["vis_acc0"])
    plan.degrid_host(pinned(d["grid_in"]), v, accumulate=True)
    assert O.rel_l2(v.numpy() - d["vis_acc0"], d["vis_out"] - d["vis_acc0"]) < REL_L2_FP32
    v2 = pinned(np.full_like(d["vis_acc0"], 5.0))
    plan.degrid_host(pinned(d["grid_in"]), v2, accumulate=False)
    assert O.rel_l2(v2.numpy(), d["vis_out"] - d["vis_acc0"]) < REL_L2_FP32
    g = pinned(d["grid_acc0"])
    plan.grid_host(pinned(d["vis_in"]), g, accumulate=True)
    assert O.rel_l2(g.numpy() - d["grid_acc0"], d["grid_out"] - d["grid_acc0"]) < REL_L2_FP32
    g2 = pinned(np.full_like(d["grid_acc0"], 3.0))
    plan.grid_host(pinned(d["vis_in"]), g2, accumulate=False)
    assert O.rel_l2(g2.numpy(), d["grid_out"] - d["grid_acc0"]) < REL_L2_FP32
    # the staging path on pageable memory gives the same numbers
    vs = plan.degrid_host(d["grid_in"], np.zeros_like(d["vis_acc0"]))
    assert O.rel_l2(vs, v2.numpy()) < 1e-7


@pytest.fixture(scope="module")
def full_size(native):
    """The full-size single-operator workload: 1e7 visibilities on the 2048 x 2048 grid (W=8),
    90% with density ~ 1/|uv| to 0.48 Nyquist and 10% in 50 Gaussian blobs."""
    rng = np.random.default_rng(2024)
    img, four, vis = nufft_setup(rng, (1024, 1024), [(-10.24, 10.24), (-10.24, 10.24)], [1.0],
                                 4, 10_000_000, 0.48, blobs=True)
    w, beta = 4, O.kb_beta(4)
    plan = make_plan(vis, four, w, beta)
    return rng, four, vis, w, beta, plan


def test_full_size_properties(full_size):
    """The weighted adjoint identity on a Hermitian-consistent grid at 1e7 visibilities, and
    degrid against the oracle on sampled visibilities."""
    rng, four, vis, w, beta, plan = full_size
    st = plan.stats
    assert st["nvis"] == 10_000_000 and st["heaviest_tile_vis"] > st["max_item_vis"]
    z = torch.randn((four.nu, four.nv), dtype=torch.float64, device="cuda")
    gh = torch.fft.rfft2(z)
    g = gh.to(torch.complex64)
    y = torch.complex(torch.randn(vis.nvis, device="cuda"), torch.randn(vis.nvis, device="cuda"))
    dg = plan.degrid(g)
    gy = plan.grid(y)
    lhs = torch.vdot(y.to(torch.complex128), dg.to(torch.complex128)).real
    wcol = torch.full((four.half_nv,), 2.0, dtype=torch.float64, device="cuda")
    wcol[0] = 1.0
    rhs = (wcol[None, :] * (g.to(torch.complex128).conj() * gy.to(torch.complex128)).real).sum()
    assert abs(float(lhs - rhs)) <= 1e-5 * float(torch.sqrt((dg.abs() ** 2).sum() * (y.abs() ** 2).sum()))
    # degrid: sampled visibilities against the oracle (degridding is per visibility)
    vis_user = plan.from_plan(dg).cpu().numpy()
    idx = np.sort(rng.choice(vis.nvis, 20000, replace=False))
    sub = O.VisGeom(vis.uvw[idx], [1.0])
    ref = O.degrid(sub, four, g.cpu().numpy().astype(np.complex128), w, beta)
    assert O.rel_l2(vis_user[idx], ref) < REL_L2_FP32


def test_full_size_fp32_vs_oracle(full_size):
    """Every one of the 1e7 visibilities, both directions, FP32 kernels against the FP64
    oracle (the C restatement of grid_cpu, all host cores): relative L2 <= 1e-5 over all
    visibilities and over the whole grid, and separately over the grid cells under the dense
    blobs, where each cell sums tens of thousands of FP32 contributions. The FP64 GPU operator
    (lentils_degrid64 / lentils_grid64, the reference the benchmark reports its error against)
    is checked on the same inputs to 1e-9."""
    rng, four, vis, w, beta, plan = full_size
    g32 = (torch.randn((four.nu, four.half_nv), dtype=torch.complex64, generator=None)
           .cuda())
    y32 = torch.randn(vis.nvis, dtype=torch.complex64).cuda()
    g64, y64 = g32.cpu().numpy().astype(np.complex128), y32.cpu().numpy().astype(np.complex128)
    dg = plan.from_plan(plan.degrid(g32)).cpu().numpy()
    gy = plan.grid(plan.to_plan(y32)).cpu().numpy().astype(np.complex128)
    ref_d = O.degrid(vis, four, g64, w, beta)
    ref_g = O.grid(vis, four, y64, w, beta)
    e_d, e_g = O.rel_l2(dg, ref_d), O.rel_l2(gy, ref_g)
    assert e_d < REL_L2_FP32, e_d
    assert e_g < REL_L2_FP32, e_g
    # cells under the blobs: the 1% of cells whose 9x9 neighbourhood holds the most visibilities
    cnt = np.zeros((four.nu, four.half_nv))
    ug = np.rint(vis.uvw[:, 0] / four.du).astype(np.int64) % four.nu
    vg = np.rint(-vis.uvw[:, 1] / four.dv).astype(np.int64) % four.nv
    fold = vg >= four.half_nv
    ug[fold], vg[fold] = (four.nu - ug[fold]) % four.nu, four.nv - vg[fold]
    np.add.at(cnt, (ug, vg), 1.0)
    dense = cnt >= np.quantile(cnt[cnt > 0], 0.99)
    assert cnt[dense].sum() > 0.05 * vis.nvis
    e_blob = O.rel_l2(gy[dense], ref_g[dense])
    assert e_blob < REL_L2_FP32, e_blob
    # the FP64 GPU operator on the same inputs (plan order -> row order in FP64)
    y64p = torch.empty(vis.nvis, dtype=torch.complex128, device="cuda")
    from lentils_gb300 import _native as N
    import ctypes
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    yt = torch.as_tensor(y64).cuda()
    N.check(N.lib().lentils_vis_to_plan64(plan.handle, ctypes.c_void_p(yt.data_ptr()),
                                          ctypes.c_void_p(y64p.data_ptr()), sp))
    G64 = plan.grid64(y64p).cpu().numpy()
    assert O.rel_l2(G64, ref_g) < 1e-9
    v64p = plan.degrid64(torch.as_tensor(g64).cuda())
    v64u = torch.zeros(vis.nvis, dtype=torch.complex128, device="cuda")
    N.check(N.lib().lentils_vis_from_plan64(plan.handle, ctypes.c_void_p(v64p.data_ptr()),
                                            ctypes.c_void_p(v64u.data_ptr()), 0, sp))
    assert O.rel_l2(v64u.cpu().numpy(), ref_d) < 1e-9
