"""lentils_grid_noalloc: gridding for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc -- code running in a host callback or a stream-ordered
section that must not synchronise, with device memory another framework's pool already
holds, or in a real-time pipeline that does not allocate after start-up. For them
lentils_grid_noalloc grids a bounded batch of visibilities from caller-owned device buffers
with all working memory in a static device array. These tests call it through the C ABI and
compare it with the plan path (lentils_plan_create + lentils_vis_to_plan + lentils_grid) on
two calls in a row with different inputs, so a result that leaned on the previous call's
scratch contents would show. This file is collected last so that a failure here cannot hide
any other test."""
import ctypes

import numpy as np
import pytest
import torch

import oracle as O
from helpers import REL_L2_FP32

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _grid_noalloc(N, four, w, beta, uvw, chans, vis, grid):
    desc = N.GridDescC(four.nu, four.nv, four.du, four.dv, four.gcx, four.gcy, w, beta, 0, 0)
    return N.lib().lentils_grid_noalloc(
        ctypes.byref(desc), _ptr(uvw), uvw.shape[0], _ptr(chans), chans.numel(), _ptr(vis),
        _ptr(grid), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def _case(seed, shape, bounds, chans, w, nrows):
    rng = np.random.default_rng(seed)
    img = O.ImageGeom(shape, bounds)
    four = O.FourierGeom(O.padded_geom(img, 2)[0])
    uvw = O.synth_uv(rng, nrows, four, 0.45, w) / max(chans)
    uvw[:3, :2] = [[0.0, 0.0], [3 * four.du, -2 * four.dv], [-7 * four.du, 5 * four.dv]]
    vis = O.complex_normal(rng, nrows * len(chans))
    return four, uvw, np.asarray(chans, float), vis


def test_noalloc_matches_plan_path_on_consecutive_calls(native):
    from lentils_gb300.gridding import GriddingPlan
    N = native
    cases = [
        _case(1, (512, 512), [(-5.12, 5.12), (-5.12, 5.12)], [1.0], 4, 60000),
        _case(2, (97, 120), [(-0.4, 0.6), (-0.7, 0.5)], [1.0, 0.6], 3, 9000),
    ]
    for four, uvw, chans, vis in cases:
        w = 4 if four.nu == 1024 else 3
        beta = O.kb_beta(w)
        uvw_t = torch.as_tensor(uvw).cuda()
        ch_t = torch.as_tensor(chans).cuda()
        vis_t = torch.as_tensor(vis.astype(np.complex64)).cuda()
        got = torch.zeros((four.nu, four.half_nv), dtype=torch.complex64, device="cuda")
        assert _grid_noalloc(N, four, w, beta, uvw_t, ch_t, vis_t, got) == 0, \
            N.lib().lentils_last_error_message()
        plan = GriddingPlan(uvw, chans, four.nu, four.nv, four.du, four.dv, four.gcx, four.gcy,
                            w, beta)
        want = plan.grid(plan.to_plan(vis_t))
        torch.cuda.synchronize()
        assert O.rel_l2(got.cpu().numpy(), want.cpu().numpy()) < REL_L2_FP32


def test_noalloc_rejects_batches_beyond_its_fixed_size(native):
    N = native
    cap = N.lib().lentils_noalloc_max_vis()
    assert cap == 65536
    assert 0 < N.lib().lentils_noalloc_scratch_bytes() < 16 << 20
    four, uvw, chans, vis = _case(3, (64, 64), [(-0.64, 0.64), (-0.64, 0.64)], [1.0], 2, cap + 1)
    uvw_t = torch.as_tensor(uvw).cuda()
    ch_t = torch.as_tensor(chans).cuda()
    vis_t = torch.as_tensor(vis.astype(np.complex64)).cuda()
    grid = torch.zeros((four.nu, four.half_nv), dtype=torch.complex64, device="cuda")
    st = _grid_noalloc(N, four, 2, O.kb_beta(2), uvw_t, ch_t, vis_t, grid)
    assert st == 1
    assert b"maximum" in N.lib().lentils_last_error_message()
    assert float(grid.abs().sum()) == 0.0


def test_noalloc_skips_nonfinite_rows_on_power_of_two_tile_count(native):
    """Rows with non-finite coordinates are skipped: on a 1024 x 1024 grid with 16-cell tiles
    (4096 tiles, a power of two) the result equals the plan path run without those rows, so the
    skipped rows' sort keys cannot fall into the last tile's range."""
    from lentils_gb300.gridding import GriddingPlan
    N = native
    four, uvw, chans, vis = _case(4, (512, 512), [(-5.12, 5.12), (-5.12, 5.12)], [1.0], 4,
                                  20000)
    assert (four.nu // 16) * (four.nv // 16) == 4096
    bad = np.array([5, 777, 19998])
    uvw_nan = uvw.copy()
    uvw_nan[bad[0], 0] = np.nan
    uvw_nan[bad[1], 1] = np.inf
    uvw_nan[bad[2], :2] = np.nan
    # a cluster in the last cell of the last tile (the top corner of the canonical window,
    # grid coordinates 511.x), whose keys would equal a skipped row's key if the key's tile
    # field had no room above the last tile
    off = np.random.default_rng(5).uniform(0.1, 0.6, (50, 2))
    uvw_nan[10:60, 0] = (four.nu // 2 - 1 + off[:, 0]) * four.du
    uvw_nan[10:60, 1] = -(four.nv // 2 - 1 + off[:, 1]) * four.dv
    w, beta = 4, O.kb_beta(4)
    got = torch.zeros((four.nu, four.half_nv), dtype=torch.complex64, device="cuda")
    vis_t = torch.as_tensor(vis.astype(np.complex64)).cuda()
    assert _grid_noalloc(N, four, w, beta, torch.as_tensor(uvw_nan).cuda(),
                         torch.as_tensor(chans).cuda(), vis_t, got) == 0, \
        N.lib().lentils_last_error_message()
    keep = np.setdiff1d(np.arange(uvw.shape[0]), bad)
    plan = GriddingPlan(uvw_nan[keep], chans, four.nu, four.nv, four.du, four.dv, four.gcx,
                        four.gcy, w, beta)
    want = plan.grid(plan.to_plan(vis_t[torch.as_tensor(keep).cuda()]))
    torch.cuda.synchronize()
    assert O.rel_l2(got.cpu().numpy(), want.cpu().numpy()) < REL_L2_FP32
