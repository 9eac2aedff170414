"""GPU lens equation through the C ABI against the FP64 oracle and the golden fixtures
generated by the reference's own deflect_points (lentils/backend/deflect.c:60-66)."""
import ctypes

import numpy as np
import pytest
import torch

import oracle as O

pytestmark = pytest.mark.gpu

# FP32 arithmetic: deflection angles within 1e-5 relative L2 of FP64, positions within
# 2e-6 arcsec (|alpha| ~ 1 arcsec here).
REL_ALPHA = 1e-5
ABS_POS = 2e-6


def gpu_deflect(lenses, pts, f32=False):
    from lentils_gb300 import _native as N
    L = N.lib()
    lenses = np.ascontiguousarray(lenses, dtype=O.MASS_MODEL_DTYPE)
    dt = torch.float32 if f32 else torch.float64
    p = torch.as_tensor(np.ascontiguousarray(pts), dtype=dt).cuda().contiguous()
    out = torch.empty_like(p)
    fn = L.lentils_deflect_f32 if f32 else L.lentils_deflect_f64io
    N.check(fn(ctypes.c_void_p(lenses.ctypes.data), len(lenses), ctypes.c_void_p(p.data_ptr()),
               ctypes.c_void_p(out.data_ptr()), p.numel() // 2,
               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return out.double().cpu().numpy()


def check(lenses, pts, f32=False):
    ref = O.deflect(lenses, pts)
    got = gpu_deflect(lenses, pts, f32)
    fin = np.isfinite(ref).all(axis=-1)
    assert np.array_equal(fin, np.isfinite(got).all(axis=-1))
    a_ref = (pts - ref)[fin]
    a_got = (pts - got)[fin]
    assert O.rel_l2(a_got.reshape(-1), a_ref.reshape(-1)) < REL_ALPHA
    if not f32:
        assert np.max(np.abs(got[fin] - ref[fin])) < ABS_POS


@pytest.mark.parametrize("case", ["pemd_shear", "pemd_lowq", "shear_grad", "multipoles"])
def test_golden(native, golden_dir, case):
    d = np.load(f"{golden_dir}/deflect.npz")
    lenses = np.ascontiguousarray(d[f"{case}_lenses"]).view(O.MASS_MODEL_DTYPE).reshape(-1)
    pts = d["points"]
    ref = d[f"{case}_out"]
    got = gpu_deflect(lenses, pts)
    fin = np.isfinite(ref).all(axis=-1)
    assert np.array_equal(fin, np.isfinite(got).all(axis=-1))
    assert O.rel_l2((pts - got)[fin].reshape(-1), (pts - ref)[fin].reshape(-1)) < REL_ALPHA


def test_config0_pemd(native):
    """128^2 pixel grid, b = 1.0, q = 0.8, PA 30, gamma = 2.1, centre (0.05, -0.03)."""
    img = O.ImageGeom((128, 128), [(-1.28, 1.28), (-1.28, 1.28)])
    lenses = O.lens_array([O.pemd_cpars(1.0, 30.0, 0.8, 0.05, -0.03, 0.55)])
    check(lenses, img.points())
    check(lenses, img.points(), f32=True)


def test_prior_sweep(native):
    """The batched sweep's priors: b in [0.8,1.6], q in [0.5,0.95], gamma in [1.8,2.3],
    shear up to 0.1, on a 64^2 grid per draw."""
    rng = np.random.default_rng(5)
    img = O.ImageGeom((64, 64), [(-2.0, 2.0), (-2.0, 2.0)])
    pts = img.points() + 1e-3
    for _ in range(20):
        g = rng.uniform(1.8, 2.3)
        x0, y0 = rng.uniform(-0.1, 0.1, 2)
        lenses = O.lens_array([
            O.pemd_cpars(rng.uniform(0.8, 1.6), rng.uniform(-90, 90), rng.uniform(0.5, 0.95),
                         x0, y0, (g - 1) / 2),
            O.shear_cpars(x0, y0, rng.uniform(0, 0.1), rng.uniform(-90, 90))])
        check(lenses, pts)


def test_many_lenses(native):
    """More lenses than one launch carries (multiple launches accumulate)."""
    rng = np.random.default_rng(6)
    pts = rng.uniform(-2, 2, (3000, 2))
    models = [O.pemd_cpars(0.3, rng.uniform(0, 90), rng.uniform(0.6, 0.9),
                           *rng.uniform(-1, 1, 2), 0.5) for _ in range(11)]
    models += [O.shear_cpars(0.0, 0.0, 0.02, 10.0)]
    check(O.lens_array(models), pts)


def test_singular_centre_gives_nan(native):
    lenses = O.lens_array([O.pemd_cpars(1.0, 30.0, 0.8, 0.05, -0.03, 0.55)])
    pts = np.array([[0.05, -0.03], [0.5, 0.5]])
    got = gpu_deflect(lenses, pts)
    ref = O.deflect(lenses, pts)
    assert not np.isfinite(ref[0]).all() and not np.isfinite(got[0]).all()
    assert np.isfinite(got[1]).all()


def test_dropin_deflect_points(native, golden_dir):
    from lentils_gb300 import _native as N
    d = np.load(f"{golden_dir}/deflect.npz")
    lenses = np.ascontiguousarray(d["pemd_shear_lenses"]).view(O.MASS_MODEL_DTYPE).reshape(-1)
    pts = np.ascontiguousarray(d["points"])
    out = np.zeros_like(pts)
    glm = N.GlobalLensModelC(len(lenses), 1, lenses.ctypes.data)
    dummy = np.zeros(1)
    N.lib().deflect_points(glm, pts.ctypes.data, pts.shape[0], out.ctypes.data, 0,
                           dummy.ctypes.data)
    N.check_last()
    ref = d["pemd_shear_out"]
    fin = np.isfinite(ref).all(axis=-1)
    assert O.rel_l2((pts - out)[fin].reshape(-1), (pts - ref)[fin].reshape(-1)) < REL_ALPHA



def _deriv_case(golden_dir, name):
    d = np.load(f"{golden_dir}/deflect_deriv.npz")
    lenses = np.ascontiguousarray(d[f"{name}_lenses"]).view(O.MASS_MODEL_DTYPE).reshape(-1)
    return d, lenses, np.ascontiguousarray(d["points"])


@pytest.mark.parametrize("name", ["pemd_shear", "two_pemd"])
def test_dropin_deflect_points_want_deriv(native, golden_dir, name):
    """want_deriv = 1: deriv[0..11] += the PEMD derivatives summed over the points, exactly
    what the compiled reference accumulates (deflect.c:330-338); the rest of the caller's
    gradient array (allocated (8, npoints, 2) by lens_models.py:71-73) is left alone."""
    from lentils_gb300 import _native as N
    d, lenses, pts = _deriv_case(golden_dir, name)
    glm = N.GlobalLensModelC(len(lenses), 1, lenses.ctypes.data)
    out = np.zeros_like(pts)
    rng = np.random.default_rng(1)
    deriv0 = rng.normal(size=(8,) + pts.shape)
    deriv = deriv0.copy()
    N.lib().deflect_points(glm, pts.ctypes.data, pts.shape[0], out.ctypes.data, 1,
                           deriv.ctypes.data)
    N.check_last()
    flat, flat0 = deriv.reshape(-1), deriv0.reshape(-1)
    scale = np.abs(d[f"{name}_per_point"]).sum(axis=0) + 1e-300
    err = np.abs((flat[:12] - flat0[:12]) - d[f"{name}_sum12"]) / scale
    assert err.max() < 1e-12, err
    assert np.array_equal(flat[12:], flat0[12:])


def test_deflect_gradients_per_point(native, golden_dir):
    """lentils_deflect_grad against the compiled reference's per-point PEMD derivatives, and
    the external shear's (x, y, ss, sa) derivatives against central differences of the
    reference's deflection."""
    from lentils_gb300 import _native as N
    from lentils_gb300.gridding import _ptr
    L = N.lib()
    for name, params in (("two_pemd", range(6)), ("pemd_shear", (0, 1, 2, 5))):
        d, lenses, pts = _deriv_case(golden_dir, name)
        p = torch.as_tensor(pts).cuda()
        g = torch.empty((8,) + pts.shape, dtype=torch.float64, device="cuda")
        N.check(L.lentils_deflect_grad(lenses.ctypes.data, len(lenses), _ptr(p), _ptr(g),
                                       pts.shape[0], None))
        got = g.cpu().numpy()
        ref = d[f"{name}_per_point"].reshape(-1, 6, 2).transpose(1, 0, 2)
        for k in params:
            assert O.rel_l2(got[k], ref[k]) < 1e-11, (name, k, O.rel_l2(got[k], ref[k]))
    d = np.load(f"{golden_dir}/deflect_deriv.npz")
    lenses = np.ascontiguousarray(d["shear_lenses"]).view(O.MASS_MODEL_DTYPE).reshape(-1)
    p = torch.as_tensor(np.ascontiguousarray(d["points"])).cuda()
    g = torch.empty((8,) + tuple(p.shape), dtype=torch.float64, device="cuda")
    N.check(L.lentils_deflect_grad(lenses.ctypes.data, 1, _ptr(p), _ptr(g), p.shape[0], None))
    got = g.cpu().numpy()
    for k, i in ((3, 0), (4, 1), (6, 2), (7, 3)):
        assert O.rel_l2(got[k], d["shear_fd"][i]) < 1e-6, (k, O.rel_l2(got[k], d["shear_fd"][i]))
    assert np.abs(got[[0, 1, 2, 5]]).max() == 0.0
