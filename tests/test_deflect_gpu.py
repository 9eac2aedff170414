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
    # derivatives are not built: the call reports UNSUPPORTED and leaves p_out untouched
    out2 = np.full_like(pts, 7.0)
    N.lib().deflect_points(glm, pts.ctypes.data, pts.shape[0], out2.ctypes.data, 1,
                           dummy.ctypes.data)
    assert N.lib().lentils_last_error() == 5
    assert np.all(out2 == 7.0)
