"""Generate the golden fixtures in tests/golden/ from the reference's own C code.

The reference's ``nufft.c`` and ``deflect.c`` are compiled unmodified by ``oracle/Makefile``
(target ``ref``) into ``oracle/_ref/`` (GSL's I0 replaced by the power-series shim in
``oracle/shim``); this script calls them through ctypes with one OpenMP thread on seeded
inputs and stores inputs and outputs as small ``.npz`` files. The fixtures pin the oracle port
(tests/test_oracle.py) and the GPU drop-ins (tests/test_dropin_gpu.py) wherever the
reference sources are absent.

Run from the repository root:  OMP_NUM_THREADS=1 python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
import oracle as O  # noqa: E402


def nufft_case(name, shape, bounds, chans, wsup, nvis, frac, seed, extra_uv=None):
    rng = np.random.default_rng(seed)
    img = O.ImageGeom(shape, bounds)
    padded, _, _ = O.padded_geom(img, 2)
    four = O.FourierGeom(padded)
    uvw = O.synth_uv(rng, nvis, four, frac, wsup) / max(chans)
    if extra_uv is not None:
        uvw = np.concatenate([uvw, extra_uv(four, chans)])
    vis = O.VisGeom(uvw, chans)
    beta = O.kb_beta(wsup)
    grid_in = (rng.normal(size=four.shape) + 1j * rng.normal(size=four.shape))
    vis_in = O.complex_normal(rng, vis.nvis)
    # accumulate onto non-zero outputs to pin the += semantics
    vis_acc0 = O.complex_normal(rng, vis.nvis) * 0.1
    grid_acc0 = (rng.normal(size=four.shape) + 1j * rng.normal(size=four.shape)) * 0.1
    vis_out = vis_acc0.copy()
    O.grid_cpu(vis, vis_out, four, grid_in.copy(), wsup, beta, 0, use_ref=True)
    grid_out = grid_acc0.copy()
    O.grid_cpu(vis, vis_in.copy(), four, grid_out, wsup, beta, 1, use_ref=True)
    np.savez_compressed(
        os.path.join(HERE, f"{name}.npz"), uvw=uvw, channels=np.asarray(chans, float),
        nu=four.nu, nv=four.nv, du=four.du, dv=four.dv, gcx=four.gcx, gcy=four.gcy,
        wsup=wsup, beta=beta, grid_in=grid_in, vis_in=vis_in, vis_acc0=vis_acc0,
        grid_acc0=grid_acc0, vis_out=vis_out, grid_out=grid_out)
    print(name, vis.nvis, four.shape)


def integer_points(four, chans):
    # uv exactly on grid cells (edge taps), the origin, and two points beyond the Nyquist
    # guard (exercise the wrap, nufft.c:83-86)
    pts = np.array([[0.0, 0.0, 0.0], [3 * four.du, -5 * four.dv, 0.0],
                    [-7 * four.du, 2 * four.dv, 0.0],
                    [0.49 * four.nu * four.du, 0.3 * four.nv * four.dv, 0.0],
                    [-0.6 * four.nu * four.du, -0.55 * four.nv * four.dv, 0.0]])
    pts[:, :2] /= chans[0]
    return pts


def deflect_case():
    rng = np.random.default_rng(11)
    img = O.ImageGeom((48, 40), [(-1.3, 1.1), (-1.0, 1.2)])
    pts = img.points().reshape(-1, 2)
    pts = np.concatenate([pts, rng.uniform(-2, 2, (200, 2)), [[0.05, -0.03]]])
    cases = {
        "pemd_shear": O.lens_array([O.pemd_cpars(1.0, 30.0, 0.8, 0.05, -0.03, 0.55),
                                    O.shear_cpars(0.05, -0.03, 0.05, 20.0)]),
        "pemd_lowq": O.lens_array([O.pemd_cpars(1.2, -40.0, 0.45, 0.1, 0.2, 0.45)]),
        "shear_grad": O.lens_array([O.shear_cpars(-0.1, 0.2, 0.07, 75.0, gks=0.02, gka=10.0,
                                                  gss=0.01, gsa=-30.0)]),
        "multipoles": O.lens_array([O.multipole_cpars(0.0, 0.1, 0.5, 4,
                                                      [[0.01, -0.02], [0.005, 0.003]])]),
    }
    out = {"points": pts}
    for k, lenses in cases.items():
        out[f"{k}_lenses"] = lenses.view(np.uint8).reshape(len(lenses), -1)
        out[f"{k}_out"] = O.deflect(lenses, pts, use_ref=True)
    np.savez_compressed(os.path.join(HERE, "deflect.npz"), **out)
    print("deflect", pts.shape)


def deflect_deriv_case():
    """Parameter derivatives (want_deriv) from the compiled reference, summed and per point;
    central finite differences of the reference's FP64 deflection for the external shear's
    parameters (whose derivative block the reference compiles out)."""
    rng = np.random.default_rng(13)
    img = O.ImageGeom((24, 20), [(-1.3, 1.1), (-1.0, 1.2)])
    pts = np.concatenate([img.points().reshape(-1, 2) + 0.013, rng.uniform(-2, 2, (100, 2))])
    cases = {
        "pemd_shear": O.lens_array([O.pemd_cpars(1.0, 30.0, 0.8, 0.05, -0.03, 0.55),
                                    O.shear_cpars(0.05, -0.03, 0.05, 20.0)]),
        "two_pemd": O.lens_array([O.pemd_cpars(1.2, -40.0, 0.55, 0.1, 0.2, 0.45),
                                  O.pemd_cpars(0.3, 75.0, 0.9, -0.4, 0.3, 0.6)]),
    }
    out = {"points": pts}
    for k, lenses in cases.items():
        total, per = O.deflect_derivatives_ref(lenses, pts)
        out[f"{k}_lenses"] = lenses.view(np.uint8).reshape(len(lenses), -1)
        out[f"{k}_sum12"] = total
        out[f"{k}_per_point"] = per
    # shear only: d beta / d (x, y, ss, sa) by central differences (beta = theta - alpha)
    par = dict(x=0.05, y=-0.03, ss=0.07, sa=20.0)
    steps = dict(x=1e-6, y=1e-6, ss=1e-6, sa=1e-4)
    fd = np.zeros((4, pts.shape[0], 2))
    for i, name in enumerate(("x", "y", "ss", "sa")):
        hi, lo = dict(par), dict(par)
        hi[name] += steps[name]
        lo[name] -= steps[name]
        bh = O.deflect(O.lens_array([O.shear_cpars(**hi)]), pts, use_ref=True)
        bl = O.deflect(O.lens_array([O.shear_cpars(**lo)]), pts, use_ref=True)
        fd[i] = -(bh - bl) / (2 * steps[name])  # d alpha = -d beta
    out["shear_lenses"] = O.lens_array([O.shear_cpars(**par)]).view(np.uint8).reshape(1, -1)
    out["shear_fd"] = fd
    np.savez_compressed(os.path.join(HERE, "deflect_deriv.npz"), **out)
    print("deflect_deriv", pts.shape)


def manifold_case():
    """The reference's ManifoldLensOperator matrix (raster.c:272-395) on two small cases: a
    PEMD + shear with a masked region, and a source grid smaller than the lensed image (pixels
    whose triangles miss it, which the reference gives a zero entry)."""
    out = {}
    cases = {
        "wide": (O.ImageGeom((24, 20), [(-0.6, 0.6), (-0.5, 0.5)]),
                 O.ImageGeom((16, 16), [(-0.4, 0.4), (-0.4, 0.4)]),
                 O.lens_array([O.pemd_cpars(0.45, 30.0, 0.75, 0.013, -0.011, 0.5),
                               O.shear_cpars(0.013, -0.011, 0.05, 20.0)])),
        "small_src": (O.ImageGeom((30, 26), [(-0.75, 0.75), (-0.65, 0.65)]),
                      O.ImageGeom((8, 10), [(-0.12, 0.12), (-0.15, 0.15)]),
                      O.lens_array([O.pemd_cpars(0.5, -20.0, 0.6, -0.02, 0.017, 0.6)])),
    }
    for k, (img, src, lenses) in cases.items():
        if k == "wide":
            img.mask[3:6, 4:9] = False
        r, c, v = O.manifold_lens_matrix_ref(img, src, lenses)
        out[f"{k}_img"] = np.concatenate([[img.nx, img.ny], img.bounds])
        out[f"{k}_src"] = np.concatenate([[src.nx, src.ny], src.bounds])
        out[f"{k}_mask"] = img.mask.astype(np.uint8)
        out[f"{k}_lenses"] = lenses.view(np.uint8).reshape(len(lenses), -1)
        out[f"{k}_rows"], out[f"{k}_cols"], out[f"{k}_vals"] = r, c, v
    np.savez_compressed(os.path.join(HERE, "manifold.npz"), **out)
    print("manifold", {k: int(out[f"{k}_rows"][-1]) for k in cases})


def delaunay_case():
    """The reference's DelaunayLensOperator pieces (lens_operators.py:43-80): rays deflected by
    the reference's deflect_points, scipy's triangulation and point location, and
    delaunay_lens_matrix_csr (triangles.c:105-140), for ncasted = 2 with a masked region."""
    from scipy.spatial import Delaunay
    img = O.ImageGeom((22, 18), [(-0.55, 0.55), (-0.45, 0.45)])
    img.mask[2:5, 3:7] = False
    lenses = O.lens_array([O.pemd_cpars(0.35, 25.0, 0.8, 0.011, -0.013, 0.5),
                           O.shear_cpars(0.011, -0.013, 0.04, 60.0)])
    ncast = 2
    pts = img.points()
    cmask = np.zeros(img.shape, bool)
    cmask[::ncast, ::ncast] = True
    umask = ~cmask
    cmask &= img.mask
    umask &= img.mask
    casted = O.deflect(lenses, pts[cmask], use_ref=True)
    uncasted = O.deflect(lenses, pts[umask], use_ref=True)
    tri = Delaunay(casted)
    tind = tri.find_simplex(uncasted)
    r, c, v = O.delaunay_lens_matrix_ref(img, ncast, casted, uncasted, tri.simplices, tind)
    np.savez_compressed(os.path.join(HERE, "delaunay.npz"), img=np.concatenate([[img.nx, img.ny], img.bounds]),
                        mask=img.mask.astype(np.uint8), ncast=ncast,
                        lenses=lenses.view(np.uint8).reshape(len(lenses), -1),
                        image_casted=pts[cmask], image_uncasted=pts[umask], casted=casted,
                        uncasted=uncasted, triangles=tri.simplices.astype(np.int32),
                        tri_inds=tind.astype(np.int32), rows=r, cols=c, vals=v)
    print("delaunay", int(r[-1]))


def grad_case():
    img = O.ImageGeom((13, 17), [(-0.4, 0.9), (-0.2, 0.6)])
    rows, cols, vals = O.grad_csr(img, use_ref=True)
    np.savez_compressed(os.path.join(HERE, "grad_csr.npz"), nx=img.nx, ny=img.ny,
                        bounds=img.bounds, rows=rows, cols=cols, vals=vals)
    print("grad_csr", img.shape)


if __name__ == "__main__":
    if not O.build_ref():
        sys.exit("the reference's C sources could not be compiled (oracle/_ref)")
    O.build_port()
    # config-0 geometry (128^2 image, 0.02" pixels, W=6), reduced visibility count
    nufft_case("nufft_cfg0_w3", (128, 128), [(-1.28, 1.28), (-1.28, 1.28)], [1.0], 3, 3000,
               0.45, 1)
    # odd, non-square, off-centre image with two channels and special points (W=8)
    nufft_case("nufft_odd_w4", (59, 64), [(-0.5, 0.7), (-0.7, 0.5)], [0.5, 0.8], 4, 400, 0.4,
               2, extra_uv=integer_points)
    # narrow kernel on a tiny grid (W=2)
    nufft_case("nufft_tiny_w1", (12, 9), [(-0.2, 0.3), (-0.1, 0.2)], [1.0], 1, 60, 0.5, 3,
               extra_uv=integer_points)
    deflect_case()
    deflect_deriv_case()
    manifold_case()
    delaunay_case()
    grad_case()
