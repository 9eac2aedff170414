"""The CPU oracle, pinned: the C restatement against the reference's own compiled C sources
(bit for bit, when they can be built here) and against the committed golden fixtures; the
restated NUFFT composition against the direct Fourier transform (the reference's
test_gridder_and_apodization, lentils/tests/nufft_tests.py:43-66, seeded); the adjoint
relations of the r2c gridder."""
import os

import numpy as np
import pytest
import scipy.special as sp

import oracle as O
from helpers import ERRTOL, load_nufft_golden

NUFFT_CASES = ["nufft_cfg0_w3", "nufft_odd_w4", "nufft_tiny_w1"]


def test_i0_shim_accuracy(oracle_mod):
    lib = O.port_lib()
    xs = np.concatenate([np.linspace(0, 45, 4001), [60.0, 80.0]])
    err = max(abs(lib.oracle_bessel_i0(x) / sp.i0(x) - 1) for x in xs)
    assert err < 1e-13


@pytest.mark.parametrize("name", NUFFT_CASES)
def test_port_matches_golden_nufft(oracle_mod, name):
    d, vis, four = load_nufft_golden(name)
    w, beta = int(d["wsup"]), float(d["beta"])
    v = d["vis_acc0"].copy()
    O.grid_cpu(vis, v, four, d["grid_in"].copy(), w, beta, 0)
    assert np.array_equal(v, d["vis_out"])
    g = d["grid_acc0"].copy()
    O.grid_cpu(vis, d["vis_in"].copy(), four, g, w, beta, 1)
    # the adjoint's OpenMP atomics make the summation order thread-dependent
    assert np.max(np.abs(g - d["grid_out"])) <= 1e-12 * np.max(np.abs(d["grid_out"]))


def test_port_matches_golden_deflect(oracle_mod, golden_dir):
    d = np.load(f"{golden_dir}/deflect.npz")
    for k in ("pemd_shear", "pemd_lowq", "shear_grad", "multipoles"):
        lenses = np.ascontiguousarray(d[f"{k}_lenses"]).view(O.MASS_MODEL_DTYPE).reshape(-1)
        out = O.deflect(lenses, d["points"])
        assert np.array_equal(out, d[f"{k}_out"], equal_nan=True), k


def test_port_matches_golden_grad(oracle_mod, golden_dir):
    d = np.load(f"{golden_dir}/grad_csr.npz")
    img = O.ImageGeom((int(d["nx"]), int(d["ny"])), d["bounds"])
    rows, cols, vals = O.grad_csr(img)
    assert np.array_equal(rows, d["rows"])
    assert np.array_equal(cols, d["cols"])
    assert np.array_equal(vals, d["vals"])


@pytest.mark.skipif(not O.build_ref(), reason="reference C sources not present")
def test_port_bitwise_equals_compiled_reference(oracle_mod):
    rng = np.random.default_rng(5)
    img = O.ImageGeom((40, 51), [(-0.3, 0.5), (-0.6, 0.2)])
    padded, _, _ = O.padded_geom(img, 2)
    four = O.FourierGeom(padded)
    vis = O.VisGeom(O.synth_uv(rng, 300, four, 0.45, 3), [1.0, 0.7])
    g = rng.normal(size=four.shape) + 1j * rng.normal(size=four.shape)
    beta = O.kb_beta(3)
    assert np.array_equal(O.degrid(vis, four, g, 3, beta), O.degrid(vis, four, g, 3, beta, True))
    lenses = O.lens_array([O.pemd_cpars(1.1, 10.0, 0.7, 0.0, 0.1, 0.5),
                           O.shear_cpars(0.0, 0.1, 0.03, 5.0)])
    pts = rng.uniform(-2, 2, (500, 2))
    assert np.array_equal(O.deflect(lenses, pts), O.deflect(lenses, pts, True))


def _kat_setup(seed):
    # nufft_tests.py:43-66: 20 scales x 4 points, channel 0.5, 236x257 image with asymmetric
    # bounds; seeded here (the reference draws unseeded)
    rng = np.random.default_rng(seed)
    all_uv = np.concatenate([rng.normal(scale=1e5 * s, size=(4, 3))
                             for s in np.linspace(0.0, 55.0, 20)])
    vis = O.VisGeom(all_uv, [0.5])
    img = O.ImageGeom((236, 257), [(-0.5, 0.7), (-0.7, 0.5)])
    return rng, vis, img


def test_nufft_vs_dft_known_answer(oracle_mod):
    rng, vis, img = _kat_setup(7)
    nufft = O.NufftOracle(vis, img, 2, 4)
    assert O.nyquist_ok(vis, nufft.four, 4)
    vdata = rng.normal(size=(vis.nrows, 2)).view(np.complex128).reshape(-1)
    mat = O.dft_matrix(vis, img)
    dftvec = O.dft_adjoint(mat, vdata).reshape(img.shape)
    assert O.max_relative_error(nufft.adjoint(vdata), dftvec) < ERRTOL
    assert O.max_relative_error(nufft.forward(dftvec), O.dft_forward(mat, dftvec)) < ERRTOL


def test_adjoint_relations(oracle_mod):
    """<degrid(g), y> = sum_cols w_col <g, grid(y)> with w = 1 on column 0 and 2 elsewhere,
    for a Hermitian-consistent g = rfft2(real); and the full NUFFT chain is self-adjoint
    under the real inner product."""
    rng = np.random.default_rng(9)
    img = O.ImageGeom((64, 64), [(-0.64, 0.64), (-0.64, 0.64)])
    vis = O.VisGeom(O.synth_uv(rng, 500, O.FourierGeom(O.padded_geom(img)[0]), 0.45, 3), [1.0])
    nufft = O.NufftOracle(vis, img, 2, 3)
    z = rng.normal(size=nufft.padded.shape)
    g = np.fft.rfft2(z)
    y = O.complex_normal(rng, vis.nvis)
    lhs = np.vdot(y, O.degrid(vis, nufft.four, g, 3, nufft.beta)).real
    gy = O.grid(vis, nufft.four, y, 3, nufft.beta)
    wcol = np.full(nufft.four.half_nv, 2.0)
    wcol[0] = 1.0
    if nufft.four.nv % 2 == 0:
        wcol[-1] = 1.0
    rhs = np.sum(wcol[None, :] * (np.conj(g) * gy).real)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    x = rng.normal(size=img.shape)
    a = np.vdot(y, nufft.forward(x)).real
    b = np.sum(x * nufft.adjoint(y))
    assert abs(a - b) <= 1e-12 * abs(a)


def test_oracle_dirty_beam_form_matches_explicit_normal_operator():
    """The dirty-beam convolution (data_base.py:115-129) equals F^T C^-1 F through the
    visibilities up to the NUFFT's own accuracy (small image, W = 8)."""
    rng = np.random.default_rng(12)
    img = O.ImageGeom((24, 20), [(-0.24, 0.24), (-0.2, 0.2)])
    four = O.FourierGeom(O.padded_geom(img, 2)[0])
    vis = O.VisGeom(O.synth_uv(rng, 3000, four, 0.45, 4), [1.0])
    w = rng.uniform(0.5, 2.0, vis.nvis)
    ora = O.NufftOracle(vis, img, 2, 4)
    beam = O.dirty_beam(vis, img, w, 4)
    assert beam.shape == (48, 40)
    x = rng.normal(size=img.shape)
    explicit = ora.adjoint(w * ora.forward(x))
    assert O.rel_l2(O.bcb_apply(beam, img, x), explicit) < 1e-6


def test_derivative_fixture_matches_reference():
    """The committed derivative fixture is what the compiled reference computes (regenerated
    here when oracle/_ref is available)."""
    import pytest
    if not O.ref_available():
        pytest.skip("compiled reference not available")
    from helpers import GOLDEN
    d = np.load(os.path.join(GOLDEN, "deflect_deriv.npz"))
    for name in ("pemd_shear", "two_pemd"):
        lenses = np.ascontiguousarray(d[f"{name}_lenses"]).view(O.MASS_MODEL_DTYPE).reshape(-1)
        total, per = O.deflect_derivatives_ref(lenses, d["points"])
        assert np.array_equal(total, d[f"{name}_sum12"])
        assert np.array_equal(per, d[f"{name}_per_point"])


def test_manifold_fixture_matches_reference():
    """The committed manifold-matrix fixture is what the compiled reference computes."""
    import pytest
    if O.ref_lib("raster") is None:
        pytest.skip("compiled reference not available")
    from helpers import GOLDEN
    d = np.load(os.path.join(GOLDEN, "manifold.npz"))
    for name in ("wide", "small_src"):
        gi, gs = d[f"{name}_img"], d[f"{name}_src"]
        img = O.ImageGeom((int(gi[0]), int(gi[1])), gi[2:6])
        img.mask[...] = d[f"{name}_mask"].astype(bool)
        src = O.ImageGeom((int(gs[0]), int(gs[1])), gs[2:6])
        lenses = np.ascontiguousarray(d[f"{name}_lenses"]).view(O.MASS_MODEL_DTYPE).reshape(-1)
        r, c, v = O.manifold_lens_matrix_ref(img, src, lenses)
        assert np.array_equal(r, d[f"{name}_rows"]) and np.array_equal(c, d[f"{name}_cols"])
        assert np.array_equal(v, d[f"{name}_vals"])


def test_delaunay_fixture_matches_reference():
    """The committed Delaunay fixture is what the compiled reference (deflect_points and
    delaunay_lens_matrix_csr) computes with scipy's triangulation."""
    import pytest
    if O.ref_lib("triangles") is None or not O.ref_available():
        pytest.skip("compiled reference not available")
    from helpers import GOLDEN
    d = np.load(os.path.join(GOLDEN, "delaunay.npz"))
    lenses = np.ascontiguousarray(d["lenses"]).view(O.MASS_MODEL_DTYPE).reshape(-1)
    assert np.array_equal(O.deflect(lenses, d["image_casted"], use_ref=True), d["casted"])
    gi = d["img"]
    img = O.ImageGeom((int(gi[0]), int(gi[1])), gi[2:6])
    img.mask[...] = d["mask"].astype(bool)
    r, c, v = O.delaunay_lens_matrix_ref(img, int(d["ncast"]), d["casted"], d["uncasted"],
                                         d["triangles"], d["tri_inds"])
    assert np.array_equal(r, d["rows"]) and np.array_equal(c, d["cols"])
    assert np.array_equal(v, d["vals"])
