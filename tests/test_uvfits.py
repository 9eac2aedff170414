"""The uvfits loader (restating lentils/common/data_util.py:5-76 without astropy): a written
random-groups file read back with the reference loader's channel, data, sigma and mask rules,
and the reference's own uvfits files (when the reference tree is present)."""
import os

import numpy as np
import pytest

import oracle as O
from lentils_gb300 import uvfits


def _write(tmp_path, rng, nrows=40, nif=2, nchan=3, nst=2):
    uvw = rng.normal(0, 1e-3, (nrows, 3))
    vis = rng.normal(size=(nrows, nif, nchan, nst)) + 1j * rng.normal(size=(nrows, nif, nchan, nst))
    w = rng.uniform(0.5, 4.0, (nrows, nif, nchan, nst))
    w[rng.uniform(size=w.shape) < 0.1] = 0.0
    freq, chw, iff = 1.6e9, [2.5e5, 2.5e5], [0.0, 8e6][:nif]
    path = str(tmp_path / "t.uvfits")
    uvfits.write_uvfits(path, uvw, vis, w, freq, chw[:nif], iff)
    return path, uvw, vis.astype(np.complex64), w.astype(np.float32), freq, chw[:nif], iff


@pytest.mark.parametrize("combine", [False, True])
def test_roundtrip_reference_rules(tmp_path, combine):
    rng = np.random.default_rng(3)
    path, uvw, vis, w, freq, chw, iff = _write(tmp_path, rng)
    space, data, sigma, mask = uvfits.load_uvfits(path, combine_stokes=combine)
    nrows, nif, nchan, nst = vis.shape
    ch = (np.multiply.outer(np.asarray(chw), np.arange(nchan)) + np.asarray(iff)[:, None] + freq)
    assert np.allclose(space.channels, ch.flatten(), rtol=0, atol=1e-3)
    assert np.array_equal(space.uvw, uvw.astype(np.float32).astype(np.float64))
    v = vis.astype(np.complex128)
    s = np.zeros(w.shape)
    m = w > 0
    s[m] = w[m].astype(np.float64) ** -0.5
    if combine:
        m = np.all(m, axis=-1)
        v = 0.5 * (v[..., 0] + v[..., 1])
        s2 = np.zeros(m.shape)
        s2[m] = 0.5 * np.sqrt(s[..., 0][m] ** 2 + s[..., 1][m] ** 2)
        s = s2
    else:
        v, s, m = v[..., 0], s[..., 0], m[..., 0]
    exp = lambda a: np.moveaxis(a.reshape(nrows, nif * nchan, 1), [0, 1, 2], [2, 0, 1])
    assert data.shape == (nif * nchan, 1, nrows)
    assert np.allclose(data, exp(v), rtol=1e-7, atol=0)
    assert np.allclose(sigma, exp(s), rtol=1e-6, atol=0)
    assert np.array_equal(mask, exp(m))


def _ref_data(name):
    root = O.reference_root()
    return None if root is None else os.path.join(root, "lentils", "tests", "data_radio_2d",
                                                  name)


@pytest.mark.parametrize("name", ["input/j0751_small_snr1x.uvfits",
                                  "new_mock/j0751_lwmp_nopos_nosub_0.000000_tiny.uvfits"])
def test_reference_files(name):
    path = _ref_data(name)
    if path is None or not os.path.exists(path):
        pytest.skip("reference data not present")
    space, data, sigma, mask = uvfits.load_uvfits(path)
    hdus = uvfits.read_hdus(path)
    h = hdus[0][0]
    assert data.shape == (space.channels.size, 1, h["GCOUNT"])
    assert space.uvw.shape == (h["GCOUNT"], 3)
    assert np.all(np.isfinite(data)) and np.all(np.isfinite(space.uvw))
    assert np.all(sigma[mask] > 0) and np.all(sigma[~mask] == 0)
    assert space.channels[0] == pytest.approx(h["CRVAL4"], rel=1e-6)


@pytest.mark.parametrize("combine", [False, True])
@pytest.mark.parametrize("name", ["input/j0751_small_snr1x.uvfits",
                                  "new_mock/j0751_lwmp_nopos_nosub_0.000000_tiny.uvfits"])
def test_reference_files_element_wise(name, combine):
    """The reference's own uvfits files, loaded by lentils_gb300.uvfits and by an independent
    decoder of the FITS random-groups standard (tests/uvfits_decode.py, numpy structured
    records) with the reference loader's rules applied: uvw, channel frequencies, data, mask
    bit for bit; sigma to the FP32 rounding of the weights the file stores (the reference
    takes weight^-1/2 of the FP32 column)."""
    import uvfits_decode as D
    path = _ref_data(name)
    if path is None or not os.path.exists(path):
        pytest.skip("reference data not present")
    space, data, sigma, mask = uvfits.load_uvfits(path, combine_stokes=combine)
    uvw, chans, d2, s2, m2 = D.decode(path, combine_stokes=combine)
    assert np.array_equal(space.uvw, uvw)
    assert np.array_equal(space.channels, chans)
    assert data.shape == d2.shape and np.array_equal(data, d2)
    assert np.array_equal(mask, m2)
    assert 0 < mask.sum() <= mask.size
    assert np.all(sigma[~mask] == 0)
    assert np.allclose(sigma[mask], s2[mask], rtol=2e-7, atol=0)
