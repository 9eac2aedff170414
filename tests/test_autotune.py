"""The autotuner's accuracy model: its KB-width error bounds hold against the direct Fourier
sum (the oracle's dft_matrix, restating dft_matrix_csr, lentils/backend/nufft.c:128-161) for
the oracle NUFFT at beta = 2.34 W, and the narrower width is really less accurate."""
import numpy as np
import pytest

import oracle as O
from lentils_gb300 import autotune
from lentils_gb300 import autotune as A


def _kb_error(W, n=32, seed=5):
    rng = np.random.default_rng(seed)
    half = 0.5 * n * 0.02
    img = O.ImageGeom((n, n), [(-half, half), (-half, half)])
    four = O.FourierGeom(O.padded_geom(img, 2)[0])
    uvw = O.synth_uv(rng, 3000, four, 0.45, W // 2)
    vis = O.VisGeom(uvw, [1.0])
    x = rng.normal(size=(n, n))
    exact = O.dft_forward(O.dft_matrix(vis, img), x)
    approx = O.NufftOracle(vis, img, 2, W // 2, beta=autotune.kb_beta(W)).forward(x)
    return np.linalg.norm(approx - exact) / np.linalg.norm(exact)


def test_width_error_bounds_hold():
    e6, e8 = _kb_error(6), _kb_error(8)
    assert e6 <= autotune.KB_ERROR[6]
    assert e8 <= autotune.KB_ERROR[8]
    assert e6 > autotune.KB_ERROR[8]


def test_width_for():
    assert autotune.width_for(1e-4) == 6
    assert autotune.width_for(autotune.KB_ERROR[6]) == 6
    assert autotune.width_for(1e-6) == 8
    assert autotune.width_for(1e-12) == 8


def test_class_keys_and_buckets():
    assert A.nvis_bucket(1) == 0 and A.nvis_bucket(1 << 20) == 20
    assert A.nvis_bucket(1.4e6) == 20 and A.nvis_bucket(1.5e6) == 21
    assert A.Autotuner.key(2048, 2048, 8, 1e7) == "2048x2048/W8/n2^23"


def test_cache_hit_needs_no_tuning_and_round_trips(tmp_path):
    import json
    path = tmp_path / "tune.json"
    key = A.Autotuner.key(1024, 1024, 8, 2e6)
    path.write_text(json.dumps({key: {"tile": 8, "chunk": 2048, "ms": 0.11}}))
    t = A.Autotuner(path=str(path))
    assert t.params(1024, 1024, 1.0, 1.0, 8, 2e6) == (8, 2048)
    assert t.params(1024, 1024, 1.0, 1.0, 8, 1.9e6) == (8, 2048)  # same class
    assert t.tuned == 0
    t.save()
    assert json.loads(path.read_text())[key]["tile"] == 8
    with pytest.raises(ValueError):
        A.Autotuner(path=str(path), mode="other")


@pytest.mark.parametrize("name,tiles,chunks", [("sm_103.json", A.TILES, A.CHUNKS),
                                               ("sm_103_batched.json", A.BATCH_TILES,
                                                A.BATCH_CHUNKS)])
def test_committed_caches_are_well_formed(name, tiles, chunks):
    """Each class in the shipped caches names a candidate it timed, the fastest of them."""
    import json
    import os
    with open(os.path.join(A.DEFAULT_CACHE_DIR, name)) as f:
        cache = json.load(f)
    assert cache
    for key, e in cache.items():
        assert e["tile"] in tiles and e["chunk"] in chunks and e["ms"] > 0, key
        cands = e["candidates"]
        best = min(cands, key=lambda c: c["ms"])
        assert (best["tile"], best["chunk"]) == (e["tile"], e["chunk"]), key
