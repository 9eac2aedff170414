"""Drop-in grad_matrix_findiff_csr (reference signature, host buffers) against the golden
CSR produced by the reference's own C (lentils/backend/nufft.c:163-194): bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_grad_csr_bitwise(native, golden_dir):
    from lentils_gb300 import _native as N
    from lentils_gb300.spaces import ImageSpace
    d = np.load(f"{golden_dir}/grad_csr.npz")
    b = d["bounds"]
    im = ImageSpace((int(d["nx"]), int(d["ny"])), [(b[0], b[1]), (b[2], b[3])])
    n = im.nx * im.ny
    rows = np.zeros(2 * n + 1, dtype=np.int32)
    cols = np.zeros(4 * n, dtype=np.int32)
    vals = np.zeros(4 * n, dtype=np.float64)
    N.lib().grad_matrix_findiff_csr(im, rows.ctypes.data, cols.ctypes.data, vals.ctypes.data)
    N.check_last()
    assert np.array_equal(rows, d["rows"])
    assert np.array_equal(cols, d["cols"])
    assert np.array_equal(vals, d["vals"])


@pytest.mark.parametrize("shape", [(1, 1), (1, 7), (6, 1), (300, 211)])
def test_grad_csr_shapes(native, shape):
    import oracle as O
    from lentils_gb300 import _native as N
    from lentils_gb300.spaces import ImageSpace
    im = ImageSpace(shape, [(-0.3, 0.4), (-0.2, 0.5)])
    n = im.nx * im.ny
    rows = np.zeros(2 * n + 1, dtype=np.int32)
    cols = np.zeros(4 * n, dtype=np.int32)
    vals = np.zeros(4 * n, dtype=np.float64)
    N.lib().grad_matrix_findiff_csr(im, rows.ctypes.data, cols.ctypes.data, vals.ctypes.data)
    N.check_last()
    r, c, v = O.grad_csr(O.ImageGeom(shape, [(-0.3, 0.4), (-0.2, 0.5)]))
    assert np.array_equal(rows, r) and np.array_equal(cols, c) and np.array_equal(vals, v)
