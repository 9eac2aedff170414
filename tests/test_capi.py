"""The C-ABI library on the CPU (no GPU calls): it loads, exports every function the public
header declares, its by-value structs have the reference's layout, and its host-only
Kaiser-Bessel polynomial table reproduces the reference weight kb_g
(lentils/backend/nufft.c:11-21) to FP32 round-off."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle as O

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "lentils_gb300.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", src)
    return sorted(set(n for n in names if n not in ("if", "while", "sizeof")))


def test_header_declares_dropins():
    fns = header_functions()
    for n in ("grid_cpu", "deflect_points", "grad_matrix_findiff_csr", "lentils_plan_create",
              "lentils_degrid", "lentils_grid"):
        assert n in fns


def test_library_exports_every_declared_symbol(native):
    lib = native.lib()
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding declares signatures for all of them
    assert set(header_functions()) <= set(native.declared_functions())


def test_struct_layouts_match_reference(native):
    # sizes of the reference structs on LP64 (common.h, deflect.h)
    assert ctypes.sizeof(native.ImageSpaceC) == 80
    assert ctypes.sizeof(native.FourierSpaceC) == 64
    assert ctypes.sizeof(native.VisibilitySpaceC) == 32
    assert ctypes.sizeof(native.GlobalLensModelC) == 16
    assert O.MASS_MODEL_DTYPE.itemsize == 320
    assert ctypes.sizeof(native.ImageSpaceC) == ctypes.sizeof(O.CImageSpace)
    assert ctypes.sizeof(native.FourierSpaceC) == ctypes.sizeof(O.CFourierSpace)
    assert ctypes.sizeof(native.VisibilitySpaceC) == ctypes.sizeof(O.CVisibilitySpace)


@pytest.mark.parametrize("w", [1, 2, 3, 4, 5, 6, 7, 8])
def test_kb_polynomial_table_matches_reference_weight(native, w, oracle_mod):
    beta = O.kb_beta(w)
    table, fit_err = native.kb_poly_table(w, beta)
    assert fit_err < 1e-8
    lib = O.port_lib()
    peak = lib.oracle_bessel_i0(beta) / (2 * w)
    worst = 0.0
    for f in np.linspace(0.0, 1.0, 57)[:-1]:
        t = np.float32(2 * f - 1)
        for i in range(2 * w):
            acc = np.float32(table[i, 0])
            for c in table[i, 1:]:
                acc = np.float32(acc * t + np.float32(c))
            a = f + w - 1 - i
            # per-axis factor of kb_g: I0(beta*sqrt(1-(a/w)^2)) / (2w), times (-1)^i
            ref = (-1) ** i * lib.oracle_bessel_i0(beta * np.sqrt(max(0.0, 1 - (a / w) ** 2))) / (2 * w)
            worst = max(worst, abs(float(acc) - ref) / peak)
    assert worst < 3e-7


def test_kb_table_rejects_bad_width(native):
    out = np.zeros(400, dtype=np.float32)
    err = ctypes.c_double()
    st = native.lib().lentils_kb_poly_table(0, 10.0, out.ctypes.data, out.size, ctypes.byref(err))
    assert st == 1 and native.lib().lentils_last_error() == 1
    st = native.lib().lentils_kb_poly_table(9, 10.0, out.ctypes.data, out.size, ctypes.byref(err))
    assert st == 1


def test_unet_entry_points_reject_bad_arguments(native):
    """The U-Net entry points check their arguments before touching a device: sizes that are not
    multiples of 8 (or below 16), unknown GEMM forms and null handles are LENTILS_ERR_INVALID."""
    lib = native.lib()
    params = np.zeros(native_param_count(lib), dtype=np.float32)
    h = ctypes.c_void_p()
    for H, W, B in ((12, 16, 1), (16, 20, 1), (16, 16, 0)):
        st = lib.lentils_unet_create(ctypes.byref(h), H, W, B, params.ctypes.data, None)
        assert st == 1 and lib.lentils_last_error() == 1, (H, W, B)
    assert lib.lentils_unet_set_gemm_form(None, 0) == 1
    assert lib.lentils_unet_set_gemm_form(None, 3) == 1


def native_param_count(lib):
    return int(lib.lentils_unet_param_count())
