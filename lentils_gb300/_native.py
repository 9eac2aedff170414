"""ctypes binding of liblentils_gb300.so (the C ABI declared in include/lentils_gb300.h).

The library is built in-tree by ``lentils_gb300.build``. Loading fails loudly when it is
missing: there is no CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import (POINTER, Structure, c_char, c_char_p, c_double, c_float, c_int,
                    c_longlong, c_void_p)

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "liblentils_gb300.so")

LENTILS_OK = 0
ERROR_NAMES = {0: "OK", 1: "INVALID", 2: "NYQUIST", 3: "ALLOC", 4: "CUDA", 5: "UNSUPPORTED",
               6: "TIMEOUT", 7: "NONFINITE", 8: "NO_DEVICE"}

PLAN_UVW_ON_DEVICE = 1
PLAN_NYQUIST_GUARD = 2


class LentilsError(RuntimeError):
    def __init__(self, code, message):
        self.code = code
        super().__init__(f"lentils_gb300 error {ERROR_NAMES.get(code, code)}: {message}")


# --- by-value structs (reference ABI: lentils/backend/common.h, deflect.h) -----------------
class ImageSpaceC(Structure):
    _fields_ = [("nx", c_int), ("ny", c_int), ("num_channels", c_int), ("num_stokes", c_int),
                ("xmin", c_double), ("xmax", c_double), ("ymin", c_double), ("ymax", c_double),
                ("dx", c_double), ("dy", c_double), ("_c_channels", POINTER(c_double)),
                ("_c_mask", POINTER(c_char))]


class FourierSpaceC(Structure):
    _fields_ = [("nu", c_int), ("nv", c_int), ("half_nv", c_int), ("num_channels", c_int),
                ("num_stokes", c_int), ("du", c_double), ("dv", c_double), ("gcx", c_double),
                ("gcy", c_double), ("_c_channels", POINTER(c_double))]


class VisibilitySpaceC(Structure):
    _fields_ = [("num_rows", c_int), ("num_channels", c_int), ("num_stokes", c_int),
                ("_c_uvw", POINTER(c_double)), ("_c_channels", POINTER(c_double))]


class GlobalLensModelC(Structure):
    _fields_ = [("num_lenses", c_int), ("num_zplanes", c_int), ("lenses", c_void_p)]


class GridDescC(Structure):
    _fields_ = [("nu", c_int), ("nv", c_int), ("du", c_double), ("dv", c_double),
                ("gcx", c_double), ("gcy", c_double), ("wsup", c_int), ("kb_beta", c_double),
                ("tile", c_int), ("chunk", c_int)]


class CGOptionsC(Structure):
    _fields_ = [("tol", c_double), ("inner_tol", c_double), ("max_outer", c_int),
                ("max_inner", c_int), ("check_every", c_int), ("use_graph", c_int),
                ("window", c_int), ("net_every", c_int)]


class CGResultC(Structure):
    _fields_ = [("converged", c_int), ("outer", c_int), ("inner_total", c_int),
                ("rel_residual", c_double), ("seconds", c_double), ("net_iterations", c_int),
                ("fallback", c_int)]


class SweepSampleC(Structure):
    _fields_ = [("plan", c_void_p), ("grid_in", c_void_p), ("vis_out", c_void_p),
                ("vis_in", c_void_p), ("grid_out", c_void_p), ("lenses", c_void_p),
                ("nlenses", c_int), ("nx", c_int), ("ny", c_int), ("x0", c_double),
                ("y0", c_double), ("dx", c_double), ("dy", c_double), ("beta_out", c_void_p)]


class SweepStatsC(Structure):
    _fields_ = [("nsamples", c_int), ("nwork", c_int), ("blocks", c_int),
                ("smem_bytes", c_longlong), ("total_vis", c_longlong),
                ("total_pixels", c_longlong), ("algorithmic_bytes", c_double)]


class PlanStatsC(Structure):
    _fields_ = [("nvis", c_longlong), ("ntiles_u", c_int), ("ntiles_v", c_int), ("tile", c_int),
                ("nitems", c_int), ("max_item_vis", c_int), ("heaviest_tile_vis", c_int),
                ("wsup", c_int), ("has_phase", c_int), ("device_bytes", c_longlong)]


# (name, restype, argtypes) for every function in include/lentils_gb300.h
_SIGNATURES = [
    ("lentils_last_error", c_int, []),
    ("lentils_last_error_message", c_char_p, []),
    ("lentils_version", c_int, []),
    ("lentils_kb_poly_table", c_int, [c_int, c_double, c_void_p, c_int, POINTER(c_double)]),
    ("lentils_kb_poly_ncoef", c_int, []),
    ("grid_cpu", None, [VisibilitySpaceC, c_void_p, FourierSpaceC, c_void_p, c_int, c_double,
                        c_int]),
    ("deflect_points", None, [GlobalLensModelC, c_void_p, c_int, c_void_p, c_int, c_void_p]),
    ("grad_matrix_findiff_csr", None, [ImageSpaceC, c_void_p, c_void_p, c_void_p]),
    ("lentils_dropin_cache_mode", c_int, [c_int]),
    ("lentils_dropin_cache_clear", c_int, []),
    ("lentils_dropin_cache_size", c_int, []),
    ("lentils_plan_create", c_int, [POINTER(c_void_p), POINTER(GridDescC), c_void_p, c_int,
                                    c_void_p, c_int, c_int, c_void_p]),
    ("lentils_plan_destroy", c_int, [c_void_p]),
    ("lentils_plan_get_stats", c_int, [c_void_p, POINTER(PlanStatsC)]),
    ("lentils_plan_set_grid_variant", c_int, [c_void_p, c_int]),
    ("lentils_plan_set_degrid_variant", c_int, [c_void_p, c_int]),
    ("lentils_degrid", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_grid", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_vis_to_plan", c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p]),
    ("lentils_vis_from_plan", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p]),
    ("lentils_degrid_host", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    ("lentils_grid_host", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    ("lentils_degrid64", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_grid64", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_vis_to_plan64", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_vis_from_plan64", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    ("lentils_plan_gather_real", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_nufft_create", c_int, [POINTER(c_void_p), c_void_p, c_int, c_int, c_int, c_int,
                                     c_void_p, c_void_p, c_int, c_void_p]),
    ("lentils_nufft_destroy", c_int, [c_void_p]),
    ("lentils_nufft_forward", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_nufft_adjoint", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_nufft_forward64", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_nufft_adjoint64", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_lensop_create", c_int, [POINTER(c_void_p), c_void_p, c_void_p, c_int, c_int, c_int,
                                      c_double, c_double, c_double, c_double, c_void_p]),
    ("lentils_lensop_destroy", c_int, [c_void_p]),
    ("lentils_lensop_nnz", c_int, [c_void_p]),
    ("lentils_lensop_apply", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_lensop_apply_t", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_lensop_apply64", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_lensop_apply_t64", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_lensop_diag_ltl", c_int, [c_void_p, c_void_p, c_void_p]),
    ("lentils_normal_op_create", c_int, [POINTER(c_void_p), c_void_p, c_void_p, c_void_p,
                                         c_longlong, c_int, c_int, c_int, c_double, c_double,
                                         c_double, c_void_p]),
    ("lentils_normal_op_destroy", c_int, [c_void_p]),
    ("lentils_normal_op_apply", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_normal_op_apply64", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_normal_op_rhs64", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_normal_op_jacobi", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_normal_op_weight_sum", c_double, [c_void_p]),
    ("lentils_device_free", c_int, [c_void_p]),
    ("lentils_copy_to_host", c_int, [c_void_p, c_void_p, c_longlong]),
    ("lentils_lensop_create_csr", c_int, [POINTER(c_void_p), c_void_p, c_void_p, c_void_p, c_int,
                                          c_int, c_int, c_void_p]),
    ("lentils_manifold_lens_matrix", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p,
                                             POINTER(c_void_p), POINTER(c_void_p),
                                             POINTER(c_void_p), POINTER(c_longlong), c_void_p]),
    ("lentils_deflect64", c_int, [c_void_p, c_int, c_void_p, c_void_p, c_longlong, c_void_p]),
    ("lentils_delaunay_lens_matrix", c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p,
                                             c_void_p, c_void_p, POINTER(c_void_p),
                                             POINTER(c_void_p), POINTER(c_void_p),
                                             POINTER(c_longlong), c_void_p]),
    ("lentils_dft_forward", c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p]),
    ("lentils_dft_adjoint", c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p]),
    ("lentils_bcb_create", c_int, [POINTER(c_void_p), c_void_p, c_int, c_int, c_void_p]),
    ("lentils_bcb_destroy", c_int, [c_void_p]),
    ("lentils_bcb_apply", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_bcb_apply64", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_bcb_centre", c_double, [c_void_p]),
    ("lentils_normal_op_create_bcb", c_int, [POINTER(c_void_p), c_void_p, c_void_p, c_int, c_int,
                                             c_int, c_double, c_double, c_double, c_void_p]),
    ("lentils_normal_op_rhs_image64", c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("lentils_cg_solve", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, POINTER(CGOptionsC),
                                 POINTER(CGResultC), c_void_p]),
    ("lentils_prior_gradient_apply", c_int, [c_void_p, c_void_p, c_int, c_int, c_double,
                                             c_double, c_double, c_void_p]),
    ("lentils_prior_gradient_apply64", c_int, [c_void_p, c_void_p, c_int, c_int, c_double,
                                               c_double, c_double, c_void_p]),
    ("lentils_dot64", c_int, [c_void_p, c_void_p, c_int, POINTER(c_double), c_void_p]),
    ("lentils_tc_timeout_selftest", c_int, [c_void_p, c_int, c_void_p]),
    ("lentils_tc_gemm_bf16", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int,
                                     c_void_p, c_void_p]),
    ("lentils_unet_param_count", c_longlong, []),
    ("lentils_unet_create", c_int, [POINTER(c_void_p), c_int, c_int, c_int, c_void_p, c_void_p]),
    ("lentils_unet_destroy", c_int, [c_void_p]),
    ("lentils_unet_get_params", c_int, [c_void_p, c_void_p]),
    ("lentils_unet_set_params", c_int, [c_void_p, c_void_p, c_void_p]),
    ("lentils_unet_forward", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    ("lentils_unet_gradients", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p,
                                       c_void_p, c_void_p]),
    ("lentils_unet_train_step", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_float,
                                        c_void_p, c_void_p]),
    ("lentils_unet_error_flag", c_int, [c_void_p, POINTER(c_int)]),
    ("lentils_unet_set_jacobi_weight", c_int, [c_void_p, c_float]),
    ("lentils_unet_set_gemm_form", c_int, [c_void_p, c_int]),
    ("lentils_unet_set_wgrad_ctas", c_int, [c_void_p, c_int]),
    ("lentils_unet_backward", c_int, [c_void_p, c_void_p, c_int, c_float, c_void_p, c_void_p]),
    ("lentils_unet_features", c_int, [c_void_p, c_void_p, c_int, c_void_p]),
    ("lentils_unet_precondition", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                          c_void_p]),
    ("lentils_fcg_solve", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                  POINTER(CGOptionsC), POINTER(CGResultC), c_void_p]),
    ("lentils_sweep_create", c_int, [POINTER(c_void_p), POINTER(SweepSampleC), c_int, c_int,
                                     c_void_p]),
    ("lentils_sweep_destroy", c_int, [c_void_p]),
    ("lentils_sweep_run", c_int, [c_void_p, c_int, c_void_p]),
    ("lentils_sweep_get_stats", c_int, [c_void_p, POINTER(SweepStatsC)]),
    ("lentils_grid_noalloc", c_int, [POINTER(GridDescC), c_void_p, c_int, c_void_p, c_int,
                                     c_void_p, c_void_p, c_void_p]),
    ("lentils_noalloc_max_vis", c_int, []),
    ("lentils_noalloc_scratch_bytes", c_longlong, []),
    ("lentils_deflect_f32", c_int, [c_void_p, c_int, c_void_p, c_void_p, c_longlong, c_void_p]),
    ("lentils_deflect_f64io", c_int, [c_void_p, c_int, c_void_p, c_void_p, c_longlong,
                                      c_void_p]),
    ("lentils_deflect_grad", c_int, [c_void_p, c_int, c_void_p, c_void_p, c_longlong,
                                     c_void_p]),
]

_LIB = None


def lib():
    """The loaded library (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise LentilsError(8, f"{LIB_PATH} is missing; run lentils_gb300.build.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in _SIGNATURES:
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def declared_functions():
    return [n for n, _, _ in _SIGNATURES]


def check(status):
    """Raise LentilsError for a non-zero status."""
    if status != LENTILS_OK:
        L = lib()
        msg = L.lentils_last_error_message()
        raise LentilsError(status, msg.decode() if msg else "")
    return status


def check_last():
    """Raise if the most recent call on this thread (a void drop-in entry) failed."""
    L = lib()
    code = L.lentils_last_error()
    if code != LENTILS_OK:
        raise LentilsError(code, L.lentils_last_error_message().decode())


def kb_poly_table(w, beta):
    """Per-tap polynomial table (2w x ncoef) and its FP64 fit error (host only)."""
    L = lib()
    ncoef = L.lentils_kb_poly_ncoef()
    out = np.zeros((2 * w, ncoef), dtype=np.float32)
    err = c_double(0.0)
    check(L.lentils_kb_poly_table(int(w), float(beta), out.ctypes.data, out.size,
                                  ctypes.byref(err)))
    return out, err.value
