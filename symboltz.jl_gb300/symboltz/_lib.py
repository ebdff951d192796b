"""ctypes binding of libsymboltz_gb300.so (include/symboltz_gb300.h).

The library is the product path: there is no CPU fallback.  Loading fails loudly when the shared
library has not been built, and compute entry points fail loudly when no CUDA device is present.
"""
import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "lib", "libsymboltz_gb300.so")

SBZ_OK, SBZ_MAXITERS, SBZ_DTMIN, SBZ_NONFINITE = 0, 1, 2, 3
SBZ_ERR_ARG, SBZ_ERR_CUDA, SBZ_ERR_NOMEM, SBZ_ERR_STATE = -1, -2, -3, -4
SBZ_FP64, SBZ_MIXED = 0, 1
SBZ_OUT_SOURCES, SBZ_OUT_DELTA_M, SBZ_OUT_STATE, SBZ_OUT_SOURCES4, SBZ_OUT_FACTORS = 0, 1, 2, 3, 4

EXPORTS = (
    "sbz_default_opts", "sbz_last_error", "sbz_momentum_quadrature", "sbz_problem_create", "sbz_problem_destroy", "sbz_problem_set_params",
    "sbz_problem_nstate", "sbz_solve_bg", "sbz_bg_knots", "sbz_bg_eval", "sbz_bg_coefficients", "sbz_solve_pt", "sbz_solve_pt_device", "sbz_pt_rhs",
    "sbz_spectrum_matter", "sbz_spectrum_primordial", "sbz_bessel_create", "sbz_bessel_destroy", "sbz_bessel_eval",
    "sbz_los_integrate", "sbz_los_integrate_device", "sbz_cl_integrate", "sbz_cl_integrate_noalloc", "sbz_autotune_pt", "sbz_mlp_gemm", "sbz_surrogate_create", "sbz_surrogate_destroy", "sbz_surrogate_nparams",
    "sbz_surrogate_get_params", "sbz_surrogate_set_params", "sbz_surrogate_set_data", "sbz_surrogate_train",
    "sbz_surrogate_gradients", "sbz_surrogate_infer", "sbz_surrogate_save", "sbz_surrogate_load", "sbz_trainset_append", "sbz_trainset_info", "sbz_trainset_read", "sbz_spectrum_cmb", "sbz_spectrum_cmb_sources", "sbz_problem_set_stream",
    "sbz_problem_timings",
)
SBZ_KINTERP_SPLINE, SBZ_KINTERP_BARYCENTRIC = 0, 1


class Params(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("h", "Omega_c", "Omega_b", "T0", "Neff", "YHe", "ln_As1e10", "ns", "m_nu_eV", "N_nu")]


class Model(C.Structure):
    _fields_ = [(n, C.c_int) for n in
                ("lmax_gamma", "lmax_nu", "lmax_h", "nx_h", "Hswitch", "Heswitch", "reionization")]


class Opts(C.Structure):
    _fields_ = [("bg_rtol", C.c_double), ("bg_atol", C.c_double), ("pt_rtol", C.c_double), ("pt_atol", C.c_double),
                ("tau_ini", C.c_double), ("tau_max", C.c_double), ("maxiters", C.c_int64), ("precision", C.c_int),
                ("refine_iters", C.c_int), ("table_points", C.c_int), ("warps_per_block", C.c_int),
                ("warps_per_mode", C.c_int), ("blocks_per_sm", C.c_int),
                ("los_precision", C.c_int), ("refine_skip", C.c_double)]


class SbzError(RuntimeError):
    pass


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise SbzError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() (no CPU fallback exists)")
    L = C.CDLL(LIB_PATH)
    dp, ip, i64p, vp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_int64), C.c_void_p
    L.sbz_default_opts.argtypes = [C.POINTER(Opts)]
    L.sbz_default_opts.restype = None
    L.sbz_last_error.restype = C.c_char_p
    L.sbz_momentum_quadrature.argtypes = [C.c_int, dp, dp]
    L.sbz_problem_create.argtypes = [C.POINTER(Model), C.POINTER(Params), C.c_int, C.POINTER(Opts), C.POINTER(vp)]
    L.sbz_problem_set_params.argtypes = [vp, C.POINTER(Params), C.c_int]
    L.sbz_problem_destroy.argtypes = [vp]
    L.sbz_problem_destroy.restype = None
    L.sbz_problem_nstate.argtypes = [vp]
    L.sbz_solve_bg.argtypes = [vp, dp, dp, dp, ip]
    L.sbz_bg_knots.argtypes = [vp, C.c_int, C.c_int, dp, dp]
    L.sbz_bg_eval.argtypes = [vp, C.c_int, C.c_int, dp, dp]
    L.sbz_bg_coefficients.argtypes = [vp, C.c_int, C.c_int, dp, dp]
    L.sbz_solve_pt.argtypes = [vp, C.c_int, ip, dp, dp, C.c_int, dp, C.c_int, dp, ip, i64p]
    L.sbz_autotune_pt.argtypes = [vp, C.c_int, ip, dp, dp, C.c_int, dp, C.c_int, ip, dp]
    fp = C.POINTER(C.c_float)
    L.sbz_surrogate_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.POINTER(vp)]
    L.sbz_surrogate_destroy.argtypes = [vp]
    L.sbz_surrogate_destroy.restype = None
    L.sbz_surrogate_nparams.argtypes = [vp]
    L.sbz_surrogate_nparams.restype = C.c_longlong
    L.sbz_surrogate_get_params.argtypes = [vp, fp]
    L.sbz_surrogate_set_params.argtypes = [vp, fp]
    L.sbz_surrogate_set_data.argtypes = [vp, C.c_longlong, fp, fp]
    L.sbz_surrogate_train.argtypes = [vp, C.c_int, C.c_double, dp]
    L.sbz_surrogate_gradients.argtypes = [vp, C.c_int, fp, fp, dp, fp]
    L.sbz_surrogate_infer.argtypes = [vp, C.c_longlong, fp, fp]
    L.sbz_surrogate_save.argtypes = [vp, C.c_char_p]
    L.sbz_surrogate_load.argtypes = [C.c_char_p, C.c_int, C.POINTER(vp)]
    fp = C.POINTER(C.c_float)
    L.sbz_trainset_append.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_longlong, fp, fp]
    L.sbz_trainset_info.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_longlong)]
    L.sbz_trainset_read.argtypes = [C.c_char_p, C.c_longlong, C.c_longlong, fp, fp]
    L.sbz_mlp_gemm.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, C.c_int, C.c_int, vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp]
    L.sbz_solve_pt_device.argtypes = [vp, C.c_int, vp, vp, vp, C.c_int, vp, C.c_int, vp, vp, vp]
    L.sbz_pt_rhs.argtypes = [vp, C.c_int, ip, dp, dp, dp, dp, dp]
    L.sbz_spectrum_matter.argtypes = [vp, C.c_int, ip, dp, C.c_double, C.c_double, dp, ip]
    L.sbz_spectrum_primordial.argtypes = [vp, C.c_int, C.c_int, dp, dp]
    L.sbz_bessel_create.argtypes = [C.c_int, ip, C.c_double, C.c_double, C.c_int, C.POINTER(vp)]
    L.sbz_bessel_destroy.argtypes = [vp]
    L.sbz_bessel_destroy.restype = None
    L.sbz_bessel_eval.argtypes = [vp, C.c_int, C.c_int, dp, dp]
    L.sbz_los_integrate.argtypes = [vp, C.c_int, dp, C.c_int, dp, C.c_int, dp, C.c_int, dp]
    L.sbz_los_integrate_device.argtypes = [vp, C.c_int, vp, C.c_int, vp, C.c_int, vp, C.c_int, vp, vp]
    L.sbz_cl_integrate.argtypes = [C.c_int, dp, dp, C.c_int, dp, dp, dp]
    L.sbz_cl_integrate_noalloc.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p]
    L.sbz_spectrum_cmb.argtypes = [vp, C.c_int, vp, C.c_int, dp, dp, dp, C.c_int, C.c_int, dp, C.c_int, dp, dp, C.c_int,
                                   ip, ip, C.c_int, dp, ip]
    L.sbz_spectrum_cmb_sources.argtypes = [vp, C.c_int, vp, C.c_int, dp, dp, dp, C.c_int, C.c_int, dp, dp, C.c_int, dp, dp, C.c_int,
                                           ip, ip, C.c_int, dp]
    L.sbz_problem_set_stream.argtypes = [vp, vp]
    L.sbz_problem_timings.argtypes = [vp, dp]
    _lib = L
    return L


def check(code, what=""):
    if code < 0:
        raise SbzError(f"{what}: {lib().sbz_last_error().decode()} (code {code})")
    return code


def dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def i64ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)
