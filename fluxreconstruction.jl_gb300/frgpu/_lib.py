"""ctypes binding of libfrgpu.so (declared in include/frgpu.h).

The library is loaded from the package directory.  There is no fallback: if
the shared object is missing or cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

OK = 0
ERR_ARG, ERR_CUDA, ERR_NONFINITE, ERR_UNPHYSICAL, ERR_DT, ERR_TIMEOUT, ERR_UNSUPPORTED = -1, -2, -3, -4, -5, -6, -7

ADVECTION, BURGERS, EULER1D, EULER2D, BGK1D = 0, 1, 2, 3, 4
FLUX_ROE, FLUX_LF, FLUX_HLL, FLUX_UPWIND, FLUX_CENTRAL = 0, 1, 2, 3, 4
FP64, FP32K = 0, 1
BC_PERIODIC, BC_COPY, BC_FIXED, BC_DIRICHLET = 0, 1, 2, 3
RADAU, SD, HUYNH = 0, 1, 2
IND_NONE, IND_PLAIN, IND_MLP = 0, 1, 2
OPT_BGK_TENSOR, OPT_FUSED_INDICATOR, OPT_FUSED_TWO_STAGE, OPT_BGK_CLOSURE, OPT_GHOSTS_PER_STEP = 1, 2, 3, 4, 5

_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int)
_VP = C.c_void_p


class ProblemDesc(C.Structure):
    _fields_ = [
        ("equation", C.c_int), ("flux", C.c_int), ("precision", C.c_int),
        ("bc", C.c_int * 4),
        ("fixed_state", (C.c_double * 4) * 4),
        ("a", C.c_double), ("gamma", C.c_double), ("tau", C.c_double),
        ("nvel", C.c_int), ("velo", _D), ("weights", _D),
        ("eps_interior", C.c_double), ("eps_periodic", C.c_double),
    ]


# name -> (restype, argtypes); exactly the entry points of include/frgpu.h
SIGNATURES = {
    "frgpu_legendre_point": (C.c_int, [C.c_int, _D, _D]),
    "frgpu_lagrange_point": (C.c_int, [_D, C.c_int, C.c_double, _D]),
    "frgpu_dlagrange": (C.c_int, [_D, C.c_int, _D]),
    "frgpu_dcorrection": (C.c_int, [C.c_int, C.c_int, _D, C.c_int, _D, _D]),
    "frgpu_vandermonde": (C.c_int, [C.c_int, _D, C.c_int, _D]),
    "frgpu_vandermonde_quad": (C.c_int, [C.c_int, _D, _D, C.c_int, _D]),
    "frgpu_space_create_1d": (C.c_int, [C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(_VP)]),
    "frgpu_space_create_2d": (C.c_int, [C.c_double, C.c_double, C.c_int, C.c_double, C.c_double, C.c_int,
                                        C.c_int, C.POINTER(_VP)]),
    "frgpu_space_create_1d_ops": (C.c_int, [C.c_int, C.c_int, _D, _D, _D, _D, _D, _D, _D, _D, C.POINTER(_VP)]),
    "frgpu_space_create_2d_ops": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _D, _D, _D, _D,
                                            _D, _D, _D, C.POINTER(_VP)]),
    "frgpu_space_info": (C.c_int, [_VP, _I, _I, _I, _I]),
    "frgpu_space_get": (C.c_int, [_VP, C.c_char_p, _D, C.c_long]),
    "frgpu_space_destroy": (None, [_VP]),
    "frgpu_problem_create": (C.c_int, [_VP, C.POINTER(ProblemDesc), C.POINTER(_VP)]),
    "frgpu_problem_destroy": (None, [_VP]),
    "frgpu_problem_ndof": (C.c_long, [_VP]),
    "frgpu_state_upload": (C.c_int, [_VP, _D]),
    "frgpu_state_download": (C.c_int, [_VP, _D]),
    "frgpu_rhs": (C.c_int, [_VP, _D, _D, C.c_double]),
    "frgpu_step_ssprk3": (C.c_int, [_VP, C.c_double, C.c_int]),
    "frgpu_step_ssprk3_async": (C.c_int, [_VP, C.c_double, C.c_int]),
    "frgpu_cfl_dt": (C.c_int, [_VP, C.c_double, _D]),
    "frgpu_reduce": (C.c_int, [_VP, _D, _D]),
    "frgpu_set_filter": (C.c_int, [_VP, C.c_int, C.c_double, C.c_double, C.c_double]),
    "frgpu_problem_set_option": (C.c_int, [_VP, C.c_int, C.c_int]),
    "frgpu_modal_filter": (C.c_int, [_VP, C.c_int, C.c_double, C.c_double, C.c_double, _I]),
    "frgpu_troubled_flags": (C.c_int, [_VP, _I, C.c_long]),
    "frgpu_positive_limiter": (C.c_int, [_VP, _D, C.c_double, _I]),
    "frgpu_step_erk": (C.c_int, [_VP, C.c_int, _D, _D, C.c_double, C.c_int]),
    "frgpu_problem_set_flux_dissipation": (C.c_int, [_VP, C.c_double]),
    "frgpu_step_ssprk3_reduce": (C.c_int, [_VP, C.c_double, C.c_int, _D, _D]),
    "frgpu_step_rock": (C.c_int, [_VP, C.c_int, _D, _D, _D, _D, C.c_int, _D, _D, C.c_double, C.c_int]),
    "frgpu_spectral_radius": (C.c_int, [_VP, C.c_int, _D, _I]),
    "frgpu_rkc2_coefficients": (C.c_int, [C.c_int, C.c_double, _D, _D, _D, _D, _D]),
    "frgpu_step_rkc2": (C.c_int, [_VP, C.c_double, C.c_int, C.c_double, C.c_int, C.c_int, _I]),
    "frgpu_problem_set_metric": (C.c_int, [_VP, _D, _D, _D]),
    "frgpu_problem_set_face_jacobians": (C.c_int, [_VP, _D, _D, _D]),
    "frgpu_vandermonde_tri": (C.c_int, [C.c_int, _D, _D, C.c_int, _D, _D, _D]),
    "frgpu_tri_operators": (C.c_int, [C.c_int, _D, _D, _D, _D, _D, _D]),
    "frgpu_tri_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, _D, _D, _D, _D, _D, _I, _I, _I, _I,
                                   C.POINTER(_VP)]),
    "frgpu_tri_destroy": (C.c_int, [_VP]),
    "frgpu_tri_set_state": (C.c_int, [_VP, _D]),
    "frgpu_tri_get_state": (C.c_int, [_VP, _D]),
    "frgpu_tri_rhs": (C.c_int, [_VP, _D, _D]),
    "frgpu_tri_rhs_device": (C.c_int, [_VP]),
    "frgpu_tri_step_erk": (C.c_int, [_VP, C.c_int, _D, _D, C.c_double, C.c_int]),
    "frgpu_tri_stream": (C.c_int, [_VP, C.POINTER(_VP)]),
    "frgpu_tri_launches": (C.c_int, [_VP, C.POINTER(C.c_longlong)]),
    "frgpu_set_limiter": (C.c_int, [_VP, C.c_int, _D, C.c_double]),
    "frgpu_problem_device_state": (C.c_int, [_VP, C.POINTER(_VP), _I]),
    "frgpu_problem_stream": (C.c_int, [_VP, C.POINTER(_VP)]),
    "frgpu_problem_launches": (C.c_long, [_VP]),
    "frgpu_synchronize": (C.c_int, [_VP]),
    "frgpu_fma_peak": (C.c_int, [C.c_int, _D]),
    "frgpu_reduce2d_noalloc": (C.c_int, [_VP, _VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                         C.c_double, _VP, _VP, _VP]),
    "frgpu_mlp_nparams": (C.c_int, []),
    "frgpu_mlp_create": (C.c_int, [C.c_int, C.POINTER(_VP)]),
    "frgpu_mlp_destroy": (None, [_VP]),
    "frgpu_mlp_get_params": (C.c_int, [_VP, _F]),
    "frgpu_mlp_set_params": (C.c_int, [_VP, _F]),
    "frgpu_mlp_forward": (C.c_int, [_VP, _F, C.c_long, _F]),
    "frgpu_mlp_loss_grad": (C.c_int, [_VP, _F, _F, C.c_long, _F, _F]),
    "frgpu_mlp_train": (C.c_int, [_VP, _F, _F, C.c_long, C.c_int, C.c_int, C.c_float, C.c_int, _F]),
    "frgpu_problem_set_mlp": (C.c_int, [_VP, _VP, C.c_double, C.c_double]),
    "frgpu_modal_features": (C.c_int, [_VP, _F, C.c_long]),
    "frgpu_indicator_stats": (C.c_int, [_VP, _I]),
    "frgpu_ensemble_config4_sizes": (C.c_int, [C.c_int, C.c_uint, _I, _I]),
    "frgpu_ensemble_create": (C.c_int, [C.c_int, _I, _I, C.c_double, C.c_double, C.c_int, C.POINTER(_VP)]),
    "frgpu_ensemble_destroy": (None, [_VP]),
    "frgpu_ensemble_ndof": (C.c_long, [_VP]),
    "frgpu_ensemble_set_state": (C.c_int, [_VP, C.c_int, _D]),
    "frgpu_ensemble_get_state": (C.c_int, [_VP, C.c_int, _D]),
    "frgpu_ensemble_init_fourier": (C.c_int, [_VP, C.c_double, C.c_uint]),
    "frgpu_ensemble_set_tiles": (C.c_int, [_VP, _I]),
    "frgpu_ensemble_get_tiles": (C.c_int, [_VP, _I]),
    "frgpu_ensemble_run": (C.c_int, [_VP, C.c_double, C.c_double, C.c_int]),
    "frgpu_ensemble_stats": (C.c_int, [_VP, _D, _I, _F, _D, _I]),
    "frgpu_ensemble_tune": (C.c_int, [_VP, C.c_double, C.c_double, C.c_int, _I]),
    "frgpu_ensemble_launches": (C.c_long, [_VP]),
    "frgpu_ensemble_set_mlp": (C.c_int, [_VP, _VP, C.c_double, C.c_double]),
    "frgpu_ensemble_indicator_stats": (C.c_int, [_VP, C.POINTER(C.c_longlong)]),
    "frgpu_ensemble_nelem": (C.c_long, [_VP]),
    "frgpu_ensemble_failed": (C.c_int, [_VP, _I]),
    "frgpu_ensemble_features": (C.c_int, [_VP, _F, _I, C.c_long]),
    "frgpu_interp_face": (C.c_int, [_D, C.c_long, C.c_int, _D, _D, _D]),
    "frgpu_poly_derivative": (C.c_int, [_D, C.c_long, C.c_int, _D, _D]),
    "frgpu_last_error": (C.c_int, [C.c_char_p, C.c_ulong]),
    "frgpu_version": (C.c_int, []),
}

_lib = None


class FRGPUError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"frgpu error {code}: {msg}")
        self.code = code


def lib(build_if_missing: bool = True):
    """Load libfrgpu.so (building it first when sources are newer)."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if build_if_missing:
            try:
                path = _build.build()
            except RuntimeError:
                if not os.path.exists(path):
                    raise
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    lib().frgpu_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(rc: int) -> int:
    if rc < 0:
        raise FRGPUError(rc, last_error())
    return rc


def dptr(a):
    return a.ctypes.data_as(_D)


def fptr(a):
    return a.ctypes.data_as(_F)
