"""frgpu: GB300-native flux-reconstruction residual and explicit time stepping.

The compute path is libfrgpu.so (hand-written CUDA for sm_103a behind the C ABI
of include/frgpu.h).  This package is its Python host binding; it mirrors the
FluxReconstruction.jl interface for the hot path (see ``api``).
"""
from ._lib import FRGPUError, lib, last_error  # noqa: F401
from .tri import (  # noqa: F401
    Euler,
    TriAdvectionProblem,
    TriFRPSpace,
    boundary_cell_type,
    read_gmsh,
    rs_jacobi,
    tri_operators,
    tri_space_from_gmsh,
    tri_square_mesh,
    tri_quadrature,
    triface_quadrature,
    xy_rs,
    vandermonde_tri,
)
from .api import (  # noqa: F401
    FRAdvectionProblem,
    FRBGKProblem,
    FRBurgersProblem,
    FREuler2DProblem,
    FREulerProblem,
    FRPSpace1D,
    FRPSpace2D,
    Integrator,
    L1_error,
    L2_error,
    Linf_error,
    quadrature_L2_error,
    refined_at_coarse_points,
    ODEProblem,
    RK4,
    SSPRK22,
    SSPRK33,
    ExplicitRK,
    Heun,
    Midpoint,
    Ralston,
    Tsit5,
    dhuynh,
    dlagrange,
    dradau,
    dsd,
    gauss_weights,
    fma_peak,
    init,
    interp_face_,
    lagrange_point,
    legendre_point,
    modal_filter_,
    poly_derivative_,
    quad_face_jacobians,
    quad_face_normals,
    quad_metric,
    rs_jacobi_quad,
    shock_detector,
    solve,
    standard_lagrange,
    step_,
    vandermonde_matrix,
)

__all__ = [n for n in dir() if not n.startswith("_")]
