"""
    FRGPU

Julia binding of libfrgpu.so (include/frgpu.h) for FluxReconstruction.jl users.
It keeps the reference's signatures for the residual / time-stepping hot path:

* `FRGPU.FRAdvectionProblem(u, tspan, ps, a, bc)` and
  `FRGPU.FREulerProblem(u, tspan, ps, γ, bc)` take the reference's own
  `FRPSpace1D` (src/struct.jl:13-88) and return an `ODEProblem` whose
  `rhs!(du, u, p, t)` runs on the GPU (src/Equation/eq_advection.jl:1-26,
  src/Equation/eq_euler.jl:1-27);
* `FRGPU.FREuler2DProblem(u, tspan, ps, γ; flux, bc, fixed)` takes the
  reference's `FRPSpace2D` (src/struct.jl:99-245) and stands in for the `dudt!`
  closure of example/shock-vortex.jl:26-118;
* `FRGPU.interp_face!(fδ, f, ll, lr)` (src/interpolate.jl:1-10);
* `FRGPU.init(prob, FRGPU.SSPRK33(); dt)` + `FRGPU.step!(itg)` + `itg.u` keep the
  state on the device between steps (OrdinaryDiffEq's init/step! API).

The library path comes from `ENV["FRGPU_LIB"]` (default: next to this file's
package, `../libfrgpu.so`).
"""
module FRGPU

using OrdinaryDiffEq: ODEProblem

const libfrgpu = get(ENV, "FRGPU_LIB", joinpath(@__DIR__, "..", "libfrgpu.so"))

const ADVECTION, BURGERS, EULER1D, EULER2D, BGK1D = Cint(0), Cint(1), Cint(2), Cint(3), Cint(4)
const FLUX = Dict(:roe => Cint(0), :lf => Cint(1), :hll => Cint(2), :upwind => Cint(3), :central => Cint(4))
const BC = Dict(:period => Cint(0), :copy => Cint(1), :fix => Cint(2), :dirichlet => Cint(3))
const PRECISION = Dict(:fp64 => Cint(0), :fp32k => Cint(1))

# mirror of frgpu_problem_desc (include/frgpu.h)
struct ProblemDesc
    equation::Cint
    flux::Cint
    precision::Cint
    bc::NTuple{4,Cint}
    fixed_state::NTuple{16,Cdouble}
    a::Cdouble
    gamma::Cdouble
    tau::Cdouble
    nvel::Cint
    velo::Ptr{Cdouble}
    weights::Ptr{Cdouble}
    eps_interior::Cdouble
    eps_periodic::Cdouble
end

function check(rc::Cint)
    if rc < 0
        buf = Vector{UInt8}(undef, 1024)
        ccall((:frgpu_last_error, libfrgpu), Cint, (Ptr{UInt8}, Culong), buf, length(buf))
        error("frgpu error $rc: " * unsafe_string(pointer(buf)))
    end
    return rc
end

mutable struct Space
    h::Ptr{Cvoid}
end

"""Device copy of the operators of a reference FRPSpace1D (src/struct.jl:40-85)."""
function Space(ps1d)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:frgpu_space_create_1d_ops, libfrgpu), Cint,
                (Cint, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble},
                 Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ref{Ptr{Cvoid}}),
                length(ps1d.J), ps1d.deg, collect(Float64, ps1d.J), collect(Float64, ps1d.ll),
                collect(Float64, ps1d.lr), Matrix{Float64}(ps1d.dl), collect(Float64, ps1d.dhl),
                collect(Float64, ps1d.dhr), Matrix{Float64}(ps1d.V), Matrix{Float64}(ps1d.iV), r))
    s = Space(r[])
    finalizer(x -> ccall((:frgpu_space_destroy, libfrgpu), Cvoid, (Ptr{Cvoid},), x.h), s)
    return s
end

"""Device copy of the operators of a reference FRPSpace2D on uniform rectangles."""
function Space2D(ps2d)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    dx = ps2d.dx[1, 1]
    dy = ps2d.dy[1, 1]
    check(ccall((:frgpu_space_create_2d_ops, libfrgpu), Cint,
                (Cint, Cint, Cint, Cdouble, Cdouble, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble},
                 Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ref{Ptr{Cvoid}}),
                ps2d.nx, ps2d.ny, ps2d.deg, dx, dy, collect(Float64, ps2d.ll), collect(Float64, ps2d.lr),
                Matrix{Float64}(ps2d.dl), collect(Float64, ps2d.dhl), collect(Float64, ps2d.dhr),
                Matrix{Float64}(ps2d.V), Matrix{Float64}(ps2d.iV), r))
    s = Space(r[])
    finalizer(x -> ccall((:frgpu_space_destroy, libfrgpu), Cvoid, (Ptr{Cvoid},), x.h), s)
    return s
end

mutable struct Problem
    h::Ptr{Cvoid}
    space::Space
    dims::Tuple
end

function Problem(space::Space, d::ProblemDesc, dims)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:frgpu_problem_create, libfrgpu), Cint, (Ptr{Cvoid}, Ref{ProblemDesc}, Ref{Ptr{Cvoid}}),
                space.h, d, r))
    p = Problem(r[], space, dims)
    finalizer(x -> ccall((:frgpu_problem_destroy, libfrgpu), Cvoid, (Ptr{Cvoid},), x.h), p)
    return p
end

desc(eq, flux, prec, bcs; a=1.0, γ=1.4, τ=1.0, fixed=zeros(16)) = ProblemDesc(eq, flux, prec, bcs,
    NTuple{16,Cdouble}(fixed), a, γ, τ, 0, C_NULL, C_NULL, 1e-8, 1e-6)

"""rhs!(du, u, p, t) on the GPU: frgpu_rhs (one host->device and one device->host copy)."""
function rhs!(du, u, p::Problem, t)
    uh = Array{Float64}(u)
    dh = similar(uh)
    check(ccall((:frgpu_rhs, libfrgpu), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Cdouble),
                p.h, dh, uh, t))
    du .= dh
    return nothing
end

"""FRAdvectionProblem(u, tspan, ps, a, bc) of src/Equation/eq_advection.jl:1-26."""
function FRAdvectionProblem(u::AbstractMatrix, tspan, ps, a, bc::Symbol; precision=:fp64)
    p = Problem(Space(ps), desc(ADVECTION, FLUX[:roe], PRECISION[precision], ntuple(_ -> BC[bc], 4); a=a), size(u))
    return ODEProblem(rhs!, Array{Float64}(u), tspan, p)
end

"""FREulerProblem(u, tspan, ps, γ, bc) of src/Equation/eq_euler.jl:1-27 (HLL flux)."""
function FREulerProblem(u::AbstractArray{<:Real,3}, tspan, ps, γ, bc::Symbol; precision=:fp64)
    p = Problem(Space(ps), desc(EULER1D, FLUX[:hll], PRECISION[precision], ntuple(_ -> BC[bc], 4); γ=γ), size(u))
    return ODEProblem(rhs!, Array{Float64}(u), tspan, p)
end

"""The `dudt!` of example/shock-vortex.jl:26-118 on the interior u[1:nx, 1:ny, :, :, :];
`bc` = (left, right, bottom, top) kinds, `fixed` the 4x4 conserved ghost states."""
function FREuler2DProblem(u::AbstractArray{<:Real,5}, tspan, ps, γ; flux=:hll, bc=(:period, :period, :period, :period),
                          fixed=zeros(16), precision=:fp64, ghosts_per_step=false)
    bcs = ntuple(i -> BC[bc[i]], 4)
    p = Problem(Space2D(ps), desc(EULER2D, FLUX[flux], PRECISION[precision], bcs; γ=γ, fixed=fixed), size(u))
    # ghosts_per_step: the periodic and copy ghosts keep the step's start values
    # through the step, as the scripts refresh their ghost layers once per step
    if ghosts_per_step
        check(ccall((:frgpu_problem_set_option, libfrgpu), Cint, (Ptr{Cvoid}, Cint, Cint), p.h, 5, 1))
    end
    return ODEProblem(rhs!, Array{Float64}(u), tspan, p)
end

"""The `mol!` closure of example/bgk_wave.jl:69-129 (1D1V BGK, kinetic upwind flux,
relaxation time τ) on the reference's FRPSpace1D and velocity grid `velo`/`weights`;
`f[i, v, k]` is the reference's layout.  `precision=:fp32k` runs the transport on the
tensor cores.  `closure=:density` takes the Maxwellian of example/advection_kinetic.jl:73-128,
prim = [ρ, a, 1] from the density alone."""
function FRBGKProblem(f::AbstractArray{<:Real,3}, tspan, ps, velo, weights, τ; precision=:fp64,
                      closure=:conserve_prim, a=1.0)
    v = collect(Float64, velo)
    w = collect(Float64, weights)
    d = ProblemDesc(BGK1D, FLUX[:upwind], PRECISION[precision], ntuple(_ -> BC[:period], 4),
                    NTuple{16,Cdouble}(zeros(16)), a, 3.0, τ, length(v), pointer(v), pointer(w), 1e-8, 1e-6)
    p = GC.@preserve v w Problem(Space(ps), d, size(f))
    if closure === :density
        check(ccall((:frgpu_problem_set_option, libfrgpu), Cint, (Ptr{Cvoid}, Cint, Cint), p.h, 4, 1))
    end
    return ODEProblem(rhs!, Array{Float64}(f), tspan, p)
end

const INDICATOR = Dict(:none => Cint(0), :plain => Cint(1), :mlp => Cint(2))

"""The post-step troubled-cell indicator + `modal_filter!(û, λ; filter=:l2)` loop of
example/shock-vortex.jl:308-321 (2D) / example/euler_highlevel.jl:37-52 (1D), run inside
every `step!` from now on (`indicator = :none` switches it off)."""
function set_filter!(itg, indicator::Symbol, λ, S0, κ)
    check(ccall((:frgpu_set_filter, libfrgpu), Cint, (Ptr{Cvoid}, Cint, Cdouble, Cdouble, Cdouble),
                itg.p.h, INDICATOR[indicator], λ, S0, κ))
    return nothing
end

"""Apply the indicator + :l2 modal filter once to the integrator's state; returns the
number of troubled elements."""
function modal_filter!(itg, indicator::Symbol, λ, S0, κ)
    n = Ref{Cint}(0)
    check(ccall((:frgpu_modal_filter, libfrgpu), Cint, (Ptr{Cvoid}, Cint, Cdouble, Cdouble, Cdouble, Ref{Cint}),
                itg.p.h, INDICATOR[indicator], λ, S0, κ, n))
    return Int(n[])
end

"""`positive_limiter(ũ, γ, weights, ll, lr, t0)` of src/dissipation.jl:38-216 on every
element of the integrator's state at once (the loop of example/shock-vortex.jl:298-303);
`weights` as the reference takes them (`ps.wp ./ 4` in 2D), or `nothing` for the space's
Gauss weights so normalised.  Returns the number of elements scaled."""
function positive_limiter!(itg, weights=nothing, t0=1.0)
    n = Ref{Cint}(0)
    w = weights === nothing ? C_NULL : Vector{Float64}(vec(weights))
    check(ccall((:frgpu_positive_limiter, libfrgpu), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Cdouble, Ref{Cint}),
                itg.p.h, w, t0, n))
    return Int(n[])
end

"""Run `positive_limiter!` before every `step!` from now on (`on = false` switches it off)."""
function set_limiter!(itg, on::Bool, weights=nothing, t0=1.0)
    w = weights === nothing ? C_NULL : Vector{Float64}(vec(weights))
    check(ccall((:frgpu_set_limiter, libfrgpu), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Cdouble),
                itg.p.h, on ? 1 : 0, w, t0))
    return nothing
end

"""General quadrilaterals: the per-point inverse Jacobian `iJ[i, j][k, l]` of FRPSpace2D
(src/struct.jl:135-158) and, for straight-sided quadrilaterals, the unit face normals
`n1[i, j]` (x faces, (nx+1) x ny) and `n2[i, j]` (y faces, nx x (ny+1)) of
dev/parallelogram.jl:115-160; `iJ = nothing` returns to the rectangles of the space."""
function set_metric!(prob, iJ; n1=nothing, n2=nothing)
    h = prob.p.h
    if iJ === nothing
        check(ccall((:frgpu_problem_set_metric, libfrgpu), Cint,
                    (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}), h, C_NULL, C_NULL, C_NULL))
        return nothing
    end
    nx, ny = size(iJ)
    np = size(iJ[1, 1], 1)
    a = Float64[iJ[i, j][k, l][r, c] for i in 1:nx, j in 1:ny, k in 1:np, l in 1:np, r in 1:2, c in 1:2]
    b1 = n1 === nothing ? C_NULL : Float64[n1[i, j][c] for i in 1:nx+1, j in 1:ny, c in 1:2]
    b2 = n2 === nothing ? C_NULL : Float64[n2[i, j][c] for i in 1:nx, j in 1:ny+1, c in 1:2]
    check(ccall((:frgpu_problem_set_metric, libfrgpu), Cint,
                (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}), h, a, b1, b2))
    return nothing
end

"""interp_face!(fδ, f, ll, lr) of src/interpolate.jl:1-10, evaluated on the GPU."""
"""Dissipation coefficient c of `flux=:central`, the interaction flux of
dev/curve_euler.jl (the script's 40 dt)."""
function set_flux_dissipation!(prob, c)
    check(ccall((:frgpu_problem_set_flux_dissipation, libfrgpu), Cint, (Ptr{Cvoid}, Cdouble), (prob.p::Problem).h, c))
end

function interp_face!(fδ, f::AbstractMatrix, ll, lr)
    fh = Matrix{Float64}(f)
    out = zeros(size(f, 1), 2)
    check(ccall((:frgpu_interp_face, libfrgpu), Cint,
                (Ptr{Cdouble}, Clong, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
                fh, size(f, 1), size(f, 2), collect(Float64, ll), collect(Float64, lr), out))
    fδ .= out
    return nothing
end

struct SSPRK33 end

"""A fixed-step explicit Runge-Kutta method by its Butcher tableau (A strictly lower
triangular, weights b), stepped on the device by `frgpu_step_erk`."""
struct ExplicitRK
    A::Matrix{Float64}
    b::Vector{Float64}
end
Midpoint() = ExplicitRK([0.0 0.0; 0.5 0.0], [0.0, 1.0])     # as example/shock-vortex.jl:294 uses it
Heun() = ExplicitRK([0.0 0.0; 1.0 0.0], [0.5, 0.5])
Ralston() = ExplicitRK([0.0 0.0; 2 / 3 0.0], [0.25, 0.75])
SSPRK22() = ExplicitRK([0.0 0.0; 1.0 0.0], [0.5, 0.5])
RK4() = ExplicitRK([0 0 0 0; 0.5 0 0 0; 0 0.5 0 0; 0 0 1 0], [1 / 6, 1 / 3, 1 / 3, 1 / 6])
"""Tsitouras 5(4) pair (Comput. Math. Appl. 62 (2011) 770-775), fifth-order weights, fixed dt."""
function Tsit5()
    A = zeros(7, 7)
    A[2, 1] = 0.161
    A[3, 1:2] = [-0.008480655492356989, 0.335480655492357]
    A[4, 1:3] = [2.897153057105493, -6.359448489975075, 4.3622954328695815]
    A[5, 1:4] = [5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525]
    A[6, 1:5] = [5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383]
    A[7, 1:6] = [0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081,
                 2.324710524099774]
    return ExplicitRK(A, [A[7, 1:6]; 0.0])
end

"""A ROCK2/ROCK4-type method stepped by `frgpu_step_rock`: before every step the
spectral radius ρ of the residual's Jacobian is estimated on the device
(`frgpu_spectral_radius`) and `select(dt * ρ)` returns `(μ, κ, A, b)`: the recurrence
Y₁ = u + dt μ₁ f(u), Yⱼ = dt μⱼ f(Yⱼ₋₁) + (1 + κⱼ) Yⱼ₋₁ - κⱼ Yⱼ₋₂ and the finishing
tableau of the chosen degree.  For ROCK4 (example/advection_kinetic.jl:133-146) `select`
reads OrdinaryDiffEq's ROCK4 tables (the recurrence coefficients and finishing
procedure of the degree it chooses for dt ρ)."""
struct ROCK
    select::Function
    maxiter::Int
end
ROCK(select) = ROCK(select, 50)

"""The built-in stabilised method: second-order Runge-Kutta-Chebyshev with damping
`eps`, its stage count chosen from the device's spectral-radius estimate before every
step, all inside `frgpu_step_rkc2` (one call per `step!(itg, n)`)."""
struct RKC2
    eps::Float64
    smax::Int
    maxiter::Int
end
RKC2(; eps=2 / 13, smax=4096, maxiter=50) = RKC2(eps, smax, maxiter)

mutable struct Integrator
    p::Problem
    t::Float64
    dt::Float64
    alg::Union{Nothing,ExplicitRK,ROCK,RKC2}
end

"""init(prob, SSPRK33(); dt) or init(prob, Midpoint(); dt): upload u0 once; the state
stays on the device."""
function init(prob::ODEProblem, alg::Union{SSPRK33,ExplicitRK,ROCK,RKC2}; dt, adaptive=false, kwargs...)
    adaptive && error("FRGPU integrates with fixed dt")
    p = prob.p::Problem
    check(ccall((:frgpu_state_upload, libfrgpu), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), p.h, Array{Float64}(prob.u0)))
    return Integrator(p, prob.tspan[1], dt, alg isa SSPRK33 ? nothing : alg)
end

function rock_step!(itg::Integrator, a::ROCK)
    ρ = Ref{Cdouble}(0)
    iters = Ref{Cint}(0)
    check(ccall((:frgpu_spectral_radius, libfrgpu), Cint, (Ptr{Cvoid}, Cint, Ref{Cdouble}, Ref{Cint}),
                itg.p.h, a.maxiter, ρ, iters))
    μ, κ, A, b = a.select(itg.dt * ρ[])
    m = length(μ)
    α = [0.0; 1.0 .+ κ[2:end]]
    β = [0.0; -κ[2:end]]
    δ = zeros(m)
    Ar = Matrix{Float64}(permutedims(A))   # row-major for the C ABI
    check(ccall((:frgpu_step_rock, libfrgpu), Cint,
                (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Cint, Ptr{Cdouble},
                 Ptr{Cdouble}, Cdouble, Cint),
                itg.p.h, m, α, β, collect(Float64, μ), δ, length(b), Ar, collect(Float64, b), itg.dt, 1))
end

"""step!(itg): one SSPRK3 step on the device (a captured CUDA graph)."""
function step!(itg::Integrator, n::Integer=1)
    a = getfield(itg, :alg)
    if a === nothing
        check(ccall((:frgpu_step_ssprk3, libfrgpu), Cint, (Ptr{Cvoid}, Cdouble, Cint), itg.p.h, itg.dt, n))
    elseif a isa ROCK
        for _ in 1:n
            rock_step!(itg, a)
        end
    elseif a isa RKC2
        check(ccall((:frgpu_step_rkc2, libfrgpu), Cint, (Ptr{Cvoid}, Cdouble, Cint, Cdouble, Cint, Cint, Ptr{Cint}),
                    itg.p.h, itg.dt, n, a.eps, a.smax, a.maxiter, C_NULL))
    else
        A = Matrix{Float64}(permutedims(a.A))   # row-major for the C ABI
        check(ccall((:frgpu_step_erk, libfrgpu), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Cdouble, Cint),
                    itg.p.h, length(a.b), A, a.b, itg.dt, n))
    end
    itg.t += n * itg.dt
    return nothing
end

function Base.getproperty(itg::Integrator, s::Symbol)
    if s === :u
        p = getfield(itg, :p)
        out = zeros(p.dims)
        check(ccall((:frgpu_state_download, libfrgpu), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), p.h, out))
        return out
    end
    return getfield(itg, s)
end

# ---------------------------------------------------------------- triangles
"""The linear-advection `dudt!` of dev/wave_triangle.jl:44-125 on the reference's
`TriFRPSpace` `ps` (src/struct.jl:305-352), held on the GPU: `u[ncell, np]`, speed `a`.
`ps.fpn[i, j, k] = (cell, face, point)` becomes 0-based neighbour tables (cell <= 0:
boundary face); only cells with `ps.base.cellType == 0` are updated, as the script does."""
mutable struct TriProblem
    h::Ptr{Cvoid}
    dims::Tuple{Int,Int}
end

function TriProblem(u::AbstractMatrix, ps, a; precision=:fp64)
    ncell, np, m = size(ps.base.cellid, 1), ps.np, ps.deg + 1
    J = Float64[ps.J[i][r, c] for i in 1:ncell, r in 1:2, c in 1:2]
    iJ = Float64[inv(ps.J[i])[r, c] for i in 1:ncell, r in 1:2, c in 1:2]
    nbc = Cint[ps.fpn[i, f, k][1] > 0 ? ps.fpn[i, f, k][1] - 1 : -1 for i in 1:ncell, f in 1:3, k in 1:m]
    nbf = Cint[ps.fpn[i, f, k][1] > 0 ? ps.fpn[i, f, k][2] - 1 : -1 for i in 1:ncell, f in 1:3, k in 1:m]
    nbk = Cint[ps.fpn[i, f, k][1] > 0 ? ps.fpn[i, f, k][3] - 1 : -1 for i in 1:ncell, f in 1:3, k in 1:m]
    ct = Cint.(ps.base.cellType)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:frgpu_tri_create, libfrgpu), Cint,
                (Cint, Cint, Cint, Cdouble, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble},
                 Ptr{Cint}, Ptr{Cint}, Ptr{Cint}, Ptr{Cint}, Ref{Ptr{Cvoid}}),
                ncell, ps.deg, PRECISION[precision], a, Array{Float64}(ps.∂l), Array{Float64}(ps.lf),
                Array{Float64}(ps.ϕ), J, iJ, nbc, nbf, nbk, ct, r))
    t = TriProblem(r[], (ncell, np))
    finalizer(x -> ccall((:frgpu_tri_destroy, libfrgpu), Cint, (Ptr{Cvoid},), x.h), t)
    check(ccall((:frgpu_tri_set_state, libfrgpu), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), t.h, Array{Float64}(u)))
    return t
end

"""dudt!(du, u, p, t) of dev/wave_triangle.jl on the GPU."""
function rhs!(du, u, p::TriProblem, t)
    dh = zeros(p.dims)
    check(ccall((:frgpu_tri_rhs, libfrgpu), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}),
                p.h, dh, Array{Float64}(u)))
    du .= dh
    return nothing
end

"""`n` fixed steps of `alg` (an `ExplicitRK` tableau, e.g. `Euler()`; `SSPRK33()`) on the state."""
function step!(p::TriProblem, alg, dt, n::Integer=1)
    A, b = alg isa SSPRK33 ? ([0.0 0 0; 1 0 0; 0.25 0.25 0], [1 / 6, 1 / 6, 2 / 3]) : (alg.A, alg.b)
    check(ccall((:frgpu_tri_step_erk, libfrgpu), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Cdouble, Cint),
                p.h, length(b), Matrix{Float64}(permutedims(A)), Vector{Float64}(b), dt, n))
    return nothing
end

"""OrdinaryDiffEq `Euler()` as dev/wave_triangle.jl:133 steps it."""
Euler() = ExplicitRK(zeros(1, 1), [1.0])

function state(p::TriProblem)
    out = zeros(p.dims)
    check(ccall((:frgpu_tri_get_state, libfrgpu), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), p.h, out))
    return out
end

end # module
