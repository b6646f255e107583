# SSEGB300.jl -- the GB300 drop-in for StableSpectralElements.jl.
#
# Include this file inside the reference's `Solvers` module (after the
# definitions of Solver, ReferenceOperators, FluxDifferencingOperators and the
# mass solvers, src/Solvers/Solvers.jl:66-272) and export `GB300`.  Then
#
#     semidiscretize(law, sd, ic, form, tspan, ReferenceOperator(),
#                    DefaultOperatorAlgorithm(); parallelism = GB300())
#
# builds the usual Solver, hands its operators, geometry, mass solver and
# connectivity to libsse_gb300.so once (`sse_create`, a deep copy onto the
# GPU), and every call of the ODE right-hand side becomes one `sse_residual`.
# The plugin seam is the Parallelism type parameter of Solver
# (Solvers.jl:259-272); nothing else in the reference changes.
#
# Every array is passed by pointer in the reference's own column-major
# layout; the only repacking is of Vector{Diagonal} fields into matrices and
# of LinearMaps into SparseMatrixCSC, once, at set-up.

using LinearAlgebra, SparseArrays
import ChainRulesCore

const libsse = get(ENV, "SSE_GB300_LIB",
                   joinpath(@__DIR__, "..", "cloud.jl_gb300", "_build", "libsse_gb300.so"))

# ---- enums of include/sse_gb300.h ------------------------------------------
const SSE_OK = Int32(0)
const SSE_STANDARD_FORM = Int32(0);     const SSE_FLUX_DIFFERENCING_FORM = Int32(1)
const SSE_LINEAR_ADVECTION = Int32(0);  const SSE_EULER = Int32(1)
const SSE_LAX_FRIEDRICHS = Int32(0);    const SSE_CENTRAL = Int32(1)
const SSE_ENTROPY_CONSERVATIVE = Int32(2)
const SSE_CONSERVATIVE_FLUX = Int32(0); const SSE_EC_FLUX = Int32(1)
const SSE_WEIGHT_ADJUSTED = Int32(0);   const SSE_DIAGONAL = Int32(1)
const SSE_FP64 = Int32(0);              const SSE_MIXED = Int32(1)
const SSE_HOST = Int32(0);              const SSE_DEVICE = Int32(1)
const SSE_CARPENTER_KENNEDY_2N54 = Int32(0); const SSE_RK4 = Int32(1)

# ---- C structs of include/sse_gb300.h: same field order and types -----------
struct SseConfig
    d::Int32
    n_p::Int32
    n_q::Int32
    n_f::Int32
    n_c::Int32
    n_e::Int32
    num_faces::Int32
    nodes_per_face::Int32
    form::Int32
    law::Int32
    numerical_flux::Int32
    two_point_flux::Int32
    mass_solver::Int32
    reserved::Int32
    half_lambda::Float64
    gamma::Float64
    a::NTuple{3, Float64}
end

struct SseCsc
    m::Int64
    n::Int64
    colptr::Ptr{Int64}
    rowval::Ptr{Int64}
    nzval::Ptr{Float64}
end

struct SseOperators
    vdm_p::Int32
    vdm_m::NTuple{3, Int32}
    vdm_A::Ptr{Float64}
    vdm_B::Ptr{Float64}
    vdm_C::Ptr{Float64}
    vdm_sigma_in::Ptr{Int64}
    R::SseCsc
    D::NTuple{3, SseCsc}
    S::NTuple{3, SseCsc}
    C::SseCsc
    V_dense::Ptr{Float64}
end

struct SseGeometry
    BJf::Ptr{Float64}
    n_f::Ptr{Float64}
    mapP::Ptr{Int64}
    halfWLambda::Ptr{Float64}
    WJ::Ptr{Float64}
    Lambda_q::Ptr{Float64}
    halfnJf::Ptr{Float64}
    halfnJq::Ptr{Float64}
    JinvW::Ptr{Float64}
    WJinv::Ptr{Float64}
end

struct SseMetricOperators
    d::Int32
    metrics::Int32
    n_map::Int32
    n_q::Int32
    n_f::Int32
    num_faces::Int32
    n_curl::Int32
    project_jacobian::Int32
    Drst::NTuple{3, Ptr{Float64}}
    Vq::Ptr{Float64}
    Vf::Ptr{Float64}
    nrstJ::NTuple{3, Ptr{Float64}}
    N_to_Nplus1::Ptr{Float64}
    Drst_Nplus1::NTuple{3, Ptr{Float64}}
    Vq_Nplus1::Ptr{Float64}
    Vf_Nplus1::Ptr{Float64}
    project::Ptr{Float64}
end

struct SseGeometricFactorsOut
    J_q::Ptr{Float64}
    Lambda_q::Ptr{Float64}
    J_f::Ptr{Float64}
    nJf::Ptr{Float64}
    nJq::Ptr{Float64}
end

const SSE_NULL_CSC = SseCsc(0, 0, C_NULL, C_NULL, C_NULL)

# ---- the parallelism tag ----------------------------------------------------
"""
    GB300(; precision = :fp64)

Parallelism tag of a Solver whose residual runs on one GB300 through
libsse_gb300.so.  `precision = :mixed` selects the FP32/FP64 mixed form
(FluxDifferencingForm, Euler, entropy-conservative flux).
"""
struct GB300 <: AbstractParallelism
    handle::Base.RefValue{Ptr{Cvoid}}
    precision::Symbol
    keep::Vector{Any}   # host arrays packed at set-up (sse_create copies them)
end
GB300(; precision::Symbol = :fp64) = GB300(Ref(C_NULL), precision, Any[])

sse_error(h) = unsafe_string(ccall((:sse_last_error, libsse), Cstring, (Ptr{Cvoid},), h))

function sse_check(st, h)
    st == SSE_OK || error("libsse_gb300 status $st: " *
                          (h == C_NULL ?
                           unsafe_string(ccall((:sse_create_error, libsse), Cstring, ())) :
                           sse_error(h)))
    return nothing
end

# ---- packing of the reference's fields ----------------------------------------
# A LinearMap or matrix as the SparseMatrixCSC{Float64,Int64} the library reads.
csc_of(A) = SparseMatrixCSC{Float64, Int64}(sparse(Matrix(A)))
function sse_csc(A::SparseMatrixCSC{Float64, Int64}, keep)
    push!(keep, A)
    return SseCsc(size(A, 1), size(A, 2), pointer(A.colptr), pointer(A.rowval), pointer(A.nzval))
end
# Vector{Diagonal} (one per element) -> N x N_e matrix
diag_columns(v) = reduce(hcat, (x.diag for x in v))
ptr(keep, a) = (push!(keep, a); pointer(a))

law_code(::LinearAdvectionEquation) = SSE_LINEAR_ADVECTION
law_code(::EulerEquations) = SSE_EULER
nflux_code(::LaxFriedrichsNumericalFlux) = SSE_LAX_FRIEDRICHS
nflux_code(::CentralNumericalFlux) = SSE_CENTRAL
nflux_code(::EntropyConservativeNumericalFlux) = SSE_ENTROPY_CONSERVATIVE
half_lambda(f::LaxFriedrichsNumericalFlux) = f.halfλ
half_lambda(_) = 0.0
two_point_code(::ConservativeFlux) = SSE_CONSERVATIVE_FLUX
two_point_code(::EntropyConservativeFlux) = SSE_EC_FLUX
gamma_of(law::EulerEquations) = law.γ
gamma_of(_) = 1.4
advection_of(law::LinearAdvectionEquation{d}) where {d} = ntuple(m -> m <= d ? law.a[m] : 0.0, 3)
advection_of(_) = (0.0, 0.0, 0.0)

# V: the warped tensor-product factors, nothing for the identity (nodal
# bases), or the dense matrix of a multidimensional modal basis
function vdm_fields(V::WarpedTensorProductMap2D, keep)
    A, B, σ = Matrix{Float64}(V.A), Array{Float64}(V.B), Array{Int64}(V.σᵢ)
    return (Int32(size(A, 2) - 1), (Int32(size(A, 1)), Int32(size(B, 1)), Int32(0)),
            ptr(keep, A), ptr(keep, B), Ptr{Float64}(C_NULL), ptr(keep, σ), Ptr{Float64}(C_NULL))
end
function vdm_fields(V::WarpedTensorProductMap3D, keep)
    A, B, C, σ = Matrix{Float64}(V.A), Array{Float64}(V.B), Array{Float64}(V.C), Array{Int64}(V.σᵢ)
    return (Int32(size(A, 2) - 1), (Int32(size(A, 1)), Int32(size(B, 1)), Int32(size(C, 1))),
            ptr(keep, A), ptr(keep, B), ptr(keep, C), ptr(keep, σ), Ptr{Float64}(C_NULL))
end
vdm_fields(::LinearMaps.UniformScalingMap, keep) =
    (Int32(0), (Int32(0), Int32(0), Int32(0)), Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL),
     Ptr{Float64}(C_NULL), Ptr{Int64}(C_NULL), Ptr{Float64}(C_NULL))
function vdm_fields(V::LinearMaps.LinearMap, keep)   # OctavianMap / GenericMatrixMap (ModalMulti)
    Vd = Matrix{Float64}(Matrix(V))
    return (Int32(0), (Int32(0), Int32(0), Int32(0)), Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL),
            Ptr{Float64}(C_NULL), Ptr{Int64}(C_NULL), ptr(keep, Vd))
end

function sse_operators(ops::FluxDifferencingOperators, d, keep)
    p, m, A, B, C, σ, Vd = vdm_fields(ops.V, keep)
    S = ntuple(i -> i <= d ? sse_csc(csc_of(ops.S[i]), keep) : SSE_NULL_CSC, 3)
    return SseOperators(p, m, A, B, C, σ, sse_csc(csc_of(ops.R), keep),
                        (SSE_NULL_CSC, SSE_NULL_CSC, SSE_NULL_CSC), S,
                        sse_csc(csc_of(ops.C), keep), Vd)
end

function sse_operators(ops::ReferenceOperators, d, keep)
    p, m, A, B, C, σ, Vd = vdm_fields(ops.V, keep)
    D = ntuple(i -> i <= d ? sse_csc(csc_of(ops.D[i]), keep) : SSE_NULL_CSC, 3)
    return SseOperators(p, m, A, B, C, σ, sse_csc(csc_of(ops.R), keep), D,
                        (SSE_NULL_CSC, SSE_NULL_CSC, SSE_NULL_CSC), SSE_NULL_CSC, Vd)
end

mass_code(::WeightAdjustedSolver) = SSE_WEIGHT_ADJUSTED
mass_code(::DiagonalSolver) = SSE_DIAGONAL
mass_fields(m::WeightAdjustedSolver, keep) = (SSE_WEIGHT_ADJUSTED, ptr(keep, diag_columns(m.J⁻¹W)),
                                              Ptr{Float64}(C_NULL))
mass_fields(m::DiagonalSolver, keep) = (SSE_DIAGONAL, Ptr{Float64}(C_NULL), ptr(keep, diag_columns(m.WJ⁻¹)))

function sse_geometry(ops::FluxDifferencingOperators, mass, mapP, keep)
    _, JinvW, WJinv = mass_fields(mass, keep)
    return SseGeometry(ptr(keep, diag_columns(ops.BJf)), ptr(keep, ops.n_f),
                       ptr(keep, Matrix{Int64}(mapP)), Ptr{Float64}(C_NULL),
                       ptr(keep, diag_columns(ops.WJ)), ptr(keep, ops.Λ_q),
                       ptr(keep, ops.halfnJf), ptr(keep, ops.halfnJq), JinvW, WJinv)
end

function sse_geometry(ops::ReferenceOperators, mass, mapP, keep)
    _, JinvW, WJinv = mass_fields(mass, keep)
    d, _, N_e = size(ops.halfWΛ)
    N_q = length(ops.halfWΛ[1, 1, 1].diag)
    halfWΛ = Array{Float64}(undef, N_q, d, d, N_e)   # N_q x d x d x N_e
    for k in 1:N_e, n in 1:d, m in 1:d
        halfWΛ[:, m, n, k] .= ops.halfWΛ[m, n, k].diag
    end
    return SseGeometry(ptr(keep, diag_columns(ops.BJf)), ptr(keep, ops.n_f),
                       ptr(keep, Matrix{Int64}(mapP)), ptr(keep, halfWΛ),
                       Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL), Ptr{Float64}(C_NULL),
                       Ptr{Float64}(C_NULL), JinvW, WJinv)
end

form_fields(f::StandardForm) = (SSE_STANDARD_FORM, SSE_CONSERVATIVE_FLUX)
form_fields(f::FluxDifferencingForm) = (SSE_FLUX_DIFFERENCING_FORM, two_point_code(f.two_point_flux))

# sse_create for a Solver built the usual way; the handle lives in the tag.
function gb300_create!(solver::Solver{<:AbstractConservationLaw{d, FirstOrder, N_c}}) where {d, N_c}
    p = solver.parallelism
    keep = p.keep
    ops = solver.operators
    form_code, tp_code = form_fields(solver.form)
    N_p, _, N_e = size(solver)
    N_q, N_f = size(ops.V, 1), size(ops.R, 1)
    num_faces = d == 2 ? 3 : 4
    nodes_per_face = ops isa FluxDifferencingOperators ? ops.nodes_per_face : N_f ÷ num_faces
    law = solver.conservation_law
    nflux = solver.form.inviscid_numerical_flux
    cfg = SseConfig(d, N_p, N_q, N_f, N_c, N_e, num_faces, nodes_per_face, form_code,
                    law_code(law), nflux_code(nflux), tp_code, mass_code(solver.mass_solver), 0,
                    half_lambda(nflux), gamma_of(law), advection_of(law))
    sops = sse_operators(ops, d, keep)
    sgeo = sse_geometry(ops, solver.mass_solver, solver.connectivity, keep)
    GC.@preserve keep begin
        st = ccall((:sse_create, libsse), Int32,
                   (Ref{SseConfig}, Ref{SseOperators}, Ref{SseGeometry}, Ptr{Ptr{Cvoid}}),
                   cfg, sops, sgeo, p.handle)
        sse_check(st, C_NULL)
    end
    empty!(keep)   # the library holds its own device copies now
    if p.precision == :mixed
        sse_check(ccall((:sse_set_precision, libsse), Int32, (Ptr{Cvoid}, Int32), p.handle[], SSE_MIXED),
                  p.handle[])
    end
    finalizer(r -> (r[] != C_NULL && ccall((:sse_destroy, libsse), Int32, (Ptr{Cvoid},), r[]);
                    r[] = C_NULL), p.handle)
    return solver
end

# ---- the Solver(...) hook: the usual constructor, then the upload -------------
function Solver(conservation_law::AbstractConservationLaw{d, FirstOrder, N_c},
        spatial_discretization::SpatialDiscretization{d},
        form::Union{StandardForm, FluxDifferencingForm},
        strategy::ReferenceOperator,
        alg::AbstractOperatorAlgorithm,
        mass_solver::AbstractMassMatrixSolver,
        parallelism::GB300) where {d, N_c}
    solver = invoke(Solver,
                    Tuple{typeof(conservation_law), typeof(spatial_discretization), typeof(form),
                          ReferenceOperator, typeof(alg), typeof(mass_solver), AbstractParallelism},
                    conservation_law, spatial_discretization, form, strategy, alg, mass_solver,
                    parallelism)
    return gb300_create!(solver)
end

# ---- the drop-in right-hand side (same contract as Solvers.jl:474-514) --------
function semi_discrete_residual!(dudt::AbstractArray{Float64, 3},
        u::AbstractArray{Float64, 3},
        solver::Solver{<:AbstractConservationLaw{<:Any, FirstOrder}, <:Any, <:Any, <:Any, GB300},
        t::Float64 = 0.0)
    h = solver.parallelism.handle[]
    st = ccall((:sse_residual, libsse), Int32,
               (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Float64, Int32),
               h, u, dudt, t, SSE_HOST)
    sse_check(st, h)
    return dudt
end

# ---- the whole fixed-step time loop on the device, and its pullback -----------
"""
    gb300_solve(u0, solver, n_steps, dt; scheme = SSE_CARPENTER_KENNEDY_2N54)

`solve(ode, CarpenterKennedy2N54(); dt, adaptive = false)` over n_steps steps
with every stage on the device (`sse_rk_steps`): returns u(t0 + n_steps dt).
"""
function gb300_solve(u0::Array{Float64, 3}, solver, n_steps::Integer, dt::Float64;
                     scheme::Int32 = SSE_CARPENTER_KENNEDY_2N54)
    h = solver.parallelism.handle[]
    u = copy(u0)
    t = Ref(0.0)
    st = ccall((:sse_rk_steps, libsse), Int32,
               (Ptr{Cvoid}, Ptr{Float64}, Int32, Float64, Int32, Ref{Float64}, Int32),
               h, u, n_steps, dt, scheme, t, SSE_HOST)
    sse_check(st, h)
    return u
end

# The stepper's rrule: the forward records the trajectory (uniform segments
# sized from free device memory, or the binomial schedule with `checkpoints`
# states when that is given), the pullback is sse_rk_adjoint.
function ChainRulesCore.rrule(::typeof(gb300_solve), u0::Array{Float64, 3}, solver,
                              n_steps::Integer, dt::Float64;
                              scheme::Int32 = SSE_CARPENTER_KENNEDY_2N54, checkpoints::Integer = -1)
    h = solver.parallelism.handle[]
    u = copy(u0)
    t = Ref(0.0)
    st = if checkpoints < 0
        ccall((:sse_rk_record, libsse), Int32,
              (Ptr{Cvoid}, Ptr{Float64}, Int32, Float64, Int32, Int32, Ref{Float64}, Int32),
              h, u, n_steps, dt, scheme, 0, t, SSE_HOST)
    else
        ccall((:sse_rk_record_binomial, libsse), Int32,
              (Ptr{Cvoid}, Ptr{Float64}, Int32, Float64, Int32, Int32, Ref{Float64}, Int32),
              h, u, n_steps, dt, scheme, checkpoints, t, SSE_HOST)
    end
    sse_check(st, h)
    function gb300_solve_pullback(ū)
        λT = Array{Float64, 3}(ChainRulesCore.unthunk(ū))
        λ0 = similar(λT)
        st2 = ccall((:sse_rk_adjoint, libsse), Int32,
                    (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int32),
                    h, λT, λ0, C_NULL, SSE_HOST)
        sse_check(st2, h)
        return (ChainRulesCore.NoTangent(), λ0, ChainRulesCore.NoTangent(),
                ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent())
    end
    return u, gb300_solve_pullback
end
