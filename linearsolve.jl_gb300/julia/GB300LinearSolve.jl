"""
    GB300LinearSolve

LinearSolve.jl algorithms backed by libgblu (the GB300 dense LU library, C ABI
in include/gblu.h).  The binding follows the pattern LinearSolve.jl uses for
OpenBLAS (src/openblas.jl): the library is opened and its symbols resolved
once, every call is a `ccall` through a fixed pointer with plain pointers and
sizes, the factorization lives in a mutable cache object reused across
refactorizations, and a singular matrix is a `ReturnCode.Failure`, not an
exception.

    using LinearSolve, GB300LinearSolve
    sol = solve(LinearProblem(A, b), GB300LUFactorization())
    sol = solve(LinearProblem(A, b), GB300MixedLUFactorization(refine = :gmres_ir))

This file is not exercised in this repository's test-suite (no Julia
toolchain here); the Python layer in this package drives the same C ABI and
carries the tests.
"""
module GB300LinearSolve

using LinearAlgebra
using LinearSolve
using LinearSolve: LinearCache, LinearVerbosity, OperatorAssumptions, @SciMLMessage
using SciMLBase
using SciMLBase: ReturnCode
using Libdl

export GB300LUFactorization, GB300MixedLUFactorization

const GBLU_OK = Int32(0)
const GBLU_FP64 = Int32(0)
const GBLU_FP32 = Int32(1)
const GBLU_HOST = Int32(0)
const GBLU_REFINE_IR = Int32(0)
const GBLU_REFINE_GMRES = Int32(1)

const libgblu_path = Ref{String}(get(ENV, "GBLU_LIBRARY",
    joinpath(@__DIR__, "..", "libgblu.so")))
const _handle = Ref{Ptr{Cvoid}}(C_NULL)
const _syms = Dict{Symbol, Ptr{Cvoid}}()

function __init__()
    _handle[] = Libdl.dlopen(libgblu_path[])
    for s in (:gblu_create, :gblu_destroy, :gblu_last_error, :gblu_factor_create,
              :gblu_factor_destroy, :gblu_getrf, :gblu_getrs, :gblu_solve_refined,
              :gblu_refine_opts_default)
        _syms[s] = Libdl.dlsym(_handle[], s)
    end
    return nothing
end

struct RefineOpts
    mode::Int32
    max_iter::Int32
    tol::Float64
    fallback::Int32
    gmres_restart::Int32
    gmres_tol::Float64
end

mutable struct RefineStats
    iterations::Int32
    inner_iterations::Int32
    converged::Int32
    fell_back::Int32
    backward_error::Float64
end
RefineStats() = RefineStats(0, 0, 0, 0, 0.0)

_check(st::Int32, ctx) = st == GBLU_OK || error("libgblu: status $st: " *
    unsafe_string(ccall(_syms[:gblu_last_error], Cstring, (Ptr{Cvoid},), ctx)))

# One context per device, created lazily (the process-wide handle of
# src/openblas.jl:48-72).
const _ctx = Ref{Ptr{Cvoid}}(C_NULL)
function default_context(device::Integer = 0)
    if _ctx[] == C_NULL
        r = Ref{Ptr{Cvoid}}(C_NULL)
        _check(ccall(_syms[:gblu_create], Int32, (Ref{Ptr{Cvoid}}, Int32, UInt64),
                     r, Int32(device), UInt64(0)), C_NULL)
        _ctx[] = r[]
    end
    return _ctx[]
end

"""
    GB300LUFactorization(; residualsafety = false)

Plain FP64 partial-pivot LU on the GPU (getrf + getrs in FP64).  Factors and
pivots are bit-identical to LinearSolve's blocked LU (src/blocked_lufact.jl).
"""
struct GB300LUFactorization <: LinearSolve.AbstractDenseFactorization
    residualsafety::Bool
end
GB300LUFactorization(; residualsafety::Bool = false) = GB300LUFactorization(residualsafety)

"""
    GB300MixedLUFactorization(; refine = :ir, maxiters = 30, tol = 0.0, fallback = true)

FP32 LU on the GPU with FP64 iterative refinement (`:ir`) or GMRES-IR
(`:gmres_ir`); the solution meets the FP64 backward-error bound, falling back
to the FP64 LU when refinement stalls.
"""
struct GB300MixedLUFactorization <: LinearSolve.AbstractDenseFactorization
    refine::Symbol
    maxiters::Int
    tol::Float64
    fallback::Bool
end
GB300MixedLUFactorization(; refine::Symbol = :ir, maxiters::Integer = 30, tol::Real = 0.0,
                          fallback::Bool = true) =
    GB300MixedLUFactorization(refine, Int(maxiters), Float64(tol), fallback)

const GB300Algs = Union{GB300LUFactorization, GB300MixedLUFactorization}

LinearSolve.needs_concrete_A(::GB300Algs) = true
LinearSolve.default_alias_A(::GB300Algs, ::Any, ::Any) = false
LinearSolve.default_alias_b(::GB300Algs, ::Any, ::Any) = false

_precision(::GB300LUFactorization) = GBLU_FP64
_precision(::GB300MixedLUFactorization) = GBLU_FP32

# The cacheval: a device-resident gblu_factor, freed by a finalizer.
mutable struct GB300LUCache
    ctx::Ptr{Cvoid}
    factor::Ptr{Cvoid}
    m::Int
    n::Int
    info::Int64
    stats::RefineStats
end

function _free!(c::GB300LUCache)
    if c.factor != C_NULL
        ccall(_syms[:gblu_factor_destroy], Int32, (Ptr{Cvoid}, Ptr{Cvoid}), c.ctx, c.factor)
        c.factor = C_NULL
    end
end

function LinearSolve.init_cacheval(alg::GB300Algs, A, b, u, Pl, Pr, maxiters::Int, abstol,
        reltol, verbose::Union{LinearVerbosity, Bool}, assumptions::OperatorAssumptions)
    ctx = default_context()
    m, n = size(A)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    _check(ccall(_syms[:gblu_factor_create], Int32,
                 (Ptr{Cvoid}, Int64, Int64, Int32, Ref{Ptr{Cvoid}}),
                 ctx, m, n, _precision(alg), r), ctx)
    c = GB300LUCache(ctx, r[], m, n, 0, RefineStats())
    finalizer(_free!, c)
    return c
end

function SciMLBase.solve!(cache::LinearCache, alg::GB300Algs; kwargs...)
    A = convert(AbstractMatrix{Float64}, cache.A)
    c = cache.cacheval
    if cache.isfresh
        info = Ref{Int64}(0)
        _check(ccall(_syms[:gblu_getrf], Int32,
                     (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Int64, Int32, Ref{Int64}),
                     c.ctx, c.factor, A, max(1, stride(A, 2)), GBLU_HOST, info), c.ctx)
        c.info = info[]
        if info[] != 0
            @SciMLMessage("Solver failed", cache.verbose, :solver_failure)
            return SciMLBase.build_linear_solution(alg, cache.u, nothing, cache;
                                                   retcode = ReturnCode.Failure)
        end
        cache.isfresh = false
    end
    copyto!(cache.u, cache.b)
    _solve_in_place!(alg, c, cache.u, 'N')
    return SciMLBase.build_linear_solution(alg, cache.u, nothing, cache; retcode = ReturnCode.Success)
end

# u := op(A) \ u with the cached device factors (op = 'N' or 'T').
function _solve_in_place!(alg::GB300Algs, c::GB300LUCache, u::VecOrMat{Float64}, trans::Char)
    nrhs = u isa AbstractVector ? 1 : size(u, 2)
    if alg isa GB300MixedLUFactorization
        opts = RefineOpts(alg.refine === :gmres_ir ? GBLU_REFINE_GMRES : GBLU_REFINE_IR,
                          Int32(alg.maxiters), alg.tol, Int32(alg.fallback), Int32(30), 1e-10)
        _check(ccall(_syms[:gblu_solve_refined], Int32,
                     (Ptr{Cvoid}, Ptr{Cvoid}, UInt8, Int64, Ptr{Float64}, Int64, Int32,
                      Ref{RefineOpts}, Ref{RefineStats}),
                     c.ctx, c.factor, UInt8(trans), nrhs, u, max(1, size(u, 1)),
                     GBLU_HOST, opts, c.stats), c.ctx)
    else
        _check(ccall(_syms[:gblu_getrs], Int32,
                     (Ptr{Cvoid}, Ptr{Cvoid}, UInt8, Int64, Ptr{Float64}, Int64, Int32),
                     c.ctx, c.factor, UInt8(trans), nrhs, u, max(1, size(u, 1)), GBLU_HOST), c.ctx)
    end
    return u
end

# solve!(cache; adjoint = true) reuses the device factors (src/adjoint_factorization.jl:
# the algorithm opts into the custom reuse and answers with a transposed getrs).
LinearSolve._adjoint_factorization_reuse(::Type{<:GB300Algs}) =
    LinearSolve._CustomAdjointFactorizationReuse()
LinearSolve._custom_can_reuse_adjoint_factorization(::GB300Algs, c::GB300LUCache) =
    c.factor != C_NULL && c.info == 0
function LinearSolve._custom_adjoint_factorization_solve(alg::GB300Algs, c::GB300LUCache, A, b)
    x = Matrix{Float64}(reshape(b, size(b, 1), :))
    _solve_in_place!(alg, c, x, 'T')
    return b isa AbstractVector ? vec(x) : x
end

end # module
