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
    sol = solve(LinearProblem(A, b), GB300RFLUFactorization())
    sol = solve(LinearProblem(A, b), GB300MixedLUFactorization(factor = :bf16))
    sol = solve(LinearProblem(A, b), GB300MixedLUFactorization(refine = :gmres_ir))
    xs  = gb300_batched_solve(As, bs)                 # thousands of small systems
    srv = GB300Server(precision = :fp32); submit!(srv, key, A, b, x, tag); poll(srv)

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

export GB300LUFactorization, GB300RFLUFactorization, GB300MixedLUFactorization,
    gb300_batched_solve, GB300Server, submit!, poll

const GBLU_OK = Int32(0)
const GBLU_FP64 = Int32(0)
const GBLU_FP32 = Int32(1)
const GBLU_BF16 = Int32(2)
const GBLU_FP16 = Int32(3)
const GBLU_HOST = Int32(0)
const GBLU_REFINE_IR = Int32(0)
const GBLU_REFINE_GMRES = Int32(1)
const GBLU_SOLVE_EXACT = Int32(0)
const GBLU_SOLVE_FAST = Int32(1)
const GBLU_PIVOT_PARTIAL = Int32(0)
const GBLU_PIVOT_TOURNAMENT = Int32(1)
const GBLU_PIVOT_RBT = Int32(2)

const libgblu_path = Ref{String}(get(ENV, "GBLU_LIBRARY",
    joinpath(@__DIR__, "..", "libgblu.so")))
const _handle = Ref{Ptr{Cvoid}}(C_NULL)
const _syms = Dict{Symbol, Ptr{Cvoid}}()

function __init__()
    _handle[] = Libdl.dlopen(libgblu_path[])
    for s in (:gblu_create, :gblu_destroy, :gblu_last_error, :gblu_factor_create,
              :gblu_factor_destroy, :gblu_getrf, :gblu_getrs, :gblu_solve_refined,
              :gblu_refine_opts_default, :gblu_get_ipiv, :gblu_factor_keep_matrix,
              :gblu_factor_set_pivoting,
              :gblu_residual_norm, :gblu_batch_create, :gblu_batch_solve, :gblu_batch_destroy,
              :gblu_serve_config_default, :gblu_serve_create, :gblu_serve_submit,
              :gblu_serve_poll, :gblu_serve_destroy)
        _syms[s] = Libdl.dlsym(_handle[], s)
    end
    return nothing
end

# gblu_refine_opts / gblu_refine_stats, field for field
struct RefineOpts
    mode::Int32
    max_iter::Int32
    tol::Float64
    fallback::Int32
    gmres_restart::Int32
    gmres_tol::Float64
    growth_limit::Float64
end

mutable struct RefineStats
    iterations::Int32
    inner_iterations::Int32
    converged::Int32
    fell_back::Int32
    backward_error::Float64
    growth::Float64
    fallback_reason::Int32
    pad_::Int32
end
RefineStats() = RefineStats(0, 0, 0, 0, 0.0, 0.0, 0, 0)

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
`residualsafety = true` runs the reference's a-posteriori residual check
(src/factorization.jl:127-156) after each refactorization, on the device.
"""
struct GB300LUFactorization <: LinearSolve.AbstractDenseFactorization
    residualsafety::Bool
end
GB300LUFactorization(; residualsafety::Bool = false) = GB300LUFactorization(residualsafety)

"""
    GB300RFLUFactorization(; pivot = Val(true), thread = Val(true), residualsafety = false)

The drop-in for `RFLUFactorization` (src/extension_algs.jl:524-537): the same
recursive partial-pivot FP64 LU and substitution, on the GPU.  `thread` is
accepted and ignored; `pivot = Val(false)` (RecursiveFactorization's pivot-free
`lu!`) is not provided.
"""
struct GB300RFLUFactorization{P, T} <: LinearSolve.AbstractDenseFactorization
    residualsafety::Bool
    function GB300RFLUFactorization(::Val{P}, ::Val{T}; residualsafety::Bool = false) where {P, T}
        P || error("GB300RFLUFactorization: pivot = Val(false) is not provided (partial pivoting only)")
        return new{P, T}(residualsafety)
    end
end
GB300RFLUFactorization(; pivot = Val(true), thread = Val(true), residualsafety::Bool = false) =
    GB300RFLUFactorization(pivot, thread; residualsafety)

"""
    GB300MixedLUFactorization(; factor = :fp32, refine = :ir, maxiters = 30, tol = 0.0,
                              fallback = true, growth_limit = 0.0, residualsafety = false,
                              pivot = :partial)

LU in low precision on the GPU with FP64 iterative refinement (`:ir`) or
GMRES-IR (`:gmres_ir`).  `factor = :fp32` keeps the trailing updates in FP32;
`:bf16` / `:fp16` run them on the tensor cores with 16-bit operands.  The
solution meets the FP64 backward-error bound: refinement that stalls, or
factors whose pivot growth exceeds `growth_limit` (0: the library's default),
fall back to the FP64 LU.  `pivot = :rbt` factors U^T A V / 4 (random
butterflies over the leading n - n mod 4 rows and columns) without pivoting; `:tournament` uses
tournament pivoting for tall leaves; `:partial` (default) is the reference's.
"""
struct GB300MixedLUFactorization <: LinearSolve.AbstractDenseFactorization
    factor::Symbol
    refine::Symbol
    maxiters::Int
    tol::Float64
    fallback::Bool
    growth_limit::Float64
    residualsafety::Bool
    pivot::Symbol
end
function GB300MixedLUFactorization(; factor::Symbol = :fp32, refine::Symbol = :ir,
        maxiters::Integer = 30, tol::Real = 0.0, fallback::Bool = true,
        growth_limit::Real = 0.0, residualsafety::Bool = false, pivot::Symbol = :partial)
    factor in (:fp32, :bf16, :fp16) || error("factor must be :fp32, :bf16 or :fp16")
    refine in (:ir, :gmres_ir) || error("refine must be :ir or :gmres_ir")
    pivot in (:partial, :tournament, :rbt) || error("pivot must be :partial, :tournament or :rbt")
    return GB300MixedLUFactorization(factor, refine, Int(maxiters), Float64(tol), fallback,
                                     Float64(growth_limit), residualsafety, pivot)
end
_pivot_mode(a::GB300MixedLUFactorization) =
    a.pivot === :rbt ? GBLU_PIVOT_RBT : a.pivot === :tournament ? GBLU_PIVOT_TOURNAMENT : GBLU_PIVOT_PARTIAL

const GB300Algs = Union{GB300LUFactorization, GB300RFLUFactorization, GB300MixedLUFactorization}

LinearSolve.needs_concrete_A(::GB300Algs) = true
LinearSolve.default_alias_A(::GB300Algs, ::Any, ::Any) = false
LinearSolve.default_alias_b(::GB300Algs, ::Any, ::Any) = false

_precision(::Union{GB300LUFactorization, GB300RFLUFactorization}) = GBLU_FP64
_precision(a::GB300MixedLUFactorization) =
    a.factor === :bf16 ? GBLU_BF16 : a.factor === :fp16 ? GBLU_FP16 : GBLU_FP32

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

# RFLUFactorization's cacheval is (LU, ipiv) (src/factorization.jl:232-255);
# the GB300 cache unpacks the same way, ipiv read back from the device.
function Base.iterate(c::GB300LUCache, state = 1)
    state == 1 && return (c, 2)
    if state == 2
        ipiv = Vector{Int64}(undef, min(c.m, c.n))
        _check(ccall(_syms[:gblu_get_ipiv], Int32, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}),
                     c.ctx, c.factor, ipiv), c.ctx)
        return (ipiv, 3)
    end
    return nothing
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
    if alg.residualsafety  # the FP64 copy of A the residual check reads
        _check(ccall(_syms[:gblu_factor_keep_matrix], Int32, (Ptr{Cvoid}, Ptr{Cvoid}, Int32),
                     ctx, c.factor, Int32(1)), ctx)
    end
    if alg isa GB300MixedLUFactorization && alg.pivot !== :partial
        _check(ccall(_syms[:gblu_factor_set_pivoting], Int32, (Ptr{Cvoid}, Ptr{Cvoid}, Int32),
                     ctx, c.factor, _pivot_mode(alg)), ctx)
    end
    return c
end

function SciMLBase.solve!(cache::LinearCache, alg::GB300Algs; kwargs...)
    A = convert(AbstractMatrix{Float64}, cache.A)
    c = cache.cacheval
    check_safety = alg.residualsafety && cache.isfresh
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
    if check_safety
        # _check_residual_safety (src/factorization.jl:127-156) on the device
        res, bnorm = _residual_norm(c, cache.u, cache.b)
        tol = cache.abstol + cache.reltol * bnorm
        if res > tol
            @SciMLMessage(cache.verbose, :residual_safety) do
                return "Residual safety check failed: ‖A*x - b‖ = $(res), tol = $(tol)"
            end
            return SciMLBase.build_linear_solution(alg, cache.u, nothing, cache;
                                                   retcode = ReturnCode.APosterioriSafetyFailure)
        end
    end
    return SciMLBase.build_linear_solution(alg, cache.u, nothing, cache; retcode = ReturnCode.Success)
end

function _residual_norm(c::GB300LUCache, u::VecOrMat{Float64}, b::VecOrMat{Float64})
    nrhs = u isa AbstractVector ? 1 : size(u, 2)
    res, bn = Ref{Float64}(0.0), Ref{Float64}(0.0)
    _check(ccall(_syms[:gblu_residual_norm], Int32,
                 (Ptr{Cvoid}, Ptr{Cvoid}, UInt8, Int64, Ptr{Float64}, Int64, Ptr{Float64}, Int64,
                  Int32, Ref{Float64}, Ref{Float64}),
                 c.ctx, c.factor, UInt8('N'), nrhs, u, max(1, size(u, 1)), b, max(1, size(b, 1)),
                 GBLU_HOST, res, bn), c.ctx)
    return res[], bn[]
end

# u := op(A) \ u with the cached device factors (op = 'N' or 'T').
function _solve_in_place!(alg::GB300Algs, c::GB300LUCache, u::VecOrMat{Float64}, trans::Char)
    nrhs = u isa AbstractVector ? 1 : size(u, 2)
    if alg isa GB300MixedLUFactorization
        opts = RefineOpts(alg.refine === :gmres_ir ? GBLU_REFINE_GMRES : GBLU_REFINE_IR,
                          Int32(alg.maxiters), alg.tol, Int32(alg.fallback), Int32(30), 1e-10,
                          alg.growth_limit)
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

# ---------------------------------------------------------------------------
# Batched uneven LU beside LinearProblem (one A per problem there): what a
# caller would otherwise loop as solve(LinearProblem(A_i, b_i), LUFactorization()).

"""
    gb300_batched_solve(As, bs; precision = :fp64) -> (xs, info)

Solves the independent square systems `As[i] * x = bs[i]` (1 <= n_i <= 256, one
right-hand side each) in one graph-captured launch (`gblu_batch_*`).
`precision = :fp32` factors in FP32 and refines each system in FP64.
"""
function gb300_batched_solve(As::AbstractVector{<:AbstractMatrix{Float64}},
        bs::AbstractVector{<:AbstractVector{Float64}}; precision::Symbol = :fp64)
    ctx = default_context()
    sizes = Int64[size(A, 1) for A in As]
    all(size(A, 1) == size(A, 2) for A in As) || error("square systems only")
    Apack = reduce(vcat, (vec(Matrix{Float64}(A)) for A in As); init = Float64[])
    Bpack = reduce(vcat, (Vector{Float64}(b) for b in bs); init = Float64[])
    h = Ref{Ptr{Cvoid}}(C_NULL)
    _check(ccall(_syms[:gblu_batch_create], Int32, (Ptr{Cvoid}, Int64, Ptr{Int64}, Int32, Ref{Ptr{Cvoid}}),
                 ctx, length(sizes), sizes, precision === :fp32 ? GBLU_FP32 : GBLU_FP64, h), ctx)
    info = zeros(Int64, length(sizes))
    try
        _check(ccall(_syms[:gblu_batch_solve], Int32,
                     (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int32, Ptr{Int64}),
                     ctx, h[], Apack, Bpack, GBLU_HOST, info), ctx)
    finally
        ccall(_syms[:gblu_batch_destroy], Int32, (Ptr{Cvoid}, Ptr{Cvoid}), ctx, h[])
    end
    offs = cumsum(vcat(0, sizes[1:end-1]))
    return [Bpack[o + 1:o + n] for (o, n) in zip(offs, sizes)], info
end

# ---------------------------------------------------------------------------
# Serving loop: continuous batching over factorizations resident in HBM.

struct ServeConfig  # gblu_serve_config, field for field
    workers::Int32
    precision::Int32
    refine_mode::Int32
    hbm_budget_bytes::UInt64
    max_rhs_batch::Int32
    small_n::Int32
    solve_mode::Int32
    max_small_batch::Int32
    large_n::Int32
    max_large::Int32
    pivoting::Int32
end

struct Request
    key::UInt64
    n::Int64
    A::Ptr{Float64}
    b::Ptr{Float64}
    x::Ptr{Float64}
    tag::UInt64
end

struct Completion
    tag::UInt64
    status::Int32
    refactored::Int32
    fell_back::Int32
    iterations::Int32
    info::Int64
    backward_error::Float64
    latency_us::Float64
    queue_us::Float64
end

"""
    GB300Server(; workers = 4, precision = :fp32, refine = :ir, hbm_budget_bytes = 0, max_rhs_batch = 8,
                  small_n = -1, solve = :fast, max_large = -1, pivot = :partial)

A `gblu_serve_*` server: `submit!(srv, key, A, b, x, tag)` (A = nothing: solve
with the resident factors of `key`), `poll(srv)` returns the completions.
The arrays of a request must stay alive until its completion is polled.
"""
mutable struct GB300Server
    handle::Ptr{Cvoid}
    live::Dict{UInt64, Any}  # keeps each request's arrays alive until completion
end

function GB300Server(; workers::Integer = 4, precision::Symbol = :fp32, refine::Symbol = :ir,
        hbm_budget_bytes::Integer = 0, max_rhs_batch::Integer = 8, small_n::Integer = -1,
        solve::Symbol = :fast, max_large::Integer = -1, pivot::Symbol = :partial)
    ctx = default_context()
    prec = precision === :fp64 ? GBLU_FP64 : precision === :bf16 ? GBLU_BF16 :
           precision === :fp16 ? GBLU_FP16 : GBLU_FP32
    d = Ref{ServeConfig}()  # the library's defaults for the fields not given here
    _check(ccall(_syms[:gblu_serve_config_default], Int32, (Ref{ServeConfig},), d), ctx)
    c = d[]
    cfg = ServeConfig(Int32(workers), prec, refine === :gmres_ir ? GBLU_REFINE_GMRES : GBLU_REFINE_IR,
                      UInt64(hbm_budget_bytes), Int32(max_rhs_batch),
                      small_n < 0 ? c.small_n : Int32(small_n),
                      solve === :exact ? GBLU_SOLVE_EXACT : GBLU_SOLVE_FAST, c.max_small_batch,
                      c.large_n, max_large < 0 ? c.max_large : Int32(max_large),
                      pivot === :rbt ? GBLU_PIVOT_RBT : pivot === :tournament ? GBLU_PIVOT_TOURNAMENT :
                      GBLU_PIVOT_PARTIAL)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    _check(ccall(_syms[:gblu_serve_create], Int32, (Ptr{Cvoid}, Ref{ServeConfig}, Ref{Ptr{Cvoid}}),
                 ctx, cfg, h), ctx)
    srv = GB300Server(h[], Dict{UInt64, Any}())
    finalizer(s -> (s.handle != C_NULL && ccall(_syms[:gblu_serve_destroy], Int32, (Ptr{Cvoid},), s.handle);
                    s.handle = C_NULL), srv)
    return srv
end

function submit!(srv::GB300Server, key::Integer, A::Union{Nothing, Matrix{Float64}},
        b::Vector{Float64}, x::Vector{Float64}, tag::Integer)
    srv.live[UInt64(tag)] = (A, b, x)
    req = Request(UInt64(key), length(b), A === nothing ? Ptr{Float64}(C_NULL) : pointer(A),
                  pointer(b), pointer(x), UInt64(tag))
    st = ccall(_syms[:gblu_serve_submit], Int32, (Ptr{Cvoid}, Ref{Request}), srv.handle, req)
    st == GBLU_OK || (delete!(srv.live, UInt64(tag)); error("gblu_serve_submit: status $st"))
    return nothing
end

function poll(srv::GB300Server; max::Integer = 64, wait_ms::Integer = 0)
    out = Vector{Completion}(undef, max)
    n = Ref{Int32}(0)
    st = ccall(_syms[:gblu_serve_poll], Int32, (Ptr{Cvoid}, Ptr{Completion}, Int32, Ref{Int32}, Int32),
               srv.handle, out, Int32(max), n, Int32(wait_ms))
    st == GBLU_OK || error("gblu_serve_poll: status $st")
    done = out[1:n[]]
    for c in done
        delete!(srv.live, c.tag)
    end
    return done
end

end # module
