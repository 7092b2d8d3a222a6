"""
    WhaleGPU

Whale.jl's amalgamated reconciliation likelihood on one GB300: `logpdf(model,
ccds)` (src/core.jl:58-64) and its gradient, evaluated by libwhalegpu's
hand-written sm_103a kernels through the library's C ABI
(include/whalegpu.h).  Whale.jl keeps its own types; this module adds methods
for a device-resident copy of the families:

    using Whale, WhaleGPU
    data = WhaleGPU.GPUData(ccds, wm)      # families packed and uploaded once
    logpdf(wm, data)                       # == logpdf(wm, ccds)
    loglikelihood(wm, data)                # what Turing's `data ~ wm` calls

Gradients, for the drivers in the reference's docs and tests:

* ForwardDiff (Turing's default AD, test/mle.jl:11-18): `logpdf` of a model
  whose rates are `ForwardDiff.Dual`s evaluates the value and the gradient
  on the rates struct once on the device (hand-written adjoint) and returns a
  Dual whose partials are that gradient contracted with the partials of
  λ, μ, q and η.  One device evaluation per call, whatever the chunk size.
* ChainRulesCore (Zygote/ReverseDiff-style drivers): an `rrule` for
  `logpdf(::WhaleModel{Float64}, ::GPUData)` whose pullback returns the
  tangent of the model's `rates` field (DLWGD: λ and μ on their log scale,
  q, η; ConstantDLWGD: λ, μ, q, η), and an `rrule` for `(m::WhaleModel)(θ)`
  (src/model.jl:147) that hands that tangent back to the NamedTuple θ of
  `model((λ=…, μ=…, q=…, η=…))` (docs/lit/wgd-turing.jl:38-45).

The leaf sampling probabilities `p` are treated as constants (no gradient),
as the reference's drivers do.  The library path is `ENV["WHALEGPU_LIB"]`
(default: `libwhalegpu` on the loader path), fixed when this module is
loaded.  Calls are synchronous; one context per device is shared by all
Julia tasks of the process and a lock serialises evaluations on it.
"""
module WhaleGPU

using Whale
using NewickTree
using Distributions
using ChainRulesCore
using ForwardDiff

import Distributions: logpdf, loglikelihood

export GPUData

const LIB = get(ENV, "WHALEGPU_LIB", "libwhalegpu")

# constants of include/whalegpu.h
const WG_OK = Cint(0)
const WG_BATCH_GRAD = UInt32(1)
const NODE_LEAF, NODE_INTERNAL, NODE_WGD, NODE_ROOT = Int32(0), Int32(1), Int32(2), Int32(3)
const COND_NONE, COND_ROOT, COND_NONEXTINCT, COND_NOWHERE = Int32(0), Int32(1), Int32(2), Int32(3)

struct WhaleGPUError <: Exception
    code::Cint
    msg::String
end
Base.showerror(io::IO, e::WhaleGPUError) = print(io, "libwhalegpu error ", e.code, ": ", e.msg)

function check(rc::Cint)
    rc == WG_OK && return nothing
    throw(WhaleGPUError(rc, unsafe_string(ccall((:wg_last_error, LIB), Cstring, ()))))
end

# ---- context: one CUDA device and stream (wg_ctx_create) -------------------
const CTXS = Dict{Int,Ptr{Cvoid}}()
const LOCK = ReentrantLock()

function context(device::Integer=0)
    lock(LOCK) do
        get!(CTXS, Int(device)) do
            h = Ref{Ptr{Cvoid}}(C_NULL)
            check(ccall((:wg_ctx_create, LIB), Cint, (Cint, Ref{Ptr{Cvoid}}), device, h))
            h[]
        end
    end
end

# ---- model structure (WhaleModel, src/model.jl:96-145) ----------------------
condition_code(::Whale.RootCondition) = COND_ROOT
condition_code(::Whale.NonExtinctCondition) = COND_NONEXTINCT
condition_code(::Whale.NowhereExtinctCondition) = COND_NOWHERE
condition_code(::Whale.NoCondition) = COND_NONE

"""
    GPUModel(wm)

The structure of `wm` in the library (wg_model_create): nodes in `wm.order`
(leaves first, then postorder, the root last), their kinds and children as
order positions, slice counts and widths (`Slices`, src/model.jl:16-22), the
MUL leaf probabilities, each node's species set (`n.data.clade`, the species
ids the CCDs use) and the sampling condition.  Valid for every model with the
same structure, i.e. every `wm(θ)`.
"""
mutable struct GPUModel
    h::Ptr{Cvoid}
    K::Int
    function GPUModel(wm::WhaleModel)
        order = wm.order
        K = length(order)
        pos = Dict(id(n) => Int32(k - 1) for (k, n) in enumerate(order))
        kind = Int32[Whale.iswgd(n) ? NODE_WGD : isroot(n) ? NODE_ROOT : isleaf(n) ? NODE_LEAF : NODE_INTERNAL
                     for n in order]
        ch = [children(n) for n in order]
        c0 = Int32[isempty(c) ? Int32(-1) : pos[id(c[1])] for c in ch]
        c1 = Int32[length(c) < 2 ? Int32(-1) : pos[id(c[2])] for c in ch]
        nrow = Int32[length(n) for n in order]
        slen = Float64[length(n) > 1 ? Float64(ForwardDiff.value(n[2, 1])) : 0.0 for n in order]
        leafp = Float64[n.data.leafℙ for n in order]
        off = Int32[0]
        sp = Int32[]
        for n in order
            append!(sp, sort!(Int32.(collect(n.data.clade))))
            push!(off, Int32(length(sp)))
        end
        h = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:wg_model_create, LIB), Cint,
                    (Int32, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32},
                     Ptr{Int32}, Int32, Ref{Ptr{Cvoid}}),
                    K, kind, c0, c1, nrow, slen, leafp, off, sp, condition_code(wm.condition), h))
        g = new(h[], K)
        finalizer(x -> ccall((:wg_model_destroy, LIB), Cint, (Ptr{Cvoid},), x.h), g)
    end
end

# ---- families ---------------------------------------------------------------
"""
    ccd_handle(x::CCD)

The library's copy of one CCD (wg_ccd_create) from Whale.jl's own `CCD`
(src/ccd.jl:80-121): clades in the CCD's order (by size, leaves first, the
ubiquitous clade last), each with its number of leaves, species set and
split triples (γ1, γ2, p) with 0-based clade ids.
"""
function ccd_handle(x::Whale.CCD)
    cl = x.clades
    nleaves = Int32[length(c.leaves) for c in cl]
    spo, sp = Int32[0], Int32[]
    so, g1, g2, pp = Int32[0], Int32[], Int32[], Float64[]
    for c in cl
        append!(sp, sort!(Int32.(collect(c.species))))
        push!(spo, Int32(length(sp)))
        for t in c.splits
            push!(g1, Int32(t.γ1 - 1))
            push!(g2, Int32(t.γ2 - 1))
            push!(pp, t.p)
        end
        push!(so, Int32(length(g1)))
    end
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:wg_ccd_create, LIB), Cint,
                (Int32, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}, Ptr{Float64}, Int64,
                 Ref{Ptr{Cvoid}}),
                length(cl), nleaves, spo, sp, so, g1, g2, pp, x.total, h))
    h[]
end

"""
    GPUData(ccds, wm; device=0)

`ccds` packed for `wm`'s structure and resident on the device
(wg_batch_create with WG_BATCH_GRAD): the argument `logpdf` takes in place of
the `Vector{CCD}`.  The per-call table allocation of the reference
(src/core.jl:41) has no counterpart: tables live in the batch.
"""
mutable struct GPUData{C<:Whale.CCD}
    ccds::Vector{C}
    model::GPUModel
    ccdh::Vector{Ptr{Cvoid}}
    h::Ptr{Cvoid}
    ctx::Ptr{Cvoid}
    n::Int
end

function GPUData(ccds::Vector{C}, wm::WhaleModel; device::Integer=0) where {C<:Whale.CCD}
    ctx = context(device)
    g = GPUModel(wm)
    hs = Ptr{Cvoid}[ccd_handle(x) for x in ccds]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:wg_batch_create, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Int32, UInt32, Ref{Ptr{Cvoid}}),
                ctx, g.h, hs, length(hs), WG_BATCH_GRAD, h))
    d = GPUData{C}(ccds, g, hs, h[], ctx, length(ccds))
    finalizer(d) do x  # the batch refers to its CCDs: it goes first
        ccall((:wg_batch_destroy, LIB), Cint, (Ptr{Cvoid},), x.h)
        for c in x.ccdh
            ccall((:wg_ccd_destroy, LIB), Cint, (Ptr{Cvoid},), c)
        end
    end
    d
end

Base.length(d::GPUData) = d.n

# ---- rates (getθ, src/rmodels.jl:14, :31-33, :55-64) -----------------------
"""
    node_rates(wm)

Per-node natural-scale λ, μ (NaN where getθ gives NaN: the root under
DLWGD), q (NaN except at WGD nodes), η and the leaf sampling probabilities
p, in `wm.order`, as primal Float64 values.
"""
function node_rates(wm::WhaleModel)
    r = wm.rates
    K = length(wm.order)
    lam, mu = fill(NaN, K), fill(NaN, K)
    q, p = fill(NaN, K), zeros(K)
    for (k, n) in enumerate(wm.order)
        θ = Whale.getθ(r, n)
        lam[k] = Float64(ForwardDiff.value(θ.λ))
        mu[k] = Float64(ForwardDiff.value(θ.μ))
        Whale.iswgd(n) && (q[k] = Float64(ForwardDiff.value(θ.q)))
        haskey(θ, :p) && (p[k] = Float64(ForwardDiff.value(θ.p)))
    end
    lam, mu, q, Float64(ForwardDiff.value(r.η)), p
end

# wg_model_set_rates: the library fills the slice tables as setmodel! does
function set_rates!(d::GPUData, wm::WhaleModel)
    lam, mu, q, η, p = node_rates(wm)
    check(ccall((:wg_model_set_rates, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Float64, Ptr{Float64}),
                d.model.h, lam, mu, q, η, p))
    lam, mu
end

# ---- evaluation -------------------------------------------------------------
function value(wm::WhaleModel, d::GPUData)
    lock(LOCK) do
        set_rates!(d, wm)
        tot = Ref{Float64}()
        check(ccall((:wg_logpdf, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ref{Float64}),
                    d.ctx, d.model.h, d.h, C_NULL, tot))
        tot[]
    end
end

# log L and the gradient on the per-node natural rates (wg_logpdf_grad)
function value_and_node_gradient(wm::WhaleModel, d::GPUData)
    lock(LOCK) do
        lam, mu = set_rates!(d, wm)
        K = d.model.K
        tot, dη = Ref{Float64}(), Ref{Float64}()
        dl, dm, dq = zeros(K), zeros(K), zeros(K)
        check(ccall((:wg_logpdf_grad, LIB), Cint,
                    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ref{Float64}, Ptr{Float64}, Ptr{Float64},
                     Ptr{Float64}, Ref{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                    d.ctx, d.model.h, d.h, C_NULL, tot, dl, dm, dq, dη, C_NULL, C_NULL, C_NULL))
        tot[], (lam, mu, dl, dm, dq, dη[])
    end
end

"""
    rates_gradient(wm, lam, mu, dl, dm, dq, dη)

The gradient on the fields of `wm.rates` from the per-node natural-rate
adjoints (the chain through getθ): DLWGD λ and μ are log rates indexed by
node id, a WGD node's rates are its non-WGD child's, q is indexed by WGD
ordinal; ConstantDLWGD λ and μ collect every node's adjoint.
"""
function rates_gradient(wm::WhaleModel, lam, mu, dl, dm, dq, dη)
    r = wm.rates
    gq = zeros(length(r.q))
    for (k, n) in enumerate(wm.order)
        Whale.iswgd(n) && (gq[Whale.wgdid(n)] += dq[k])
    end
    if r isa ConstantDLWGD
        ok = .!isnan.(lam)
        return (λ=sum(dl[ok]), μ=sum(dm[ok]), q=gq, η=dη)
    end
    gλ, gμ = zeros(length(r.λ)), zeros(length(r.μ))
    for (k, n) in enumerate(wm.order)
        isnan(lam[k]) && continue
        tgt = Whale.iswgd(n) ? id(Whale.nonwgdchild(n)) : id(n)
        gλ[tgt] += dl[k] * lam[k]  # λ = exp(log λ)
        gμ[tgt] += dm[k] * mu[k]
    end
    (λ=gλ, μ=gμ, q=gq, η=dη)
end

"""
    logpdf(wm::WhaleModel{Float64}, d::GPUData)

Σ_i log L_i − N·condition, non-finite mapped to −Inf (src/core.jl:15,
:58-64), on the device.
"""
logpdf(wm::WhaleModel{Float64}, d::GPUData) = value(wm, d)
loglikelihood(wm::WhaleModel, d::GPUData) = logpdf(wm, d)

# ForwardDiff: the value and the rates gradient from one device evaluation,
# contracted with the partials of the rates the Duals carry
_partials(x::ForwardDiff.Dual, z) = ForwardDiff.partials(x)
_partials(x::Real, z) = z

function logpdf(wm::WhaleModel{D}, d::GPUData) where {Tg,V,N,D<:ForwardDiff.Dual{Tg,V,N}}
    v, (lam, mu, dl, dm, dq, dη) = value_and_node_gradient(wm, d)
    g = rates_gradient(wm, lam, mu, dl, dm, dq, dη)
    r = wm.rates
    z = zero(ForwardDiff.Partials{N,V})
    acc = g.η * _partials(r.η, z)
    if r isa ConstantDLWGD
        acc += g.λ * _partials(r.λ, z) + g.μ * _partials(r.μ, z)
    else
        for i in eachindex(r.λ)
            acc += g.λ[i] * _partials(r.λ[i], z)
        end
        for i in eachindex(r.μ)
            acc += g.μ[i] * _partials(r.μ[i], z)
        end
    end
    for i in eachindex(r.q)
        acc += g.q[i] * _partials(r.q[i], z)
    end
    ForwardDiff.Dual{Tg}(V(v), acc)
end

# ChainRulesCore: the pullback gives the tangent of the model's rates field
function ChainRulesCore.rrule(::typeof(logpdf), wm::WhaleModel{Float64}, d::GPUData)
    v, (lam, mu, dl, dm, dq, dη) = value_and_node_gradient(wm, d)
    g = rates_gradient(wm, lam, mu, dl, dm, dq, dη)
    function logpdf_pullback(Δ)
        δ = unthunk(Δ)
        dr = Tangent{typeof(wm.rates)}(; λ=δ .* g.λ, μ=δ .* g.μ, q=δ .* g.q, η=δ * g.η)
        (NoTangent(), Tangent{typeof(wm)}(; rates=dr), NoTangent())
    end
    v, logpdf_pullback
end

function ChainRulesCore.rrule(::typeof(loglikelihood), wm::WhaleModel{Float64}, d::GPUData)
    v, pb = ChainRulesCore.rrule(logpdf, wm, d)
    v, pb
end

# (m::WhaleModel)(θ) re-parameterises the same structure (src/model.jl:147,
# src/rmodels.jl:8-11): the rates' tangent goes back to θ field by field
function ChainRulesCore.rrule(m::WhaleModel, θ::NamedTuple)
    y = m(θ)
    function model_pullback(Δ)
        δ = unthunk(Δ)
        δ isa AbstractZero && return (NoTangent(), δ)
        δr = δ.rates
        δr isa AbstractZero && return (NoTangent(), δr)
        dθ = Tangent{typeof(θ)}(; (k => getproperty(δr, k) for k in keys(θ))...)
        (NoTangent(), dθ)
    end
    y, model_pullback
end

end # module
