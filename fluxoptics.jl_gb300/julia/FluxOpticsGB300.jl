"""
    FluxOpticsGB300

Drop-in GB300 components for FluxOptics.jl: each type subtypes the reference's
component hierarchy and implements its method set (propagate!, backpropagate!,
propagate_and_save!, backpropagate_with_gradient!, trainable, ...) through
`ccall` into libfluxoptics_gb300 (include/fluxoptics_gb300.h).  Fields must be
`CuArray{ComplexF32}`; work is ordered on CUDA.jl's task-local stream.

Replaces, for CuArray fields:
- ASProp / RSProp  (src/optical_components/freespace_propagators/angular_spectrum.jl:193-234,
                    rayleigh_sommerfeld.jl:128-169)
- Phase / Mask     (src/optical_components/modulators/phasemask.jl:38-150, mask.jl:39-142)
- AS_BPM           (src/optical_components/bulk_propagators/bpm.jl:130-142, 244-321), with
                   √N-slice checkpoints instead of every slice (GB300AS_BPM)
- a fused run of the above (GB300Chain), the GPU counterpart of the merge rules
  (src/optical_components/system/merge_rules.jl:45-52)
- TeaDOE / TeaReflector, FourierPhase / FourierMask, ASPropZ, DotProduct / PowerCoupling
- SquaredIntensityDifference (src/metrics/squared_intensity_difference.jl:58-90), also
  evaluated inside a chain's last forward pass (forward_with_metric!)
- SquaredFieldDifference (src/metrics/squared_field_difference.jl:35-61), also with the
  forward sweep, the metric and the adjoint sweep in one call (withgradient!)
- Fista, ProxRule(Fista, ClampProx) in one pass, ClampProx, IstaProx, PositiveProx and
  TVProx (src/OptimisersExt.jl:33-54, 222-244; src/proximal_operators/clamp_prox.jl:35-37,
  ista_prox.jl:1-56, positive_prox.jl:1-40, tv_prox.jl:94-195) as in-place device steps (fista_step!, gb300_clamp!, gb300_ista!,
  gb300_positive!, tv_prox!)
- the ragged batch of independent problems in one persistent launch (GB300Ragged)
"""
module FluxOpticsGB300

using CUDA
using Functors
using FluxOptics
using FluxOptics.OpticalComponents: AbstractCustomComponent, Static, Trainable, Buffered, Unbuffered,
                                    Direction, Forward, Backward
import FluxOptics.OpticalComponents: propagate!, backpropagate!, propagate_and_save!,
                                     backpropagate_with_gradient!, get_preallocated_gradient,
                                     get_saved_buffer, alloc_saved_buffer, trainable, get_data

const LIB = joinpath(@__DIR__, "..", "lib", "libfluxoptics_gb300.so")
const FO_FLAG_AUTOTUNE = Cint(1)
const FO_FLAG_GRAD_SPECTRA = Cint(2)
const FO_FLAG_DEVICE_Z = Cint(4)
const FO_MOD_NONE, FO_MOD_PHASE, FO_MOD_MASK, FO_MOD_DN, FO_MOD_TEA = Cint(0), Cint(1), Cint(2), Cint(3), Cint(4)

struct FoMod            # mirrors `fo_mod`
    kind::Cint
    param::Ptr{Cvoid}
    saved::Ptr{Cvoid}
    grad::Ptr{Cvoid}
    scale::Cdouble
    field_coef::Ptr{Cvoid}  # FO_MOD_TEA only
end
FoMod(kind, param, saved, grad, scale) = FoMod(kind, param, saved, grad, scale, C_NULL)

function check(rc::Cint)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:fo_last_error, LIB), Cstring, ()))
    error("libfluxoptics_gb300 error $rc: $msg")
end

cstream() = CUDA.stream().handle
dptr(x::CuArray) = reinterpret(Ptr{Cvoid}, pointer(x))
dptr(::Nothing) = C_NULL
dims_of(u::ScalarField) = (size(u.electric, 1), size(u.electric, 2), div(length(u.electric), size(u.electric, 1) * size(u.electric, 2)))
dirsign(::Type{Forward}) = Cint(1)
dirsign(::Type{Backward}) = Cint(-1)

# one value per field, in the column-major order of the trailing dims: `val` is the
# reference's broadcastable (1, 1, d3, ...) array (Fields.jl:18-38)
per_field(u::ScalarField, val) =
    Float64.(vec(broadcast((l, _) -> l, Array(val), zeros(1, 1, size(u.electric)[3:end]...))))
lambdas_per_field(u::ScalarField) = per_field(u, FluxOptics.get_lambdas(u))
# (theta_x, theta_y) pairs per field, flattened as the C ABI takes them
function tilts_per_field(u::ScalarField)
    tx, ty = FluxOptics.get_tilts(u)
    vec(permutedims(hcat(per_field(u, tx), per_field(u, ty))))
end

# ---------------------------------------------------------------------------
# Propagators
# ---------------------------------------------------------------------------
mutable struct GB300Prop <: AbstractCustomComponent{Static}
    plan::Ptr{Cvoid}
    kind::Symbol
    z::Float64
end

function _finalize(p::GB300Prop)
    p.plan == C_NULL || ccall((:fo_prop_destroy, LIB), Cint, (Ptr{Cvoid},), p.plan)
    p.plan = C_NULL
end

struct FoASOptions          # mirrors `fo_as_options` (no filter callback from Julia here)
    paraxial::Cint
    track_tilts::Cint
    tilts::Ptr{Cdouble}
    n_tilts::Cint
    filter::Ptr{Cvoid}
    filter_ctx::Ptr{Cvoid}
end

"""GB300ASProp(u, z; n0=1, paraxial=false, track_tilts=false) -- angular-spectrum
propagation on the GPU path; tilted fields (u.tilts) select the tilted kernel."""
function GB300ASProp(u::ScalarField, z::Real; n0::Real = 1, paraxial::Bool = false, track_tilts::Bool = false)
    nx, ny, b = dims_of(u)
    lam = lambdas_per_field(u)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    if !paraxial && !track_tilts && FluxOptics.is_on_axis(u)
        check(ccall((:fo_asprop_create, LIB), Cint,
                    (Ref{Ptr{Cvoid}}, Cint, Cint, Cint, Cdouble, Cdouble, Ptr{Cdouble}, Cint, Cdouble, Cdouble, Cint),
                    h, nx, ny, b, u.ds[1], u.ds[2], lam, length(lam), z, n0, FO_FLAG_AUTOTUNE))
    else
        th = tilts_per_field(u)
        GC.@preserve th begin
            opt = Ref(FoASOptions(Cint(paraxial), Cint(track_tilts), pointer(th), Cint(b), C_NULL, C_NULL))
            check(ccall((:fo_asprop_create_ex, LIB), Cint,
                        (Ref{Ptr{Cvoid}}, Cint, Cint, Cint, Cdouble, Cdouble, Ptr{Cdouble}, Cint, Cdouble, Cdouble,
                         Ref{FoASOptions}, Cint),
                        h, nx, ny, b, u.ds[1], u.ds[2], lam, length(lam), z, n0, opt, FO_FLAG_AUTOTUNE))
        end
    end
    finalizer(_finalize, GB300Prop(h[], :AS, Float64(z)))
end

"""GB300RSProp(u, z) -- Rayleigh-Sommerfeld propagation on the GPU path."""
function GB300RSProp(u::ScalarField, z::Real)
    nx, ny, b = dims_of(u)
    lam = lambdas_per_field(u)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:fo_rsprop_create, LIB), Cint,
                (Ref{Ptr{Cvoid}}, Cint, Cint, Cint, Cdouble, Cdouble, Ptr{Cdouble}, Cint, Cdouble, Cint),
                h, nx, ny, b, u.ds[1], u.ds[2], lam, length(lam), z, FO_FLAG_AUTOTUNE))
    finalizer(_finalize, GB300Prop(h[], :RS, Float64(z)))
end

Functors.@functor GB300Prop ()
get_data(p::GB300Prop) = ()

function propagate!(u::ScalarField, p::GB300Prop, dir::Type{<:Direction})
    check(ccall((:fo_propagate, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                p.plan, dptr(u.electric), dirsign(dir), cstream()))
    u
end

backpropagate!(u::ScalarField, p::GB300Prop, dir::Type{<:Direction}) = propagate!(u, p, reverse(dir))

# ---------------------------------------------------------------------------
# Phase
# ---------------------------------------------------------------------------
struct GB300Phase{M, A, U} <: AbstractCustomComponent{M}
    ϕ::A
    ∂p::Union{Nothing, @NamedTuple{ϕ::A}}
    u::Union{Nothing, U}
end

function GB300Phase(p::Phase)   # adopt a reference Phase (same arrays)
    M = FluxOptics.OpticalComponents.get_trainability(p)
    GB300Phase{M, typeof(p.ϕ), typeof(p.u)}(p.ϕ, p.∂p, p.u)
end

Functors.@functor GB300Phase (ϕ,)
get_data(p::GB300Phase) = p.ϕ
trainable(p::GB300Phase{<:Trainable}) = (; ϕ = p.ϕ)
get_preallocated_gradient(p::GB300Phase{Trainable{Buffered}}) = p.∂p
get_saved_buffer(p::GB300Phase{Trainable{Buffered}}) = p.u
alloc_saved_buffer(u::ScalarField, p::GB300Phase{Trainable{Unbuffered}}) = similar(u.electric)

function _phase_fwd!(u::ScalarField, p::GB300Phase, saved, dir)
    nx, ny, b = dims_of(u)
    check(ccall((:fo_phase_forward, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cint, Cint, Ptr{Cvoid}),
                dptr(u.electric), dptr(p.ϕ), dptr(saved), nx, ny, b, dirsign(dir), cstream()))
    u
end

propagate!(u::ScalarField, p::GB300Phase, dir::Type{<:Direction}) = _phase_fwd!(u, p, nothing, dir)
propagate_and_save!(u::ScalarField, p::GB300Phase{Trainable{Buffered}}, dir::Type{<:Direction}) =
    _phase_fwd!(u, p, p.u, dir)
propagate_and_save!(u::ScalarField, u_saved::AbstractArray, p::GB300Phase{Trainable{Unbuffered}},
                    dir::Type{<:Direction}) = _phase_fwd!(u, p, u_saved, dir)
backpropagate!(u::ScalarField, p::GB300Phase, dir::Type{<:Direction}) = _phase_fwd!(u, p, nothing, reverse(dir))

function backpropagate_with_gradient!(∂v::ScalarField, u_saved::AbstractArray, ∂p::NamedTuple,
                                      p::GB300Phase{<:Trainable}, dir::Type{<:Direction})
    nx, ny, b = dims_of(∂v)
    check(ccall((:fo_phase_backward, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cint, Cint, Ptr{Cvoid}),
                dptr(∂v.electric), dptr(p.ϕ), dptr(u_saved), dptr(∂p.ϕ), nx, ny, b, dirsign(dir), cstream()))
    (∂v, ∂p)
end

# ---------------------------------------------------------------------------
# Mask
# ---------------------------------------------------------------------------
struct GB300Mask{M, A, U} <: AbstractCustomComponent{M}
    m::A
    ∂p::Union{Nothing, @NamedTuple{m::A}}
    u::Union{Nothing, U}
end

function GB300Mask(p::Mask)
    M = FluxOptics.OpticalComponents.get_trainability(p)
    GB300Mask{M, typeof(p.m), typeof(p.u)}(p.m, p.∂p, p.u)
end

Functors.@functor GB300Mask (m,)
get_data(p::GB300Mask) = p.m
trainable(p::GB300Mask{<:Trainable}) = (; m = p.m)
get_preallocated_gradient(p::GB300Mask{Trainable{Buffered}}) = p.∂p
get_saved_buffer(p::GB300Mask{Trainable{Buffered}}) = p.u
alloc_saved_buffer(u::ScalarField, p::GB300Mask{Trainable{Unbuffered}}) = similar(u.electric)

function _mask_fwd!(u::ScalarField, p::GB300Mask, saved, dir)
    nx, ny, b = dims_of(u)
    check(ccall((:fo_mask_forward, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cint, Cint, Ptr{Cvoid}),
                dptr(u.electric), dptr(p.m), dptr(saved), nx, ny, b, dirsign(dir), cstream()))
    u
end

propagate!(u::ScalarField, p::GB300Mask, dir::Type{<:Direction}) = _mask_fwd!(u, p, nothing, dir)
propagate_and_save!(u::ScalarField, p::GB300Mask{Trainable{Buffered}}, dir::Type{<:Direction}) =
    _mask_fwd!(u, p, p.u, dir)
propagate_and_save!(u::ScalarField, u_saved::AbstractArray, p::GB300Mask{Trainable{Unbuffered}},
                    dir::Type{<:Direction}) = _mask_fwd!(u, p, u_saved, dir)

function backpropagate_with_gradient!(∂v::ScalarField, u_saved::AbstractArray, ∂p::NamedTuple,
                                      p::GB300Mask{<:Trainable}, dir::Type{<:Direction})
    nx, ny, b = dims_of(∂v)
    check(ccall((:fo_mask_backward, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cint, Cint, Ptr{Cvoid}),
                dptr(∂v.electric), dptr(p.m), dptr(u_saved), dptr(∂p.m), nx, ny, b, dirsign(dir), cstream()))
    (∂v, ∂p)
end

# ---------------------------------------------------------------------------
# Fused chain: [mod] prop [mod] prop ... [mod] on one grid
# ---------------------------------------------------------------------------
mutable struct GB300Chain{M, P, D} <: AbstractCustomComponent{M}
    chain::Ptr{Cvoid}
    props::P                 # GB300Prop, kept alive
    mods::D                  # Tuple of Nothing / GB300Phase / GB300Mask, length(props)+1
end

function GB300Chain(props::Vector{GB300Prop}, mods::Vector)
    @assert length(mods) == length(props) + 1
    h = Ref{Ptr{Cvoid}}(C_NULL)
    plans = [p.plan for p in props]
    check(ccall((:fo_chain_create, LIB), Cint, (Ref{Ptr{Cvoid}}, Cint, Ptr{Ptr{Cvoid}}), h, length(plans), plans))
    M = any(m -> m !== nothing && FluxOptics.istrainable(m), mods) ? Trainable{Buffered} : Static
    c = GB300Chain{M, typeof(Tuple(props)), typeof(Tuple(mods))}(h[], Tuple(props), Tuple(mods))
    finalizer(x -> ccall((:fo_chain_destroy, LIB), Cint, (Ptr{Cvoid},), x.chain), c)
end

Functors.@functor GB300Chain (mods,)
trainable(p::GB300Chain{<:Trainable}) = (; mods = p.mods)

_fomod(::Nothing, saved, grad) = FoMod(FO_MOD_NONE, C_NULL, C_NULL, C_NULL, 0.0)
_fomod(m::GB300Phase, saved, grad) = FoMod(FO_MOD_PHASE, dptr(m.ϕ), dptr(saved), dptr(grad), 1.0)
_fomod(m::GB300Mask, saved, grad) = FoMod(FO_MOD_MASK, dptr(m.m), dptr(saved), dptr(grad), 1.0)
_saved(m) = (m === nothing || !FluxOptics.istrainable(m)) ? nothing : m.u
_grad(m::GB300Phase) = FluxOptics.istrainable(m) ? m.∂p.ϕ : nothing
_grad(m::GB300Mask) = FluxOptics.istrainable(m) ? m.∂p.m : nothing
_grad(::Nothing) = nothing

function propagate!(u::ScalarField, p::GB300Chain, dir::Type{<:Direction})
    mods = [_fomod(m, nothing, nothing) for m in p.mods]
    check(ccall((:fo_chain_forward, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{FoMod}, Cint, Ptr{Cvoid}),
                p.chain, dptr(u.electric), mods, dirsign(dir), cstream()))
    u
end

function propagate_and_save!(u::ScalarField, p::GB300Chain{Trainable{Buffered}}, dir::Type{<:Direction})
    mods = [_fomod(m, _saved(m), nothing) for m in p.mods]
    check(ccall((:fo_chain_forward, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{FoMod}, Cint, Ptr{Cvoid}),
                p.chain, dptr(u.electric), mods, dirsign(dir), cstream()))
    u
end

get_preallocated_gradient(p::GB300Chain{Trainable{Buffered}}) = (; mods = map(m -> m === nothing ? nothing : m.∂p, p.mods))
get_saved_buffer(p::GB300Chain{Trainable{Buffered}}) = map(_saved, p.mods)

function backpropagate_with_gradient!(∂v::ScalarField, u_saved, ∂p::NamedTuple, p::GB300Chain{<:Trainable},
                                      dir::Type{<:Direction})
    mods = [_fomod(m, _saved(m), _grad(m)) for m in p.mods]
    check(ccall((:fo_chain_backward, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{FoMod}, Cint, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                p.chain, dptr(∂v.electric), mods, dirsign(dir), C_NULL, C_NULL, cstream()))
    (∂v, ∂p)
end

backpropagate!(u::ScalarField, p::GB300Chain, dir::Type{<:Direction}) =
    error("GB300Chain: use backpropagate_with_gradient! (the adjoint sweep needs the saved inputs)")

"""
    gb300(system::OpticalSystem) -> OpticalSystem

Replace ASProp/RSProp/Phase/Mask components by their GB300 counterparts and fuse
every maximal run [mod] prop [mod] prop ... [mod] into one GB300Chain.
"""
function gb300(system::OpticalSystem; template::ScalarField)
    comps = FluxOptics.get_components(system)
    out = Any[]
    i = 1
    while i <= length(comps)
        c = comps[i]
        if c isa ASProp || c isa RSProp || c isa Phase || c isa Mask
            mods = Any[nothing]
            props = GB300Prop[]
            if c isa Phase || c isa Mask
                mods[1] = c isa Phase ? GB300Phase(c) : GB300Mask(c)
                i += 1
            end
            while i <= length(comps) && (comps[i] isa ASProp || comps[i] isa RSProp)
                push!(props, _convert_prop(comps[i], template))
                push!(mods, nothing)
                i += 1
                if i <= length(comps) && (comps[i] isa Phase || comps[i] isa Mask)
                    mods[end] = comps[i] isa Phase ? GB300Phase(comps[i]) : GB300Mask(comps[i])
                    i += 1
                end
            end
            isempty(props) ? push!(out, mods[1]) : push!(out, GB300Chain(props, mods))
        else
            push!(out, c)
            i += 1
        end
    end
    OpticalSystem(FluxOptics.get_source(system), out...)
end

# the propagation distance is kept by the wrapped kernel component
_convert_prop(c::ASProp, u) = GB300ASProp(u, c.optical_components[2].z; n0 = c.optical_components[2].n0)
_convert_prop(c::RSProp, u) = GB300RSProp(u, c.optical_components[3].z)

# ---------------------------------------------------------------------------
# TeaDOE / TeaReflector: per-field {2 pi dn(lambda)/lambda, Re r, Im r, 0}
# ---------------------------------------------------------------------------
struct GB300TeaDOE{M, A, C, U} <: AbstractCustomComponent{M}
    h::A
    coef::C                   # CuArray{Float32} of 4 x batch
    ∂p::Union{Nothing, @NamedTuple{h::A}}
    u::Union{Nothing, U}
end

function GB300TeaDOE(p::TeaDOE, u::ScalarField)   # adopt a reference TeaDOE for fields like u
    M = FluxOptics.OpticalComponents.get_trainability(p)
    lam = lambdas_per_field(u)
    c = zeros(Float32, 4, length(lam))
    for (k, l) in enumerate(lam)
        r = ComplexF64(p.r(l))
        c[:, k] .= (2π * p.dn(l) / l, real(r), imag(r), 0)
    end
    cd = CuArray(c)
    GB300TeaDOE{M, typeof(p.h), typeof(cd), typeof(p.u)}(p.h, cd, p.∂p, p.u)
end

Functors.@functor GB300TeaDOE (h,)
get_data(p::GB300TeaDOE) = p.h
trainable(p::GB300TeaDOE{<:Trainable}) = (; h = p.h)
get_preallocated_gradient(p::GB300TeaDOE{Trainable{Buffered}}) = p.∂p
get_saved_buffer(p::GB300TeaDOE{Trainable{Buffered}}) = p.u
alloc_saved_buffer(u::ScalarField, p::GB300TeaDOE{Trainable{Unbuffered}}) = similar(u.electric)

function _tea_fwd!(u::ScalarField, p::GB300TeaDOE, saved, dir)
    nx, ny, b = dims_of(u)
    check(ccall((:fo_tea_forward, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cint, Cint, Ptr{Cvoid}),
                dptr(u.electric), dptr(p.h), dptr(p.coef), dptr(saved), nx, ny, b, dirsign(dir), cstream()))
    u
end

propagate!(u::ScalarField, p::GB300TeaDOE, dir::Type{<:Direction}) = _tea_fwd!(u, p, nothing, dir)
propagate_and_save!(u::ScalarField, p::GB300TeaDOE{Trainable{Buffered}}, dir::Type{<:Direction}) =
    _tea_fwd!(u, p, p.u, dir)
propagate_and_save!(u::ScalarField, u_saved::AbstractArray, p::GB300TeaDOE{Trainable{Unbuffered}},
                    dir::Type{<:Direction}) = _tea_fwd!(u, p, u_saved, dir)

function backpropagate!(∂v::ScalarField, p::GB300TeaDOE, dir::Type{<:Direction})
    nx, ny, b = dims_of(∂v)
    check(ccall((:fo_tea_backward, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cint, Cint, Ptr{Cvoid}),
                dptr(∂v.electric), dptr(p.h), dptr(p.coef), C_NULL, C_NULL, nx, ny, b, dirsign(dir), cstream()))
    ∂v
end

function backpropagate_with_gradient!(∂v::ScalarField, u_saved::AbstractArray, ∂p::NamedTuple,
                                      p::GB300TeaDOE{<:Trainable}, dir::Type{<:Direction})
    nx, ny, b = dims_of(∂v)
    check(ccall((:fo_tea_backward, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cint, Cint, Ptr{Cvoid}),
                dptr(∂v.electric), dptr(p.h), dptr(p.coef), dptr(u_saved), dptr(∂p.h), nx, ny, b, dirsign(dir),
                cstream()))
    (∂v, ∂p)
end

# ---------------------------------------------------------------------------
# FourierPhase / FourierMask: a propagator plan with the Fourier-domain multiplier
# ---------------------------------------------------------------------------
mutable struct GB300Fourier{M, A} <: AbstractCustomComponent{M}
    plan::Ptr{Cvoid}
    kind::Cint                # FO_MOD_PHASE or FO_MOD_MASK
    p::A                      # ϕ or m on the FFT-ordered frequency grid
    ∂p::Union{Nothing, NamedTuple}
end

function GB300Fourier(u::ScalarField, p::AbstractArray, kind::Cint; trainable::Bool = false)
    nx, ny, b = dims_of(u)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:fo_fourier_create, LIB), Cint, (Ref{Ptr{Cvoid}}, Cint, Cint, Cint, Cint),
                h, nx, ny, b, FO_FLAG_AUTOTUNE | (trainable ? Cint(2) : Cint(0))))
    M = trainable ? Trainable{Unbuffered} : Static
    f = GB300Fourier{M, typeof(p)}(h[], kind, p, trainable ? NamedTuple{(:p,)}((similar(p),)) : nothing)
    finalizer(x -> ccall((:fo_prop_destroy, LIB), Cint, (Ptr{Cvoid},), x.plan), f)
end
GB300FourierPhase(u::ScalarField, ϕ; trainable = false) = GB300Fourier(u, ϕ, FO_MOD_PHASE; trainable)
GB300FourierMask(u::ScalarField, m; trainable = false) = GB300Fourier(u, m, FO_MOD_MASK; trainable)

Functors.@functor GB300Fourier (p,)
get_data(f::GB300Fourier) = f.p
trainable(f::GB300Fourier{<:Trainable}) = (; p = f.p)
alloc_saved_buffer(u::ScalarField, f::GB300Fourier{Trainable{Unbuffered}}) = similar(u.electric)

function propagate!(u::ScalarField, f::GB300Fourier, dir::Type{<:Direction})
    check(ccall((:fo_fourier_set, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Cvoid}, Ptr{Cvoid}),
                f.plan, f.kind, dptr(f.p), cstream()))
    check(ccall((:fo_propagate, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                f.plan, dptr(u.electric), dirsign(dir), cstream()))
    u
end
function propagate_and_save!(u::ScalarField, u_saved::AbstractArray, f::GB300Fourier{Trainable{Unbuffered}},
                             dir::Type{<:Direction})
    copyto!(u_saved, u.electric)
    propagate!(u, f, dir)
end
function backpropagate!(∂v::ScalarField, f::GB300Fourier, dir::Type{<:Direction})
    check(ccall((:fo_propagate, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                f.plan, dptr(∂v.electric), -dirsign(dir), cstream()))
    ∂v
end
function backpropagate_with_gradient!(∂v::ScalarField, u_saved::AbstractArray, ∂p::NamedTuple,
                                      f::GB300Fourier{<:Trainable}, dir::Type{<:Direction})
    check(ccall((:fo_fourier_gradient, LIB), Cint,
                (Ptr{Cvoid}, Cint, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                f.plan, f.kind, dptr(f.p), dptr(u_saved), dptr(∂v.electric), dptr(∂p.p), dirsign(dir), cstream()))
    (backpropagate!(∂v, f, dir), ∂p)
end

# ---------------------------------------------------------------------------
# ASPropZ: trainable distance, z in device memory
# ---------------------------------------------------------------------------
mutable struct GB300ASPropZ{M, A} <: AbstractCustomComponent{M}
    plan::Ptr{Cvoid}
    z::A                      # CuArray{Float32}(1)
end

"""GB300ASPropZ(u, z; n0=1, trainable=false, paraxial=false, track_tilts=false) -- ASPropZ
(angular_spectrum.jl:274-344) with the on-axis, tilted (u.tilts) or paraxial kernel; the
transfer functions are rebuilt from the device-resident z on every call."""
function GB300ASPropZ(u::ScalarField, z::Real; n0::Real = 1, trainable::Bool = false, paraxial::Bool = false,
                      track_tilts::Bool = false)
    nx, ny, b = dims_of(u)
    lam = lambdas_per_field(u)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    flags = FO_FLAG_AUTOTUNE | FO_FLAG_DEVICE_Z | (trainable ? FO_FLAG_GRAD_SPECTRA : Cint(0))
    if !paraxial && !track_tilts && FluxOptics.is_on_axis(u)
        check(ccall((:fo_asprop_create, LIB), Cint,
                    (Ref{Ptr{Cvoid}}, Cint, Cint, Cint, Cdouble, Cdouble, Ptr{Cdouble}, Cint, Cdouble, Cdouble, Cint),
                    h, nx, ny, b, u.ds[1], u.ds[2], lam, length(lam), z, n0, flags))
    else
        th = tilts_per_field(u)
        GC.@preserve th begin
            opt = Ref(FoASOptions(Cint(paraxial), Cint(track_tilts), pointer(th), Cint(b), C_NULL, C_NULL))
            check(ccall((:fo_asprop_create_ex, LIB), Cint,
                        (Ref{Ptr{Cvoid}}, Cint, Cint, Cint, Cdouble, Cdouble, Ptr{Cdouble}, Cint, Cdouble, Cdouble,
                         Ref{FoASOptions}, Cint),
                        h, nx, ny, b, u.ds[1], u.ds[2], lam, length(lam), z, n0, opt, flags))
        end
    end
    zd = CuArray(Float32[z])
    M = trainable ? Trainable{Unbuffered} : Static
    p = GB300ASPropZ{M, typeof(zd)}(h[], zd)
    finalizer(x -> ccall((:fo_prop_destroy, LIB), Cint, (Ptr{Cvoid},), x.plan), p)
end

Functors.@functor GB300ASPropZ (z,)
get_data(p::GB300ASPropZ) = p.z
trainable(p::GB300ASPropZ{<:Trainable}) = (; z = p.z)
alloc_saved_buffer(u::ScalarField, p::GB300ASPropZ{Trainable{Unbuffered}}) = similar(u.electric)

function propagate!(u::ScalarField, p::GB300ASPropZ, dir::Type{<:Direction})
    check(ccall((:fo_prop_set_z, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}), p.plan, dptr(p.z), cstream()))
    check(ccall((:fo_propagate, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                p.plan, dptr(u.electric), dirsign(dir), cstream()))
    u
end
function propagate_and_save!(u::ScalarField, u_saved::AbstractArray, p::GB300ASPropZ{Trainable{Unbuffered}},
                             dir::Type{<:Direction})
    copyto!(u_saved, u.electric)
    propagate!(u, p, dir)
end
function backpropagate!(∂v::ScalarField, p::GB300ASPropZ, dir::Type{<:Direction})
    check(ccall((:fo_propagate, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                p.plan, dptr(∂v.electric), -dirsign(dir), cstream()))
    ∂v
end
function backpropagate_with_gradient!(∂v::ScalarField, u_saved::AbstractArray, ∂p::NamedTuple,
                                      p::GB300ASPropZ{<:Trainable}, dir::Type{<:Direction})
    check(ccall((:fo_prop_z_gradient, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}, Ptr{Cvoid}),
                p.plan, dptr(p.z), dptr(u_saved), dptr(∂v.electric), dirsign(dir), dptr(∂p.z), cstream()))
    (backpropagate!(∂v, p, dir), ∂p)
end

# ---------------------------------------------------------------------------
# AS_BPM: split-step march with sqrt(N) checkpoints kept inside the plan
# ---------------------------------------------------------------------------
mutable struct GB300BPM{M, A} <: AbstractCustomComponent{M}
    plan::Ptr{Cvoid}
    dn::A                     # CuArray{Float32, 3}: nx x ny x n_slices (the reference's layout)
    ∂p::Union{Nothing, @NamedTuple{dn::A}}
end

# Token standing for the slice inputs of the last saving forward: the plan keeps
# every checkpoint_every-th slice input itself and recomputes the others in the
# adjoint, so no (nx, ny, batch, n_slices) buffer exists on the Julia side.
struct GB300BPMSaved
    plan::Ptr{Cvoid}
end

"""
    GB300AS_BPM(u, thickness, n0, dn0; paraxial=false, trainable=false, buffered=false, checkpoint_every=0)

AS_BPM (bpm.jl:130-142) on the GPU path: the symmetric split-step march of
`propagate!` (bpm.jl:244-260) and its adjoint with the ∂dn gradient
(bpm.jl:275-321).  Instead of saving every slice input (bpm.jl:49, 2 GiB at
1024² × 256) the plan keeps every `checkpoint_every`-th one (0: round(√n_slices))
and recomputes each segment during the adjoint.  `paraxial` selects Fresnel steps;
fields with tilts take the tilted steps and kdz = 2π dz / (cos θx cos θy) per field
(bpm.jl:3-6).  `dn0` is nx × ny × n_slices.
"""
function GB300AS_BPM(u::ScalarField, thickness::Real, n0::Real, dn0::AbstractArray{<:Real, 3};
                     paraxial::Bool = false, trainable::Bool = false, buffered::Bool = false,
                     checkpoint_every::Integer = 0)
    nx, ny, b = dims_of(u)
    size(dn0, 1) == nx && size(dn0, 2) == ny || error("GB300AS_BPM: dn0 must be nx x ny x n_slices")
    ns = size(dn0, 3)
    ns >= 2 || error("GB300AS_BPM: at least 2 slices")
    lam = lambdas_per_field(u)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    if !paraxial && FluxOptics.is_on_axis(u)
        check(ccall((:fo_bpm_create, LIB), Cint,
                    (Ref{Ptr{Cvoid}}, Cint, Cint, Cint, Cdouble, Cdouble, Ptr{Cdouble}, Cint, Cdouble, Cdouble,
                     Cint, Cint, Cdouble, Cint),
                    h, nx, ny, b, u.ds[1], u.ds[2], lam, length(lam), thickness, n0, ns, checkpoint_every, 1.0,
                    FO_FLAG_AUTOTUNE))
    else
        # tilted steps and kdz = 2π dz / (cos θx cos θy) per field (bpm.jl:3-6)
        th = tilts_per_field(u)
        GC.@preserve th begin
            opt = Ref(FoASOptions(Cint(paraxial), Cint(0), pointer(th), Cint(b), C_NULL, C_NULL))
            check(ccall((:fo_bpm_create_ex, LIB), Cint,
                        (Ref{Ptr{Cvoid}}, Cint, Cint, Cint, Cdouble, Cdouble, Ptr{Cdouble}, Cint, Cdouble, Cdouble,
                         Cint, Cint, Ref{FoASOptions}, Cint),
                        h, nx, ny, b, u.ds[1], u.ds[2], lam, length(lam), thickness, n0, ns, checkpoint_every,
                        opt, FO_FLAG_AUTOTUNE))
        end
    end
    dn = CuArray{Float32}(dn0)
    M = trainable ? (buffered ? Trainable{Buffered} : Trainable{Unbuffered}) : Static
    ∂p = (trainable && buffered) ? (; dn = similar(dn)) : nothing
    p = GB300BPM{M, typeof(dn)}(h[], dn, ∂p)
    finalizer(x -> ccall((:fo_bpm_destroy, LIB), Cint, (Ptr{Cvoid},), x.plan), p)
end

Functors.@functor GB300BPM (dn,)
get_data(p::GB300BPM) = p.dn
trainable(p::GB300BPM{<:Trainable}) = (; dn = p.dn)
get_preallocated_gradient(p::GB300BPM{Trainable{Buffered}}) = p.∂p
get_saved_buffer(p::GB300BPM{Trainable{Buffered}}) = GB300BPMSaved(p.plan)
alloc_saved_buffer(u::ScalarField, p::GB300BPM{Trainable{Unbuffered}}) = GB300BPMSaved(p.plan)

function _bpm_fwd!(u::ScalarField, p::GB300BPM, save::Bool, dir)
    check(ccall((:fo_bpm_forward, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Ptr{Cvoid}),
                p.plan, dptr(u.electric), dptr(p.dn), dirsign(dir), Cint(save), cstream()))
    u
end

propagate!(u::ScalarField, p::GB300BPM, dir::Type{<:Direction}) = _bpm_fwd!(u, p, false, dir)
propagate_and_save!(u::ScalarField, p::GB300BPM{Trainable{Buffered}}, dir::Type{<:Direction}) =
    _bpm_fwd!(u, p, true, dir)
propagate_and_save!(u::ScalarField, ::GB300BPMSaved, p::GB300BPM{Trainable{Unbuffered}},
                    dir::Type{<:Direction}) = _bpm_fwd!(u, p, true, dir)

# the adjoint march without a gradient still needs the saved slice inputs of the plan
backpropagate!(∂v::ScalarField, p::GB300BPM, dir::Type{<:Direction}) =
    error("GB300AS_BPM: use backpropagate_with_gradient! after propagate_and_save!")

function backpropagate_with_gradient!(∂v::ScalarField, ::GB300BPMSaved, ∂p::NamedTuple,
                                      p::GB300BPM{<:Trainable}, dir::Type{<:Direction})
    check(ccall((:fo_bpm_backward, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                p.plan, dptr(∂v.electric), dptr(p.dn), dptr(∂p.dn), dirsign(dir), cstream()))
    (∂v, ∂p)
end

# ---------------------------------------------------------------------------
# SquaredIntensityDifference: the metric, its pullback, and the metric fused
# into a chain's last forward pass
# ---------------------------------------------------------------------------
mutable struct GB300SID{T}
    handle::Ptr{Cvoid}
    target::T                 # CuArray{Float32}: nx x ny x n_targets
    loss::CuArray{Float32, 1}
end

"""
    GB300SquaredIntensityDifference(u, target)

SquaredIntensityDifference (squared_intensity_difference.jl:58-90) for fields
like `u`: I_t = Σ|u_b|² over the fields b of target slice t (field b belongs to
slice b mod n_targets, the broadcast of an nx × ny × T target over
nx × ny × T × M fields), loss_t = Σ(I_t − target_t)².
"""
function GB300SquaredIntensityDifference(u::ScalarField, target::AbstractArray{<:Real})
    nx, ny, b = dims_of(u)
    t = CuArray{Float32}(target)
    nt = div(length(t), nx * ny)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:fo_sid_create, LIB), Cint, (Ref{Ptr{Cvoid}}, Cint, Cint, Cint, Cint, Ptr{Cint}),
                h, nx, ny, b, nt, C_NULL))
    m = GB300SID(h[], t, CUDA.zeros(Float32, nt))
    finalizer(x -> ccall((:fo_sid_destroy, LIB), Cint, (Ptr{Cvoid},), x.handle), m)
end

# compute_metric: per-slice losses (device), residuals kept for the pullback
function (m::GB300SID)(u::ScalarField)
    check(ccall((:fo_sid_forward, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                m.handle, dptr(u.electric), dptr(m.target), dptr(m.loss), cstream()))
    m.loss
end

# backpropagate_metric: ∂u = 4 ∂c_t (I_t − target_t) u (∂c = nothing: all ones)
function pullback!(m::GB300SID, ∂c, u::ScalarField, ∂u::ScalarField)
    check(ccall((:fo_sid_backward, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                m.handle, dptr(u.electric), ∂c === nothing ? C_NULL : dptr(∂c), dptr(∂u.electric), cstream()))
    ∂u
end

"""
    forward_with_metric!(u_out, c::GB300Chain, u_in, m::GB300SID; dir=Forward) -> losses

The chain's saving forward from `u_in` into `u_out` with the metric evaluated
inside the last pass (fo_chain_forward_sid); the device losses are returned and
the residuals stay in `m` for [`backward_from_metric!`](@ref).
"""
function forward_with_metric!(u_out::ScalarField, c::GB300Chain, u_in::ScalarField, m::GB300SID;
                              dir::Type{<:Direction} = Forward)
    mods = [_fomod(x, _saved(x), nothing) for x in c.mods]
    check(ccall((:fo_chain_forward_sid, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{FoMod}, Cint, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid},
                 Ptr{Cvoid}),
                c.chain, dptr(u_in.electric), dptr(u_out.electric), mods, dirsign(dir), m.handle,
                dptr(m.target), dptr(m.loss), cstream()))
    m.loss
end

"""
    backward_from_metric!(∂u, c::GB300Chain, u_out, m::GB300SID; dir=Forward, input_grad=true)

The chain's adjoint sweep seeded with the metric's pullback of the last
[`forward_with_metric!`](@ref): every trainable modulator's gradient buffer is
filled.  With `input_grad = false` the final write of the input gradient is
skipped (FO_BWD_DISCARD_INPUT_GRAD) and `∂u` holds scratch values.
"""
function backward_from_metric!(∂u::ScalarField, c::GB300Chain, u_out::ScalarField, m::GB300SID;
                               dir::Type{<:Direction} = Forward, input_grad::Bool = true)
    mods = [_fomod(x, _saved(x), _grad(x)) for x in c.mods]
    check(ccall((:fo_chain_backward_ex, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{FoMod}, Cint, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                c.chain, dptr(∂u.electric), mods, dirsign(dir), m.handle, dptr(u_out.electric),
                input_grad ? Cint(0) : Cint(1), cstream()))
    ∂u
end

"""
    withgradient!(∂u, c::GB300Chain, u_in, m::GB300SID; u_out=nothing, input_grad=true) -> losses

Zygote.withgradient(metric, system) for a chain ending in a propagator and
SquaredIntensityDifference, in one call (fo_chain_withgradient_sid): the forward
sweep from `u_in`, the metric and the seeded adjoint sweep, whose first row pass is
shared with the forward's last.  Trainable modulators' gradient buffers are filled;
`∂u` ends holding the gradient with respect to `u_in` (scratch with
`input_grad=false`); `u_out` receives the output field when given.
"""
function withgradient!(∂u::ScalarField, c::GB300Chain, u_in::ScalarField, m::GB300SID;
                       u_out = nothing, input_grad::Bool = true, dir::Type{<:Direction} = Forward)
    mf = [_fomod(x, _saved(x), nothing) for x in c.mods]
    mb = [_fomod(x, _saved(x), _grad(x)) for x in c.mods]
    check(ccall((:fo_chain_withgradient_sid, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{FoMod}, Ptr{FoMod}, Cint, Ptr{Cvoid},
                 Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                c.chain, dptr(u_in.electric), u_out === nothing ? C_NULL : dptr(u_out.electric),
                dptr(∂u.electric), mf, mb, dirsign(dir), m.handle, dptr(m.target), dptr(m.loss),
                input_grad ? Cint(0) : Cint(1), cstream()))
    m.loss
end

# ---------------------------------------------------------------------------
# Optimiser steps: Fista (η stored squared, OptimisersExt.jl:33-54), ProxRule(Fista,
# ClampProx) in one pass (OptimisersExt.jl:222-244, clamp_prox.jl:35-37), TVProx
# (tv_prox.jl:94-195).  Each call updates the parameter in place on the stream.
# ---------------------------------------------------------------------------
mutable struct GB300FistaState{A}
    eta::Float64
    xk::A                     # previous iterate
    newdx::A                  # the step of the last update
    t::CuArray{Float64, 1}    # Fista's t, advanced on the device
end

"""GB300FistaState(eta, x) -- the state Fista(eta) keeps for parameter x."""
GB300FistaState(eta::Real, x::CuArray{Float32}) = GB300FistaState(Float64(eta), copy(x), similar(x), CuArray([1.0]))

"""
    fista_step!(st, x, dx; clamp=nothing)

One Fista update of `x` with gradient `dx`; with `clamp = (lo, hi)` the
ClampProx of ProxRule(Fista(eta), ClampProx(lo, hi)) runs in the same pass.
"""
function fista_step!(st::GB300FistaState, x::CuArray{Float32}, dx::CuArray{Float32}; clamp = nothing)
    n = Clonglong(length(x))
    if clamp === nothing
        check(ccall((:fo_fista_step, LIB), Cint,
                    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Clonglong, Cdouble, Ptr{Cvoid}, Ptr{Cvoid}),
                    dptr(x), dptr(st.xk), dptr(st.newdx), dptr(dx), n, st.eta, dptr(st.t), cstream()))
    else
        check(ccall((:fo_fista_clamp_step, LIB), Cint,
                    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Clonglong, Cdouble, Ptr{Cvoid}, Cdouble,
                     Cdouble, Ptr{Cvoid}),
                    dptr(x), dptr(st.xk), dptr(st.newdx), dptr(dx), n, st.eta, dptr(st.t),
                    Float64(clamp[1]), Float64(clamp[2]), cstream()))
    end
    x
end

"""clamp!(x, lo, hi) on the device -- ClampProx (clamp_prox.jl:35-37)."""
function gb300_clamp!(x::CuArray{Float32}, lo::Real, hi::Real)
    check(ccall((:fo_clamp, LIB), Cint, (Ptr{Cvoid}, Clonglong, Cdouble, Cdouble, Ptr{Cvoid}),
                dptr(x), Clonglong(length(x)), lo, hi, cstream()))
    x
end

# IstaProx(s, c) (ista_prox.jl:1-56): soft threshold towards c; a complex array is
# passed as its interleaved real and imaginary parts, each shrunk towards c
function gb300_ista!(x::Union{CuArray{Float32}, CuArray{ComplexF32}}, s::Real, c::Real = 0)
    n = length(x) * (eltype(x) <: Complex ? 2 : 1)
    check(ccall((:fo_ista, LIB), Cint, (Ptr{Cvoid}, Clonglong, Cdouble, Cdouble, Ptr{Cvoid}),
                dptr(x), Clonglong(n), s, c, cstream()))
    x
end

# PositiveProx (positive_prox.jl:1-40): x = max(x, 0)
function gb300_positive!(x::CuArray{Float32})
    check(ccall((:fo_positive, LIB), Cint, (Ptr{Cvoid}, Clonglong, Ptr{Cvoid}),
                dptr(x), Clonglong(length(x)), cstream()))
    x
end

# ---------------------------------------------------------------------------
# SquaredFieldDifference (squared_field_difference.jl:35-61)
# ---------------------------------------------------------------------------
mutable struct GB300SFD{V}
    handle::Ptr{Cvoid}
    v::V                      # reference field
    c::CuArray{Float32, 1}
end

"""
    GB300SquaredFieldDifference(v::ScalarField)

c_b = Σ|u_b − v_b|² per field over the pixels (no dx dy factor), and the pullback
∂u = 2 ∂c_b (u_b − v_b).
"""
function GB300SquaredFieldDifference(v::ScalarField)
    nx, ny, b = dims_of(v)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:fo_sfd_create, LIB), Cint, (Ref{Ptr{Cvoid}}, Cint, Cint, Cint), h, nx, ny, b))
    m = GB300SFD(h[], v, CUDA.zeros(Float32, b))
    finalizer(x -> ccall((:fo_sfd_destroy, LIB), Cint, (Ptr{Cvoid},), x.handle), m)
end

function (m::GB300SFD)(u::ScalarField)
    check(ccall((:fo_sfd_forward, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                m.handle, dptr(u.electric), dptr(m.v.electric), dptr(m.c), cstream()))
    m.c
end

function pullback!(m::GB300SFD, ∂c, u::ScalarField, ∂u::ScalarField)
    check(ccall((:fo_sfd_backward, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                m.handle, dptr(u.electric), dptr(m.v.electric), ∂c === nothing ? C_NULL : dptr(∂c),
                dptr(∂u.electric), cstream()))
    ∂u
end

"""
    withgradient!(∂u, c::GB300Chain, u_in, m::GB300SFD; ∂c=nothing, u_out=nothing, input_grad=true) -> c

Zygote.withgradient for a chain with SquaredFieldDifference as the loss
(fo_chain_withgradient_sfd): forward sweep, metric, its pullback 2 ∂c_b (u_b − v_b)
and the adjoint sweep, the forward's last row pass and the adjoint's first shared
when the chain ends in a propagator.  Returns the per-field values `m.c`.
"""
function withgradient!(∂u::ScalarField, c::GB300Chain, u_in::ScalarField, m::GB300SFD;
                       ∂c = nothing, u_out = nothing, input_grad::Bool = true, dir::Type{<:Direction} = Forward)
    mf = [_fomod(x, _saved(x), nothing) for x in c.mods]
    mb = [_fomod(x, _saved(x), _grad(x)) for x in c.mods]
    check(ccall((:fo_chain_withgradient_sfd, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{FoMod}, Ptr{FoMod}, Cint, Ptr{Cvoid},
                 Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                c.chain, dptr(u_in.electric), u_out === nothing ? C_NULL : dptr(u_out.electric),
                dptr(∂u.electric), mf, mb, dirsign(dir), m.handle, dptr(m.v.electric),
                ∂c === nothing ? C_NULL : dptr(∂c), dptr(m.c), input_grad ? Cint(0) : Cint(1), cstream()))
    m.c
end

mutable struct GB300TV
    handle::Ptr{Cvoid}
end

"""
    GB300TVProx(nx, ny, λ; n_iter=50, tol=nothing, isotropic=true, eta=0.25)

TVProx(λ, n_iter; tol, isotropic, rule = Fista(eta)) for nx × ny parameters; apply
with `tv_prox!(tv, x)`.  `tol` stops the iterations on the device (tv_prox.jl:150-166).
"""
function GB300TVProx(nx::Integer, ny::Integer, λ::Real; n_iter::Integer = 50, tol = nothing,
                     isotropic::Bool = true, eta::Real = 0.25)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:fo_tv_create_ex, LIB), Cint,
                (Ref{Ptr{Cvoid}}, Cint, Cint, Cdouble, Cint, Cint, Cdouble, Cdouble),
                h, nx, ny, λ, n_iter, Cint(isotropic), eta, tol === nothing ? 0.0 : Float64(tol)))
    tv = GB300TV(h[])
    finalizer(x -> ccall((:fo_tv_destroy, LIB), Cint, (Ptr{Cvoid},), x.handle), tv)
end

# the same for a 1-, 2- or 3-D parameter of size `dims` (Julia order, x fastest)
function GB300TVProx(dims::NTuple{N, Integer}, λ::Real; n_iter::Integer = 50, tol = nothing,
                     isotropic::Bool = true, eta::Real = 0.25) where {N}
    d = Cint[dims...]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:fo_tv_create_nd, LIB), Cint,
                (Ref{Ptr{Cvoid}}, Cint, Ptr{Cint}, Cdouble, Cint, Cint, Cdouble, Cdouble),
                h, Cint(N), d, λ, n_iter, Cint(isotropic), eta, tol === nothing ? 0.0 : Float64(tol)))
    tv = GB300TV(h[])
    finalizer(x -> ccall((:fo_tv_destroy, LIB), Cint, (Ptr{Cvoid},), x.handle), tv)
end

function tv_prox!(tv::GB300TV, x::CuArray{Float32})
    check(ccall((:fo_tv_apply, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}), tv.handle, dptr(x), cstream()))
    x
end

# ---------------------------------------------------------------------------
# DotProduct / PowerCoupling against reference fields v (same grid and batch)
# ---------------------------------------------------------------------------
mutable struct GB300Overlap
    handle::Ptr{Cvoid}
    out::Any                  # CuArray{ComplexF32} (DotProduct) or CuArray{Float32} (PowerCoupling)
end

function GB300Overlap(v::ScalarField; mode_selective::Bool = true, power::Bool = false)
    nx, ny, b = dims_of(v)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:fo_overlap_create, LIB), Cint,
                (Ref{Ptr{Cvoid}}, Cint, Cint, Cint, Cdouble, Cdouble, Ptr{Cvoid}, Cint, Cint),
                h, nx, ny, b, v.ds[1], v.ds[2], dptr(v.electric), Cint(mode_selective), Cint(power)))
    n = mode_selective ? b : b * b
    out = power ? CUDA.zeros(Float32, n) : CUDA.zeros(ComplexF32, n)
    o = GB300Overlap(h[], out)
    finalizer(x -> ccall((:fo_overlap_destroy, LIB), Cint, (Ptr{Cvoid},), x.handle), o)
end
GB300DotProduct(v::ScalarField; mode_selective = true) = GB300Overlap(v; mode_selective, power = false)
GB300PowerCoupling(v::ScalarField; mode_selective = true) = GB300Overlap(v; mode_selective, power = true)

# compute_metric / backpropagate_metric of dot_product.jl:70-100 and power_coupling.jl:59-66
function (o::GB300Overlap)(u::ScalarField)
    check(ccall((:fo_overlap_forward, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                o.handle, dptr(u.electric), dptr(o.out), cstream()))
    o.out
end
function pullback!(o::GB300Overlap, ∂c, ∂u::ScalarField)
    check(ccall((:fo_overlap_backward, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                o.handle, dptr(∂c), dptr(∂u.electric), cstream()))
    ∂u
end

# ---------------------------------------------------------------------------
# Ragged batch: independent Phase |> ASProp |> SquaredIntensityDifference problems
# of different sizes, forward + adjoint of all of them in one persistent launch.
# ---------------------------------------------------------------------------
struct FoRaggedProblem  # mirrors `fo_ragged_problem`
    n::Cint
    dx::Cdouble
    dy::Cdouble
    lambda::Cdouble
    z::Cdouble
    n0::Cdouble
    u_in::Ptr{Cvoid}
    phase::Ptr{Cvoid}
    target::Ptr{Cvoid}
    u_out::Ptr{Cvoid}
    grad_phase::Ptr{Cvoid}
    loss::Ptr{Cvoid}
end

mutable struct GB300Ragged
    handle::Ptr{Cvoid}
    outputs::Vector{CuArray{ComplexF32, 2}}
    grads::Vector{CuArray{Float32, 2}}
    losses::CuArray{Float32, 1}
    keep::Vector{Any}          # the bound input arrays stay alive with the plan
end

# problems: tuples (u::ScalarField (one n x n field, n a power of two 256..4096),
#                    ϕ::CuMatrix{Float32}, target::CuMatrix{Float32}, z; n0 = 1)
function GB300Ragged(problems)
    m = length(problems)
    losses = CUDA.zeros(Float32, m)
    outs = CuArray{ComplexF32, 2}[]
    grads = CuArray{Float32, 2}[]
    keep = Any[]
    descs = FoRaggedProblem[]
    for (k, (u, ϕ, t, z)) in enumerate(problems)
        n = size(u.electric, 1)
        uin = reshape(u.electric, n, n)
        out = similar(uin)
        g = similar(ϕ)
        push!(outs, out); push!(grads, g); push!(keep, uin, ϕ, t)
        ds = FluxOptics.get_ds(u)
        push!(descs, FoRaggedProblem(n, ds[1], ds[2], lambdas_per_field(u)[1], z, 1.0,
                                     dptr(uin), dptr(ϕ), dptr(t), dptr(out), dptr(g),
                                     dptr(losses) + (k - 1) * sizeof(Float32)))
    end
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:fo_ragged_create, LIB), Cint, (Ref{Ptr{Cvoid}}, Ptr{FoRaggedProblem}, Cint, Cint),
                h, descs, m, 0))
    r = GB300Ragged(h[], outs, grads, losses, keep)
    finalizer(x -> ccall((:fo_ragged_destroy, LIB), Cint, (Ptr{Cvoid},), x.handle), r)
    r
end

# withgradient of every problem at once: (losses, propagated fields, ∂ϕ)
function run!(r::GB300Ragged)
    check(ccall((:fo_ragged_batch, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), r.handle, cstream()))
    (r.losses, r.outputs, r.grads)
end

end # module
