"""
    PushPullGB300

GPU methods of PushPull.jl's resampling functions for `CuArray{Float32}` arguments,
running the GB300 kernels of `libpushpull_gb300.so` through `ccall` on device pointers.
It is a drop-in for the package's CUDA extension (`ext/pushpull_gpu.jl`). The argument
order, `Settings` semantics, array layouts and return shapes are the same; each call
covers every (channel, batch) slice at once on the task's CUDA stream.

    using PushPull, CUDA
    include(joinpath(ENV["PUSHPULL_GB300"], "pushpull.jl_gb300", "julia", "PushPullGB300.jl"))
    using .PushPullGB300

Load it instead of the package's CUDA extension: both define methods for the same
`CuArray` signatures. Set `PUSHPULL_GB300_LIB` to point at the library when it is not
next to this file (`../lib/libpushpull_gb300.so`).

Beyond the reference's functions it provides:
- `fused_step(f₀, ϕ, g, sett)`: the loss Σ(pull(f₀, ϕ) − g)² and both cotangents in one
  pass;
- `pull_grad_dot` and `pull_hess_dot`, the contractions the rrules below use instead of
  building `pull_grad` / `pull_hess` temporaries.
"""
module PushPullGB300

using CUDA
using Libdl
using PushPull
import ChainRulesCore
using ChainRulesCore: NoTangent, @thunk, unthunk

export fused_step, pull_grad_dot, pull_hess_dot

const Settings = PushPull.Settings
const _lib = Ref{Ptr{Cvoid}}(C_NULL)

function __init__()
    path = get(ENV, "PUSHPULL_GB300_LIB", joinpath(@__DIR__, "..", "lib", "libpushpull_gb300.so"))
    _lib[] = Libdl.dlopen(path)
end

_sym(s::Symbol) = Libdl.dlsym(_lib[], s)

function _check(fn::Symbol, rc::Cint)
    rc == 0 && return nothing
    msg = unsafe_string(ccall(_sym(:pp_last_error), Cstring, ()))
    error("pushpull_gb300 $fn failed ($rc): $msg")
end

_deg(s::Settings) = Cint[Int(d) for d in s.deg]

# one boundary triple for every channel, or one per channel (pp_* `bnd`, `nbnd`)
function _bnd(s::Settings)
    v = Cint[]
    for b in s.bnd
        append!(v, Cint.(collect(b)))
    end
    return v, Cint(length(s.bnd))
end

_d3(a) = Culonglong[size(a)[1:3]...]
_stream() = CUDA.stream().handle

function _pull_family(fn::Symbol, f₀::CuArray{Float32}, ϕ::CuArray{Float32}, s::Settings, extra::Tuple)
    @assert(ndims(f₀) >= 3 && ndims(f₀) <= 5, "`f₀` must have between 3 & 5 dimensions")
    @assert(ndims(ϕ)  >= 4 && ndims(ϕ)  <= 5, "`ϕ` must have 4 or 5 dimensions")
    @assert(size(ϕ,4) == 3,                   "`ϕ` must have three channels")
    @assert(size(ϕ,5) == size(f₀,5),          "`ϕ` & `f₀` must have the same batch size")
    @assert(length(s.bnd)==size(f₀,4) || length(s.bnd)==1)
    Nc, Nb = size(f₀,4), size(f₀,5)
    out = CuArray{Float32}(undef, (size(ϕ)[1:3]..., extra..., size(f₀)[4:end]...))
    bnd, nbnd = _bnd(s)
    rc = ccall(_sym(fn), Cint,
               (CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat}, Ptr{Culonglong}, Ptr{Culonglong},
                Cint, Cint, Ptr{Cint}, Cint, Ptr{Cint}, Cint, Ptr{Cvoid}),
               out, ϕ, f₀, _d3(f₀), _d3(ϕ), Nc, Nb, bnd, nbnd, _deg(s),
               Cint(s.ext), _stream())
    _check(fn, rc)
    return out
end

function _push_family(fn::Symbol, f₁::CuArray{Float32}, ϕ::CuArray{Float32}, d₀, s::Settings, lead::Int)
    @assert(ndims(ϕ) >= 4 && ndims(ϕ) <= 5, "`ϕ` must have 4 or 5 dimensions")
    @assert(size(ϕ,4) == 3,                  "`ϕ` must have three channels")
    @assert(size(f₁)[1:3] == size(ϕ)[1:3],   "`f₁` and `ϕ` must have the same volume dimensions")
    Nc, Nb = size(f₁, lead+1), size(f₁, lead+2)
    @assert(size(ϕ,5) == Nb,                 "`ϕ` & `f₁` must have the same batch size")
    @assert(length(s.bnd)==Nc || length(s.bnd)==1)
    f₀ = CuArray{Float32}(undef, (d₀..., size(f₁)[lead+1:end]...))
    bnd, nbnd = _bnd(s)
    rc = ccall(_sym(fn), Cint,
               (CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat}, Ptr{Culonglong}, Ptr{Culonglong},
                Cint, Cint, Ptr{Cint}, Cint, Ptr{Cint}, Cint, Cint, Ptr{Cvoid}),
               f₀, ϕ, f₁, Culonglong[d₀...], _d3(ϕ), Nc, Nb, bnd, nbnd,
               _deg(s), Cint(s.ext), Cint(0), _stream())       # accumulate = 0: zeroed in-stream
    _check(fn, rc)
    return f₀
end

# ---- the reference's functions on CuArrays (ext/pushpull_gpu.jl) ------------

PushPull.pull(f₀::CuArray{Float32}, ϕ::CuArray{Float32}, s::Settings = Settings()) =
    _pull_family(:pp_pull, f₀, ϕ, s, ())

PushPull.pull_grad(f₀::CuArray{Float32}, ϕ::CuArray{Float32}, s::Settings = Settings()) =
    _pull_family(:pp_pull_grad, f₀, ϕ, s, (3,))

PushPull.pull_hess(f₀::CuArray{Float32}, ϕ::CuArray{Float32}, s::Settings = Settings()) =
    _pull_family(:pp_pull_hess, f₀, ϕ, s, (3, 3))

PushPull.push(f₁::CuArray{Float32}, ϕ::CuArray{Float32}, d₀::NTuple{3,Integer}, s::Settings = Settings()) =
    _push_family(:pp_push, f₁, ϕ, d₀, s, 3)

PushPull.push_grad(g₁::CuArray{Float32}, ϕ::CuArray{Float32}, d₀::NTuple{3,Integer}, s::Settings = Settings()) =
    _push_family(:pp_push_grad, g₁, ϕ, d₀, s, 4)

function _affine(fn::Symbol, push::Bool, x::CuArray{Float32}, Aff::Array{Float32,2}, dother, s::Settings)
    A = Vector{Cfloat}(vec(PushPull.adjust_affine(Aff)))        # 3x4, column-major, 0-based
    Nc, Nb = size(x,4), size(x,5)
    d₀, d₁ = push ? (dother, size(x)[1:3]) : (size(x)[1:3], dother)
    out = CuArray{Float32}(undef, (dother..., size(x)[4:end]...))
    bnd, nbnd = _bnd(s)
    rc = push ?
        ccall(_sym(fn), Cint, (CuPtr{Cfloat}, CuPtr{Cfloat}, Ptr{Cfloat}, Ptr{Culonglong}, Ptr{Culonglong},
                               Cint, Cint, Ptr{Cint}, Cint, Ptr{Cint}, Cint, Cint, Ptr{Cvoid}),
              out, x, A, Culonglong[d₀...], Culonglong[d₁...], Nc, Nb, bnd, nbnd, _deg(s), Cint(s.ext), Cint(0),
              _stream()) :
        ccall(_sym(fn), Cint, (CuPtr{Cfloat}, CuPtr{Cfloat}, Ptr{Cfloat}, Ptr{Culonglong}, Ptr{Culonglong},
                               Cint, Cint, Ptr{Cint}, Cint, Ptr{Cint}, Cint, Ptr{Cvoid}),
              out, x, A, Culonglong[d₀...], Culonglong[d₁...], Nc, Nb, bnd, nbnd, _deg(s), Cint(s.ext), _stream())
    _check(fn, rc)
    return out
end

PushPull.affine_pull(f₀::CuArray{Float32}, Aff::Array{Float32,2}, d₁::NTuple{3,Integer}, s::Settings = Settings()) =
    _affine(:pp_pull_affine, false, f₀, Aff, d₁, s)

PushPull.affine_push(f₁::CuArray{Float32}, Aff::Array{Float32,2}, d₀::NTuple{3,Integer}, s::Settings = Settings()) =
    _affine(:pp_push_affine, true, f₁, Aff, d₀, s)

# ---- contractions for the rrules, and the fused step ---------------------------

"""
    pull_grad_dot(f₀, ϕ, up, sett)

Σ_c up_c ⋅ ∇pull(f₀_c, ϕ): the deformation cotangent of `pull` for upstream `up`
(the layout of a `pull` output), shaped like `ϕ`.
"""
function pull_grad_dot(f₀::CuArray{Float32}, ϕ::CuArray{Float32}, up::CuArray{Float32}, s::Settings)
    Nc, Nb = size(f₀,4), size(f₀,5)
    dϕ = CuArray{Float32}(undef, size(ϕ))
    bnd, nbnd = _bnd(s)
    rc = ccall(_sym(:pp_pull_grad_dot), Cint,
               (CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat}, Ptr{Culonglong},
                Ptr{Culonglong}, Cint, Cint, Ptr{Cint}, Cint, Ptr{Cint}, Cint, Ptr{Cvoid}),
               dϕ, ϕ, f₀, up, _d3(f₀), _d3(ϕ), Nc, Nb, bnd, nbnd,
               _deg(s), Cint(s.ext), _stream())
    _check(:pp_pull_grad_dot, rc)
    return dϕ
end

"""
    pull_hess_dot(f₀, ϕ, up, sett)

Σ_c Σ_q H_c[:, q] up_c[q]: the deformation cotangent of `pull_grad` for upstream `up`
(the layout of a `pull_grad` output), shaped like `ϕ`.
"""
function pull_hess_dot(f₀::CuArray{Float32}, ϕ::CuArray{Float32}, up::CuArray{Float32}, s::Settings)
    Nc, Nb = size(f₀,4), size(f₀,5)
    dϕ = CuArray{Float32}(undef, size(ϕ))
    bnd, nbnd = _bnd(s)
    rc = ccall(_sym(:pp_pull_hess_dot), Cint,
               (CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat}, Ptr{Culonglong},
                Ptr{Culonglong}, Cint, Cint, Ptr{Cint}, Cint, Ptr{Cint}, Cint, Ptr{Cvoid}),
               dϕ, ϕ, f₀, up, _d3(f₀), _d3(ϕ), Nc, Nb, bnd, nbnd,
               _deg(s), Cint(s.ext), _stream())
    _check(:pp_pull_hess_dot, rc)
    return dϕ
end

"""
    loss, ∂f₀, ∂ϕ = fused_step(f₀, ϕ, g, sett)

loss = Σ (pull(f₀, ϕ) − g)², ∂f₀ = push(2r, ϕ) and ∂ϕ = Σ_c 2r ∇pull in one pass.
"""
function fused_step(f₀::CuArray{Float32}, ϕ::CuArray{Float32}, g::CuArray{Float32}, s::Settings)
    Nc, Nb = size(f₀,4), size(f₀,5)
    loss = CUDA.zeros(Float64, 1)
    ∂f = CuArray{Float32}(undef, size(f₀))
    ∂ϕ = CuArray{Float32}(undef, size(ϕ))
    bnd, nbnd = _bnd(s)
    rc = ccall(_sym(:pp_fused_step), Cint,
               (CuPtr{Cdouble}, CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat}, CuPtr{Cfloat},
                Ptr{Culonglong}, Ptr{Culonglong}, Cint, Cint, Ptr{Cint}, Cint, Ptr{Cint}, Cint, Cint, Ptr{Cvoid}),
               loss, ∂f, ∂ϕ, f₀, ϕ, g, _d3(f₀), _d3(ϕ), Nc, Nb, bnd, nbnd, _deg(s), Cint(s.ext), Cint(0),
               _stream())
    _check(:pp_fused_step, rc)
    return Array(loss)[1], ∂f, ∂ϕ
end

# ---- rrules (src/pushpull_pb.jl:11-51) on CuArrays ----------------------------

function ChainRulesCore.rrule(::typeof(PushPull.pull), f₀::CuArray{Float32}, ϕ::CuArray{Float32},
                              s::Settings = Settings())
    f₁ = PushPull.pull(f₀, ϕ, s)
    pb(δ) = (NoTangent(),
             @thunk(PushPull.push(unthunk(δ), ϕ, size(f₀)[1:3], s)),   # f₀
             @thunk(pull_grad_dot(f₀, ϕ, unthunk(δ), s)),             # ϕ
             NoTangent())
    return f₁, pb
end

function ChainRulesCore.rrule(::typeof(PushPull.pull_grad), f₀::CuArray{Float32}, ϕ::CuArray{Float32},
                              s::Settings = Settings())
    ∇f = PushPull.pull_grad(f₀, ϕ, s)
    pb(δ) = (NoTangent(),
             @thunk(PushPull.push_grad(unthunk(δ), ϕ, size(f₀)[1:3], s)),   # f₀
             @thunk(pull_hess_dot(f₀, ϕ, unthunk(δ), s)),                  # ϕ
             NoTangent())
    return ∇f, pb
end

function ChainRulesCore.rrule(::typeof(PushPull.push), f₁::CuArray{Float32}, ϕ::CuArray{Float32},
                              d₀::NTuple{3,Integer}, s::Settings = Settings())
    f₀ = PushPull.push(f₁, ϕ, d₀, s)
    pb(δ) = (NoTangent(),
             @thunk(PushPull.pull(unthunk(δ), ϕ, s)),               # f₁
             @thunk(pull_grad_dot(unthunk(δ), ϕ, f₁, s)),           # ϕ: Σ_c f₁ ⋅ ∇pull(δ)
             NoTangent(), NoTangent())
    return f₀, pb
end

end # module
