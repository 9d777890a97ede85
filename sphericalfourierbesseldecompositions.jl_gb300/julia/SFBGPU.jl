# SFBGPU.jl - Julia binding of libsfbgpu.so (include/sfb_gpu.h) for
# SphericalFourierBesselDecompositions.jl.
#
# Drop-in replacements for SFB.cat2amln / SFB.cat2nlm, SFB.field2anlm,
# SFB.anlm2field and SFB.win_rhat_ln (reference src/cat2anlm.jl:257-422,
# src/windows.jl:244-270) with the same argument meaning, and for the window
# helpers SFB.apply_window, SFB.win_lnn, SFB.calc_wmix, SFB.amln2clnn and
# SFB.winweights2galweights.  The device plan is
# built once per AnlmModes (its k_nl, spline tables and ordering) and freed by
# a finalizer.  Errors map to the exceptions the reference raises.
#
# Differentiation: ChainRulesCore.rrule methods for cat2amln (with respect to
# the galaxy weights) and field2anlm (with respect to the shell x pixel field)
# pull a cotangent ā = ∂L/∂Re(a) + i ∂L/∂Im(a) back through the library's
# hand-written adjoint kernels (sfb_cat2amln_vjp, sfb_field2anlm_vjp_typed).
# Both transforms are linear in the differentiated argument, so the pullbacks
# keep no activations: the only state is the inputs the caller already holds.
# A field larger than the device budget streams through HBM one chunk of
# shells at a time in the forward and in the pullback alike.
module SFBGPU

using SphericalFourierBesselDecompositions
const SFB = SphericalFourierBesselDecompositions
using Random
import ChainRulesCore
using ChainRulesCore: NoTangent, ZeroTangent, AbstractZero, unthunk, @not_implemented

const libsfb = get(ENV, "SFBGPU_LIB", joinpath(@__DIR__, "..", "libsfbgpu.so"))

const SFB_OK, SFB_EINVAL, SFB_ENOMEM, SFB_ENONFINITE, SFB_ERANGE, SFB_ETIMEOUT, SFB_ECUDA, SFB_ENOTSUP = 0:7
const PRECISION = Dict(:fp64 => Int32(0), :mixed => Int32(1))
const DTYPE = Dict(Float64 => Int32(0), Float32 => Int32(1))     # sfb_dtype
const RADIAL = Dict(:poly => Int32(0), :spline => Int32(1))

# Field order and types follow sfb_plan_desc / sfb_window exactly.
struct PlanDesc
    nside::Int64
    lmax::Int64
    nmax::Int64
    lmax_n::Ptr{Int64}
    rmin::Float64
    rmax::Float64
    spl_offset::Ptr{Int64}
    spl_x::Ptr{Float64}
    spl_y::Ptr{Float64}
    spl_ypp::Ptr{Float64}
    niter::Int32
    precision::Int32
    radial_mode::Int32
    radial_pieces::Int32
    radial_degree::Int32
    radial_tol::Float64
end

struct Window
    kind::Int32
    mask::Ptr{Float64}
    w_ln::Ptr{Float64}
    dense::Ptr{Float64}
end

function lasterror()
    buf = Vector{UInt8}(undef, 1024)
    ccall((:sfb_last_error, libsfb), Cint, (Ptr{UInt8}, Csize_t), buf, length(buf))
    return unsafe_string(pointer(buf))
end

function check(st::Integer)
    st == SFB_OK && return nothing
    msg = lasterror()
    st == SFB_ENONFINITE && throw(AssertionError(msg))      # @assert all(isfinite.(anlm))
    st == SFB_EINVAL && throw(ArgumentError(msg))
    st == SFB_ERANGE && error(msg)                           # mymap2alm!'s lmax > 4*nside error
    error("libsfbgpu status $st: $msg")
end

mutable struct Plan
    handle::Ptr{Cvoid}
    nlmsize::Int
    npix::Int
end

function Plan(amodes::SFB.AnlmModes; niter=3, precision=:mixed, radial=:poly,
              pieces=0, degree=0, tol=0.0)
    pairs = [(n, l) for n in 1:amodes.nmax for l in 0:amodes.lmax_n[n]]
    gnl = amodes.basisfunctions.gnl          # Spline1D{3} per (n, l+1)
    xs = [gnl[n, l+1].x for (n, l) in pairs]
    off = Int64[0; cumsum(length.(xs))]
    x = reduce(vcat, xs)
    y = reduce(vcat, [gnl[n, l+1].y for (n, l) in pairs])
    ypp = reduce(vcat, [gnl[n, l+1].ypp for (n, l) in pairs])
    lmax_n = Int64.(amodes.lmax_n)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve x y ypp off lmax_n begin
        d = PlanDesc(amodes.nside, amodes.lmax, amodes.nmax, pointer(lmax_n), amodes.rmin, amodes.rmax,
                     pointer(off), pointer(x), pointer(y), pointer(ypp), niter, PRECISION[precision],
                     RADIAL[radial], pieces, degree, tol)
        check(ccall((:sfb_plan_create, libsfb), Cint, (Ref{PlanDesc}, Ref{Ptr{Cvoid}}), d, h))
    end
    p = Plan(h[], SFB.getnlmsize(amodes), 12 * amodes.nside^2)
    finalizer(q -> ccall((:sfb_plan_destroy, libsfb), Cvoid, (Ptr{Cvoid},), q.handle), p)
    return p
end

const PLANS = IdDict{Any,Plan}()
getplan(amodes; kw...) = get!(() -> Plan(amodes; kw...), PLANS, (amodes, kw...))

function window(w, amodes)
    if w isa SFB.SeparableArrays.SeparableArray
        return Window(1, pointer(w.mask), pointer(w.w_ln), C_NULL), (w.mask, w.w_ln)
    end
    W = Array{Float64,3}(w)                  # npix x (lmax+1) x nmax, column-major
    return Window(2, C_NULL, C_NULL, pointer(W)), (W,)
end

"""
    cat2amln(rθϕ, amodes, nbar, win_rhat_ln, weight=ones(N); kw...)

Same contract as `SFB.cat2amln` (src/cat2anlm.jl:257-310); runs on the GPU.
"""
function cat2amln(rθϕ, amodes, nbar, win_rhat_ln, weight=ones(size(rθϕ, 2)); kw...)
    p = getplan(amodes; kw...)
    r = Matrix{Float64}(rθϕ)
    N = size(r, 2)
    w = isempty(weight) ? C_NULL : Vector{Float64}(weight)
    anlm = Vector{ComplexF64}(undef, p.nlmsize)
    win, keep = window(win_rhat_ln, amodes)
    GC.@preserve r w keep anlm begin
        check(ccall((:sfb_cat2amln, libsfb), Cint,
                    (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64, Float64, Ref{Window}, Ptr{ComplexF64}),
                    p.handle, N == 0 ? C_NULL : r, w, N, nbar, win, anlm))
    end
    return anlm
end

const cat2nlm = cat2amln

"""
    cat2amln_batched(catalogues, amodes, nbars, win_rhat_ln, weights=nothing; kw...)

Mock batches: `catalogues` a vector of 3×N_k matrices, `nbars` one n̄ per mock;
returns nlmsize × nmocks, column k = `SFB.cat2amln(catalogues[k], amodes,
nbars[k], win_rhat_ln, weights[k])` (src/cat2anlm.jl:257-310 per mock).
"""
function cat2amln_batched(catalogues, amodes, nbars, win_rhat_ln, weights=nothing; kw...)
    p = getplan(amodes; kw...)
    sizes = [size(c, 2) for c in catalogues]
    offsets = Int64[0; cumsum(sizes)]
    r = isempty(catalogues) ? zeros(3, 0) : reduce(hcat, [Matrix{Float64}(c) for c in catalogues])
    w = weights === nothing ? C_NULL : Vector{Float64}(reduce(vcat, weights))
    nb = Vector{Float64}(nbars)
    anlm = Matrix{ComplexF64}(undef, p.nlmsize, length(catalogues))
    win, keep = window(win_rhat_ln, amodes)
    GC.@preserve r w nb offsets keep anlm begin
        check(ccall((:sfb_cat2amln_batched, libsfb), Cint,
                    (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Int64}, Int64, Ptr{Float64}, Ref{Window},
                     Ptr{ComplexF64}),
                    p.handle, offsets[end] == 0 ? C_NULL : r, w, offsets, length(catalogues), nb, win, anlm))
    end
    return anlm
end

"""
    field2anlm(f_xyz, wmodes, amodes)    (src/cat2anlm.jl:323-357)

A `Matrix{Float32}` field is passed as it is (no Float64 copy); any other
real matrix is converted to `Matrix{Float64}`.
"""
function field2anlm(f_xyz, wmodes, amodes; kw...)
    p = getplan(amodes; kw...)
    T = eltype(f_xyz) === Float32 ? Float32 : Float64
    f = Matrix{T}(f_xyz)
    out = Vector{ComplexF64}(undef, p.nlmsize)
    GC.@preserve f out check(ccall((:sfb_field2anlm_typed, libsfb), Cint,
                                   (Ptr{Cvoid}, Ptr{Cvoid}, Int32, Int64, Float64, Float64, Ptr{ComplexF64}),
                                   p.handle, f, DTYPE[T], wmodes.nr, wmodes.rmin, wmodes.rmax, out))
    return out
end

"""
    anlm2field(f_nlm, wmodes, amodes)    (src/cat2anlm.jl:383-422)
"""
function anlm2field(f_nlm, wmodes, amodes; kw...)
    p = getplan(amodes; kw...)
    a = Vector{ComplexF64}(f_nlm)
    f = Matrix{Float64}(undef, wmodes.nr, p.npix)
    GC.@preserve a f check(ccall((:sfb_anlm2field, libsfb), Cint,
                                 (Ptr{Cvoid}, Ptr{ComplexF64}, Int64, Float64, Float64, Ptr{Float64}),
                                 p.handle, a, wmodes.nr, wmodes.rmin, wmodes.rmax, f))
    return f
end

"""
    win_rhat_ln(win, wmodes, amodes)    (src/windows.jl:244-270)
"""
function win_rhat_ln(win, wmodes, amodes; kw...)
    p = getplan(amodes; kw...)
    if win isa SFB.SeparableArrays.SeparableArray
        phi = Vector{Float64}(win.phi)
        W = Matrix{Float64}(undef, amodes.lmax + 1, amodes.nmax)
        GC.@preserve phi W check(ccall((:sfb_win_rhat_ln_separable, libsfb), Cint,
                                       (Ptr{Cvoid}, Ptr{Float64}, Int64, Float64, Float64, Ptr{Float64}),
                                       p.handle, phi, wmodes.nr, wmodes.rmin, wmodes.rmax, W))
        return SFB.SeparableArrays.SeparableArray(win.mask, W, name1=:mask, name2=:w_ln)
    end
    w = Matrix{Float64}(win)
    W = Array{Float64,3}(undef, p.npix, amodes.lmax + 1, amodes.nmax)
    GC.@preserve w W check(ccall((:sfb_win_rhat_ln_dense, libsfb), Cint,
                                 (Ptr{Cvoid}, Ptr{Float64}, Int64, Float64, Float64, Ptr{Float64}),
                                 p.handle, w, wmodes.nr, wmodes.rmin, wmodes.rmax, W))
    return W
end

"""
    amln2clnn(anlm, cmodes)    (src/SphericalFourierBesselDecompositions.jl:133-150)

Pseudo-SFB power spectrum C_l(n1, n2) in the order of `cmodes.lnn` (3 × nlnn);
`anlm` is one a_nlm vector or a matrix of them (one per column).
"""
function amln2clnn(anlm, cmodes; kw...)
    amodes = cmodes.amodesA
    p = getplan(amodes; kw...)
    a = Matrix{ComplexF64}(reshape(anlm, p.nlmsize, :))
    nbatch = size(a, 2)
    lnn = Matrix{Int64}(cmodes.lnn)
    nlnn = size(lnn, 2)
    out = Matrix{Float64}(undef, nlnn, nbatch)
    GC.@preserve a lnn out check(ccall((:sfb_amln2clnn, libsfb), Cint,
                                       (Ptr{Cvoid}, Ptr{ComplexF64}, Ptr{ComplexF64}, Int64, Ptr{Int64}, Int64,
                                        Ptr{Float64}),
                                       p.handle, a, C_NULL, nbatch, lnn, nlnn, out))
    return nbatch == 1 ? vec(out) : out
end

"""
    win_lnn(win, wmodes, cmodes)    (src/windows.jl:382-392)

W_l(n, n') = Σ_s r_s² Δr g_nl(r_s) g_n'l(r_s) W_00(r_s) / √(4π) for every column
(l, n, n') of `cmodes.lnn`, with W_00 the shell a_00 of the window at 2 lmax (the
reference's `calc_Wr_lm(win, 2 lmax, nside)`).  `win` is the nr × npix window at
the plan's nside (a `SeparableArray` is materialised with `Matrix`).
"""
function win_lnn(win, wmodes, cmodes; kw...)
    p = getplan(cmodes.amodesA; kw...)
    W = Matrix{Float64}(win)
    lnn = Matrix{Int64}(cmodes.lnn)
    nlnn = size(lnn, 2)
    out = Vector{Float64}(undef, nlnn)
    GC.@preserve W lnn out check(ccall((:sfb_win_lnn, libsfb), Cint,
                                       (Ptr{Cvoid}, Ptr{Float64}, Int64, Float64, Float64, Ptr{Int64}, Int64,
                                        Ptr{Float64}),
                                       p.handle, W, wmodes.nr, wmodes.rmin, wmodes.rmax, lnn, nlnn, out))
    return out
end

"""
    calc_wmix(win, wmodes, amodes; neg_m=false)    (src/windows.jl:299-366)

The window mixing matrix W[(n l m), (n' l' m')] in `getidx` order on both axes,
an nlmsize × nlmsize `Matrix{ComplexF64}` (lmax ≤ 128).  `win` as in `win_lnn`.
"""
function calc_wmix(win, wmodes, amodes; neg_m=false, kw...)
    p = getplan(amodes; kw...)
    W = Matrix{Float64}(win)
    out = Matrix{ComplexF64}(undef, p.nlmsize, p.nlmsize)
    GC.@preserve W out check(ccall((:sfb_calc_wmix, libsfb), Cint,
                                   (Ptr{Cvoid}, Ptr{Float64}, Int64, Float64, Float64, Int32, Ptr{ComplexF64}),
                                   p.handle, W, wmodes.nr, wmodes.rmin, wmodes.rmax, Int32(neg_m), out))
    return out
end

"""
    cat2amln_vjp(rθϕ, amodes, nbar, abar; kw...) -> dL/dw

Gradient of a real loss L through `cat2amln` with respect to the galaxy
weights, given `abar = ∂L/∂Re(a) + i ∂L/∂Im(a)` (FP64 adjoint; the pullback of
the `ChainRulesCore.rrule` for `cat2amln` below).
"""
function cat2amln_vjp(rθϕ, amodes, nbar, abar; kw...)
    p = getplan(amodes; kw...)
    r = Matrix{Float64}(rθϕ)
    a = Vector{ComplexF64}(abar)
    dw = Vector{Float64}(undef, size(r, 2))
    GC.@preserve r a dw check(ccall((:sfb_cat2amln_vjp, libsfb), Cint,
                                    (Ptr{Cvoid}, Ptr{Float64}, Int64, Float64, Ptr{ComplexF64}, Ptr{Float64}),
                                    p.handle, size(r, 2) == 0 ? C_NULL : r, size(r, 2), nbar, a, dw))
    return dw
end

"""
    field2anlm_vjp(abar, wmodes, amodes; eltype=Float64, kw...) -> dL/df  (nr × npix)

`eltype=Float32` writes the gradient in Float32 (the element type of an FP32 field).
"""
function field2anlm_vjp(abar, wmodes, amodes; eltype=Float64, kw...)
    p = getplan(amodes; kw...)
    T = eltype === Float32 ? Float32 : Float64
    a = Vector{ComplexF64}(abar)
    df = Matrix{T}(undef, wmodes.nr, p.npix)
    GC.@preserve a df check(ccall((:sfb_field2anlm_vjp_typed, libsfb), Cint,
                                  (Ptr{Cvoid}, Ptr{ComplexF64}, Int64, Float64, Float64, Ptr{Cvoid}, Int32),
                                  p.handle, a, wmodes.nr, wmodes.rmin, wmodes.rmax, df, DTYPE[T]))
    return df
end

# ---------------------------------------------------------------- rrules ----
# cat2amln(rθϕ, amodes, nbar, win_rhat_ln[, weight]): the weight cotangent is
# the adjoint kernel's dL/dw; positions, n̄ and the window are not
# differentiated by this library (@not_implemented), amodes is not a tangent.
function ChainRulesCore.rrule(::typeof(cat2amln), rθϕ, amodes, nbar, win_rhat_ln,
                              weight=ones(size(rθϕ, 2)); kw...)
    a = cat2amln(rθϕ, amodes, nbar, win_rhat_ln, weight; kw...)
    function cat2amln_pullback(ā)
        ā = unthunk(ā)
        dw = ā isa AbstractZero ? ZeroTangent() : cat2amln_vjp(rθϕ, amodes, nbar, ā; kw...)
        return (NoTangent(), @not_implemented("galaxy positions"), NoTangent(), @not_implemented("nbar"),
                @not_implemented("win_rhat_ln"), dw)
    end
    return a, cat2amln_pullback
end

# field2anlm(f_xyz, wmodes, amodes): the field cotangent has the field's element type.
function ChainRulesCore.rrule(::typeof(field2anlm), f_xyz, wmodes, amodes; kw...)
    a = field2anlm(f_xyz, wmodes, amodes; kw...)
    T = eltype(f_xyz) === Float32 ? Float32 : Float64
    function field2anlm_pullback(ā)
        ā = unthunk(ā)
        df = ā isa AbstractZero ? ZeroTangent() : field2anlm_vjp(ā, wmodes, amodes; eltype=T, kw...)
        return (NoTangent(), df, NoTangent(), NoTangent())
    end
    return a, field2anlm_pullback
end

"""
    apply_window(rθϕ, win, wmodes; rng=Random.GLOBAL_RNG)    (src/windows.jl:169-216)

Same contract as `SFB.apply_window`: the galaxies kept by the window, in input
order.  The uniform draws come from `rand(rng, N)` on the host, so the same
`rng` state gives the reference's selection; the test on each galaxy runs on
the GPU.
"""
function apply_window(rθϕ, win, wmodes; rng=Random.GLOBAL_RNG)
    r = Matrix{Float64}(rθϕ)
    N = size(r, 2)
    W = Matrix{Float64}(win)                  # nr × npix
    u = rand(rng, N)
    out = Matrix{Float64}(undef, 3, N)
    kept = Ref{Int64}(0)
    GC.@preserve r W u out check(ccall((:sfb_apply_window, libsfb), Cint,
                                       (Int64, Ptr{Float64}, Int64, Float64, Float64, Float64, Ptr{Float64}, Int64,
                                        Ptr{Float64}, UInt64, Ptr{Float64}, Ref{Int64}),
                                       wmodes.nside, W, size(W, 1), wmodes.rmin, wmodes.rmax, wmodes.Δr,
                                       N == 0 ? C_NULL : r, N, N == 0 ? C_NULL : u, UInt64(0),
                                       N == 0 ? C_NULL : out, kept))
    return out[:, 1:kept[]]
end

"""
    winweights2galweights(weights, wmodes, rθϕ)    (src/cat2anlm.jl:218-238)
"""
function winweights2galweights(weights, wmodes, rθϕ)
    W = Matrix{Float64}(weights)              # nr × npix
    rb = Vector{Float64}(SFB.get_rbounds(wmodes))
    r = Matrix{Float64}(rθϕ)
    out = Vector{Float64}(undef, size(r, 2))
    GC.@preserve W rb r out check(ccall((:sfb_winweights2galweights, libsfb), Cint,
                                        (Int64, Ptr{Float64}, Int64, Ptr{Float64}, Ptr{Float64}, Int64,
                                         Ptr{Float64}),
                                        wmodes.nside, W, wmodes.nr, rb, r, size(r, 2), out))
    return out
end

end # module
