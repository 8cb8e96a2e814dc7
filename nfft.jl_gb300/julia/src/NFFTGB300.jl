"""
    NFFTGB300

AbstractNFFTs backend whose plans run on one NVIDIA GB300 through the C ABI
of `include/nfft_gb300.h` (libnfftgb300.so).  It is the drop-in replacement
of NFFT.jl's GPU plan (ext/NFFTGPUArraysExt/implementation.jl): the same
`plan_nfft(CuArray, k, N; m, σ, window, precompute, blocking)`, `mul!`,
`adjoint`, `nodes!` and optional `convolve!`/`convolve_transpose!`/
`deconvolve!`/`deconvolve_transpose!` surface, with the same exception types.

Usage:
    using CUDA, AbstractNFFTs, NFFTGB300
    NFFTGB300.activate!()
    p = plan_nfft(CuArray, k, N; m=4, σ=2.0)
    fHat = p * CuArray(f)
"""
module NFFTGB300

using AbstractNFFTs
using LinearAlgebra
using CUDA

const libnfft = Ref{String}(joinpath(@__DIR__, "..", "..", "nfftgb300", "libnfftgb300.so"))

# ---------------------------------------------------------------- C structs

struct CParams            # nfft_params
  m::Int32
  sigma::Float64
  window::Int32
  precompute::Int32
  blocking::Int32
  sort_nodes::Int32
  store_deconv_idx::Int32
  block_size::NTuple{3,Int64}
  compensated::Int32
  timing::Int32
end

struct CInfo              # nfft_info
  precision::Int32
  D::Int32
  N::NTuple{3,Int64}
  Ntilde::NTuple{3,Int64}
  M::Int64
  m::Int32
  sigma::Float64
  window::Int32
  precompute::Int32
  lut_size::Int64
  block_size::NTuple{3,Int64}
  num_tiles::Int64
  num_spread_tasks::Int64
  num_spread_entries::Int64
  scratch_bytes::Int64
end

const WINDOWS = Dict(:kaiser_bessel => 0, :gauss => 1, :spline => 2, :kaiser_bessel_rev => 3, :cosh_type => 4)

# Status codes -> the reference's exceptions (src/utils.jl:46-55, :98-105,
# src/convolution.jl:47-53, src/windowFunctions.jl:16).
function check(rc::Integer)
  rc == 0 && return nothing
  msg = unsafe_string(ccall((:nfft_last_error, libnfft[]), Cstring, ()))
  (rc == 1 || rc == 3) && throw(ArgumentError(msg))
  rc == 2 && throw(DimensionMismatch(msg))
  rc == 8 && error(msg)
  throw(ErrorException(unsafe_string(ccall((:nfft_status_string, libnfft[]), Cstring, (Cint,), rc)) * ": " * msg))
end

# ------------------------------------------------------------------ backend

struct GB300Backend <: AbstractNFFTBackend end
activate!() = AbstractNFFTs.set_active_backend!(NFFTGB300)
backend() = GB300Backend()

Base.@kwdef mutable struct GB300Params{T}
  m::Int = 4
  σ::T = 2.0
  reltol::T = 1e-7
  window::Symbol = :kaiser_bessel
  LUTSize::Int = 0
  precompute::AbstractNFFTs.PrecomputeFlags = AbstractNFFTs.POLYNOMIAL
  sortNodes::Bool = false
  storeDeconvolutionIdx::Bool = false
  blocking::Bool = true
  blockSize::NTuple{3,Int} = (0, 0, 0)
end

mutable struct GB300NFFTPlan{T,D} <: AbstractNFFTPlan{T,D,1}
  handle::Ptr{Cvoid}
  N::NTuple{D,Int}
  NOut::NTuple{1,Int}
  J::Int
  k::Matrix{T}
  Ñ::NTuple{D,Int}
  dims::UnitRange{Int}
  params::GB300Params{T}
  tmpVec::CuArray{Complex{T},D}
end

function AbstractNFFTs.plan_nfft(::GB300Backend, ::Type{<:CuArray}, k::Matrix{T}, N::NTuple{D,Int}, rest...;
                                 timing::Union{Nothing,TimingStats}=nothing, dims=1:D, fftflags=nothing,
                                 window::Symbol=:kaiser_bessel, precompute=AbstractNFFTs.POLYNOMIAL,
                                 blocking::Bool=true, sortNodes::Bool=false, storeDeconvolutionIdx::Bool=false,
                                 blockSize=nothing, kwargs...) where {T<:Union{Float32,Float64},D}
  dims_ = dims isa Integer ? (dims:dims) : dims
  if dims_ != 1:D
    return GB300DirectionalPlan(k, N, dims_; window, kwargs...)
  end
  size(k, 1) == D || throw(ArgumentError("Nodes x have dimension $(size(k,1)) != $D"))
  haskey(WINDOWS, window) || error("Window $(window) not yet implemented!")
  t = @elapsed begin
    m, σ, reltol = AbstractNFFTs.accuracyParams(; kwargs...)
    bs = blockSize === nothing ? (0, 0, 0) : ntuple(d -> d <= length(blockSize) ? blockSize[d] : 0, 3)
    cp = CParams(m, σ, WINDOWS[window], Int(precompute), blocking, sortNodes, storeDeconvolutionIdx, bs, 0,
                 timing === nothing ? 0 : 1)
    Nc = Int64[N...; ones(Int64, 3 - D)]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:nfft_plan_create, libnfft[]), Cint,
                (Ref{Ptr{Cvoid}}, Cint, Cint, Ptr{Int64}, Int64, Ref{CParams}, Ptr{Cvoid}),
                h, T == Float32 ? 32 : 64, D, Nc, size(k, 2), cp, CUDA.stream().handle))
    info = Ref{CInfo}()
    check(ccall((:nfft_get_info, libnfft[]), Cint, (Ptr{Cvoid}, Ref{CInfo}), h[], info))
    Ñ = ntuple(d -> Int(info[].Ntilde[d]), D)
    grid = ccall((:nfft_grid, libnfft[]), Ptr{Cvoid}, (Ptr{Cvoid},), h[])
    tmpVec = unsafe_wrap(CuArray, CuPtr{Complex{T}}(UInt(grid)), Ñ; own=false)
    params = GB300Params{T}(; m, σ=T(info[].sigma), reltol=T(reltol), window, LUTSize=Int(info[].lut_size),
                            precompute, sortNodes, storeDeconvolutionIdx, blocking,
                            blockSize=ntuple(d -> Int(info[].block_size[d]), 3))
    p = GB300NFFTPlan{T,D}(h[], N, (size(k, 2),), size(k, 2), k, Ñ, 1:D, params, tmpVec)
    finalizer(p) do q
      q.handle == C_NULL || ccall((:nfft_plan_destroy, libnfft[]), Cint, (Ptr{Cvoid},), q.handle)
      q.handle = C_NULL
    end
    AbstractNFFTs.nodes!(p, k)
  end
  timing === nothing || (timing.pre = t)
  return p
end

AbstractNFFTs.size_in(p::GB300NFFTPlan) = p.N
AbstractNFFTs.size_out(p::GB300NFFTPlan) = p.NOut

function bind_stream!(p::GB300NFFTPlan)
  check(ccall((:nfft_set_stream, libnfft[]), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), p.handle, CUDA.stream().handle))
end

# k .= sortslices(k, dims=2) on the caller's array (sortNodes = true,
# src/precomputation.jl:52-54, src/implementation.jl:112-114), sorted on the
# device by nfft_sort_nodes after the checkNodes test.
function sort_nodes!(k::Matrix{T}) where {T<:Union{Float32,Float64}}
  check(ccall((:nfft_sort_nodes, libnfft[]), Cint, (Cint, Cint, Int64, Ptr{T}, Cint, Ptr{Cvoid}),
              T == Float32 ? 32 : 64, size(k, 1), size(k, 2), k, 0, CUDA.stream().handle))
  return k
end

function AbstractNFFTs.nodes!(p::GB300NFFTPlan{T}, k::Matrix{T}) where {T}
  size(k, 2) == p.J || throw(DimensionMismatch("nodes! keeps the number of nodes; build a new plan for J ≠ $(p.J)"))
  bind_stream!(p)
  p.params.sortNodes && sort_nodes!(k)
  check(ccall((:nfft_set_nodes, libnfft[]), Cint, (Ptr{Cvoid}, Ptr{T}, Cint), p.handle, k, 0))
  p.k = k
  return p
end

function consistency(p::GB300NFFTPlan, f, fHat)
  (size_in(p) == size(f) && size_out(p) == size(fHat)) ||
    throw(DimensionMismatch("Data is not consistent with NFFTPlan"))
end

function LinearAlgebra.mul!(fHat::CuVector{Complex{T}}, p::GB300NFFTPlan{T,D}, f::CuArray{Complex{T},D};
                            verbose=false, timing::Union{Nothing,TimingStats}=nothing) where {T,D}
  consistency(p, f, fHat)
  bind_stream!(p)
  check(ccall((:nfft_forward, libnfft[]), Cint, (Ptr{Cvoid}, CuPtr{Complex{T}}, CuPtr{Complex{T}}),
              p.handle, f, fHat))
  timing === nothing || fill_timing!(p, timing)
  return fHat
end

function LinearAlgebra.mul!(f::CuArray{Complex{T},D}, pl::Adjoint{Complex{T},<:GB300NFFTPlan{T,D}},
                            fHat::CuVector{Complex{T}}; verbose=false,
                            timing::Union{Nothing,TimingStats}=nothing) where {T,D}
  p = pl.parent
  consistency(p, f, fHat)
  bind_stream!(p)
  check(ccall((:nfft_adjoint, libnfft[]), Cint, (Ptr{Cvoid}, CuPtr{Complex{T}}, CuPtr{Complex{T}}),
              p.handle, fHat, f))
  timing === nothing || fill_timing!(p, timing)
  return f
end

function fill_timing!(p::GB300NFFTPlan, t::TimingStats)
  v = zeros(Float64, 7)
  check(ccall((:nfft_get_timing, libnfft[]), Cint, (Ptr{Cvoid}, Ptr{Float64}), p.handle, v))
  t.conv, t.fft, t.deconv = v[2], v[3], v[4]
  t.conv_adjoint, t.fft_adjoint, t.deconv_adjoint = v[5], v[6], v[7]
  return t
end

# Optional interface; real arrays are accepted for NFFTTools.sdc.
const RC{T} = Union{T,Complex{T}}

function AbstractNFFTs.convolve!(p::GB300NFFTPlan{T,D}, g::CuArray{<:RC{T},D}, fHat::CuVector{<:RC{T}}) where {T,D}
  size(g) == p.Ñ || throw(DimensionMismatch("size(g)=$(size(g)) ≠ Ñ = $(p.Ñ)"))
  size(fHat) == (p.J,) || throw(DimensionMismatch("size(fHat)=$(size(fHat)) ≠ J = $(p.J)"))
  bind_stream!(p)
  check(ccall((:nfft_convolve, libnfft[]), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, Cint, CuPtr{Cvoid}, Cint),
              p.handle, g, eltype(g) <: Real, fHat, eltype(fHat) <: Real))
  return fHat
end

function AbstractNFFTs.convolve_transpose!(p::GB300NFFTPlan{T,D}, fHat::CuVector{<:RC{T}},
                                           g::CuArray{<:RC{T},D}) where {T,D}
  size(g) == p.Ñ || throw(DimensionMismatch("size(g)=$(size(g)) ≠ Ñ = $(p.Ñ)"))
  size(fHat) == (p.J,) || throw(DimensionMismatch("size(fHat)=$(size(fHat)) ≠ J = $(p.J)"))
  bind_stream!(p)
  check(ccall((:nfft_convolve_transpose, libnfft[]), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, Cint, CuPtr{Cvoid}, Cint),
              p.handle, fHat, eltype(fHat) <: Real, g, eltype(g) <: Real))
  return g
end

function AbstractNFFTs.deconvolve!(p::GB300NFFTPlan{T,D}, f::CuArray{Complex{T},D}, g::CuArray{Complex{T},D}) where {T,D}
  bind_stream!(p)
  check(ccall((:nfft_deconvolve, libnfft[]), Cint, (Ptr{Cvoid}, CuPtr{Complex{T}}, CuPtr{Complex{T}}),
              p.handle, f, g))
  return g
end

function AbstractNFFTs.deconvolve_transpose!(p::GB300NFFTPlan{T,D}, g::CuArray{Complex{T},D},
                                             f::CuArray{Complex{T},D}) where {T,D}
  bind_stream!(p)
  check(ccall((:nfft_deconvolve_transpose, libnfft[]), Cint, (Ptr{Cvoid}, CuPtr{Complex{T}}, CuPtr{Complex{T}}),
              p.handle, g, f))
  return f
end

"""
    grad_nodes!(dk, p, v, w)

dk[d, j] = Re(conj(w[j]) * ∂(A v)_j / ∂k[d, j]); the node gradient the
ChainRules pullback of `p * v` uses (no reference counterpart).
"""
function grad_nodes!(dk::CuMatrix{T}, p::GB300NFFTPlan{T,D}, v::CuArray{Complex{T},D},
                     w::CuVector{Complex{T}}) where {T,D}
  bind_stream!(p)
  check(ccall((:nfft_grad_nodes, libnfft[]), Cint,
              (Ptr{Cvoid}, CuPtr{Complex{T}}, CuPtr{Complex{T}}, CuPtr{T}), p.handle, v, w, dk))
  return dk
end

function Base.copy(p::GB300NFFTPlan{T,D}) where {T,D}
  AbstractNFFTs.plan_nfft(GB300Backend(), CuArray, copy(p.k), p.N; m=p.params.m, σ=p.params.σ,
                          window=p.params.window, precompute=p.params.precompute, blocking=p.params.blocking,
                          sortNodes=p.params.sortNodes)
end

# nfft(k, f) / nfft_adjoint(k, N, fHat) on device arrays with this backend
# active (AbstractNFFTs/src/derived.jl:140-151 builds an Array plan; a CuArray
# argument gets a GPU plan here).  The ChainRulesCore extension
# (ext/NFFTGB300ChainRulesCoreExt.jl) differentiates both in x and in k.
function AbstractNFFTs.nfft(b::GB300Backend, k, f::CuArray{Complex{T},D}; kwargs...) where {T,D}
  p = AbstractNFFTs.plan_nfft(b, CuArray, Matrix{T}(k), size(f); kwargs...)
  return p * f
end

function AbstractNFFTs.nfft_adjoint(b::GB300Backend, k, N, fHat::CuVector{Complex{T}}; kwargs...) where {T}
  p = AbstractNFFTs.plan_nfft(b, CuArray, Matrix{T}(k), Tuple(N); kwargs...)
  return adjoint(p) * fHat
end

"""
    autotune!(p; use_cache=true)

Pick the spreading tile shape (and 3-D warp layout) by timing the plan's own
nodes (`nfft_autotune`); the choice is cached in the file named by
`NFFT_GB300_TUNE_CACHE`.
"""
function autotune!(p::GB300NFFTPlan; use_cache::Bool=true)
  bind_stream!(p)
  check(ccall((:nfft_autotune, libnfft[]), Cint, (Ptr{Cvoid}, Cint), p.handle, use_cache))
  return p
end

"""
    set_tiling!(p, blockSize; row_parity_warps=1)

Re-tile the plan (the reference's `blockSize`) and re-bin its nodes; for
D = 3, `row_parity_warps = 2` spreads with 16 warps per tile.
"""
function set_tiling!(p::GB300NFFTPlan, blockSize; row_parity_warps::Integer=1)
  bs = Int64[ntuple(d -> d <= length(blockSize) ? blockSize[d] : 1, 3)...]
  bind_stream!(p)
  check(ccall((:nfft_set_tiling, libnfft[]), Cint, (Ptr{Cvoid}, Ptr{Int64}, Cint), p.handle, bs, row_parity_warps))
  return p
end

# ------------------------------------------------------------ directional plans

"""
    GB300DirectionalPlan

`plan_nfft(CuArray, k, N; dims)` with `dims` a contiguous range that is not
1:D (src/implementation.jl:73-104, src/directional.jl): the NFFT along `dims`,
every other index a batch column; `NOut` replaces the `dims` range of `N` by
J.  LINEAR window, as in the reference.
"""
mutable struct GB300DirectionalPlan{T,D,R} <: AbstractNFFTPlan{T,D,R}
  handle::Ptr{Cvoid}
  N::NTuple{D,Int}
  NOut::NTuple{R,Int}
  J::Int
  k::Matrix{T}
  dims::UnitRange{Int}
end

function GB300DirectionalPlan(k::Matrix{T}, N::NTuple{D,Int}, dims::UnitRange{Int}; window::Symbol=:kaiser_bessel,
                              kwargs...) where {T<:Union{Float32,Float64},D}
  size(k, 1) == length(dims) || throw(ArgumentError("Nodes x have dimension $(size(k,1)) != $(length(dims))"))
  (first(dims) >= 1 && last(dims) <= D) || throw(ArgumentError("dims $dims do not fit $D dimensions"))
  m, σ, reltol = AbstractNFFTs.accuracyParams(; kwargs...)
  cp = CParams(m, σ, WINDOWS[window], Int(AbstractNFFTs.LINEAR), false, false, false, (0, 0, 0), 0, 0)
  Nc = Int64[N...; ones(Int64, 3 - D)]
  h = Ref{Ptr{Cvoid}}(C_NULL)
  check(ccall((:nfft_dplan_create, libnfft[]), Cint,
              (Ref{Ptr{Cvoid}}, Cint, Cint, Ptr{Int64}, Cint, Cint, Int64, Ref{CParams}, Ptr{Cvoid}),
              h, T == Float32 ? 32 : 64, D, Nc, first(dims) - 1, last(dims) - 1, size(k, 2), cp, CUDA.stream().handle))
  J = size(k, 2)
  NOut = (N[1:first(dims)-1]..., J, N[last(dims)+1:end]...)
  p = GB300DirectionalPlan{T,D,length(NOut)}(h[], N, NOut, J, k, dims)
  finalizer(p) do q
    q.handle == C_NULL || ccall((:nfft_dplan_destroy, libnfft[]), Cint, (Ptr{Cvoid},), q.handle)
    q.handle = C_NULL
  end
  check(ccall((:nfft_dplan_set_nodes, libnfft[]), Cint, (Ptr{Cvoid}, Ptr{T}, Cint), p.handle, k, 0))
  return p
end

AbstractNFFTs.size_in(p::GB300DirectionalPlan) = p.N
AbstractNFFTs.size_out(p::GB300DirectionalPlan) = p.NOut

function LinearAlgebra.mul!(fHat::CuArray{Complex{T}}, p::GB300DirectionalPlan{T,D},
                            f::CuArray{Complex{T},D}) where {T,D}
  (size(f) == p.N && size(fHat) == p.NOut) || throw(DimensionMismatch("Data is not consistent with NFFTPlan"))
  check(ccall((:nfft_dplan_set_stream, libnfft[]), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), p.handle, CUDA.stream().handle))
  check(ccall((:nfft_dplan_forward, libnfft[]), Cint, (Ptr{Cvoid}, CuPtr{Complex{T}}, CuPtr{Complex{T}}),
              p.handle, f, fHat))
  return fHat
end

function LinearAlgebra.mul!(f::CuArray{Complex{T},D}, pl::Adjoint{Complex{T},<:GB300DirectionalPlan{T,D}},
                            fHat::CuArray{Complex{T}}) where {T,D}
  p = pl.parent
  (size(f) == p.N && size(fHat) == p.NOut) || throw(DimensionMismatch("Data is not consistent with NFFTPlan"))
  check(ccall((:nfft_dplan_set_stream, libnfft[]), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), p.handle, CUDA.stream().handle))
  check(ccall((:nfft_dplan_adjoint, libnfft[]), Cint, (Ptr{Cvoid}, CuPtr{Complex{T}}, CuPtr{Complex{T}}),
              p.handle, fHat, f))
  return f
end

# ---------------------------------------------------------------- batched plans

"""
    GB300Batch(plans)

Many plans of uneven N and M transformed together (`nfft_batch_*`, no
reference counterpart): one launch per stage over all plans, replayed from a
CUDA graph captured on the current stream.  `batch_mul!(fHats, b, fs)` and
`batch_mul_adjoint!(fs, b, fHats)` transform every plan.
"""
mutable struct GB300Batch
  handle::Ptr{Cvoid}
  plans::Vector{GB300NFFTPlan}
end

function GB300Batch(plans::Vector{<:GB300NFFTPlan})
  h = Ref{Ptr{Cvoid}}(C_NULL)
  handles = Ptr{Cvoid}[p.handle for p in plans]
  check(ccall((:nfft_batch_create, libnfft[]), Cint, (Ref{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Cint, Ptr{Cvoid}),
              h, handles, length(plans), CUDA.stream().handle))
  b = GB300Batch(h[], Vector{GB300NFFTPlan}(plans))
  finalizer(b) do q
    q.handle == C_NULL || ccall((:nfft_batch_destroy, libnfft[]), Cint, (Ptr{Cvoid},), q.handle)
    q.handle = C_NULL
  end
  return b
end

function batch_mul!(fHats::Vector{<:CuVector}, b::GB300Batch, fs::Vector{<:CuArray})
  length(fHats) == length(fs) == length(b.plans) || throw(DimensionMismatch("one input and output per plan"))
  fp = Ptr{Cvoid}[Ptr{Cvoid}(UInt(pointer(f))) for f in fs]
  hp = Ptr{Cvoid}[Ptr{Cvoid}(UInt(pointer(v))) for v in fHats]
  check(ccall((:nfft_batch_forward, libnfft[]), Cint, (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}),
              b.handle, fp, hp))
  return fHats
end

function batch_mul_adjoint!(fs::Vector{<:CuArray}, b::GB300Batch, fHats::Vector{<:CuVector})
  length(fHats) == length(fs) == length(b.plans) || throw(DimensionMismatch("one input and output per plan"))
  fp = Ptr{Cvoid}[Ptr{Cvoid}(UInt(pointer(f))) for f in fs]
  hp = Ptr{Cvoid}[Ptr{Cvoid}(UInt(pointer(v))) for v in fHats]
  check(ccall((:nfft_batch_adjoint, libnfft[]), Cint, (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}),
              b.handle, hp, fp))
  return fs
end

# ---------------------------------------------------------------- Toeplitz tools

"""
    GB300Toeplitz(shape, T; fft=:auto)

Workspace of NFFTTools' Toeplitz tools (NFFTTools/src/Toeplitz.jl) for images
of size `shape` and element type Complex{T}: the 2N grid and transforms that
`convolveToeplitzKernel!` takes as `fftplan, ifftplan, xOS1, xOS2`.
`fft=:cufft` forces the cuFFT sequence; `:auto` fuses the pruned transforms
with the kernel product where every 2N_d is a power of two in [64, 1024].
The methods below mirror NFFTTools' functions for CuArrays; a maintainer
hooks them into NFFTTools with, e.g.,
`NFFTTools.convolveToeplitzKernel!(y::CuArray, λ::CuArray, args...) =
NFFTGB300.convolveToeplitzKernel!(y, λ)`.
"""
mutable struct GB300Toeplitz{T,D}
  handle::Ptr{Cvoid}
  shape::NTuple{D,Int}
end

function GB300Toeplitz(shape::NTuple{D,Int}, ::Type{T}; fft::Symbol=:auto) where {T<:Union{Float32,Float64},D}
  fft in (:auto, :cufft) || throw(ArgumentError("fft must be :auto or :cufft"))
  h = Ref{Ptr{Cvoid}}(C_NULL)
  N = Int64[shape..., ones(Int64, 3 - D)...]
  check(ccall((:nfft_toeplitz_create, libnfft[]), Cint, (Ref{Ptr{Cvoid}}, Cint, Cint, Ptr{Int64}, Cint, Ptr{Cvoid}),
              h, T == Float32 ? 32 : 64, D, N, fft == :cufft ? 1 : 0, CUDA.stream().handle))
  t = GB300Toeplitz{T,D}(h[], shape)
  finalizer(t) do q
    q.handle == C_NULL || ccall((:nfft_toeplitz_destroy, libnfft[]), Cint, (Ptr{Cvoid},), q.handle)
    q.handle = C_NULL
  end
  return t
end

bind_stream!(t::GB300Toeplitz) =
  check(ccall((:nfft_toeplitz_set_stream, libnfft[]), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), t.handle, CUDA.stream().handle))

function isfused(t::GB300Toeplitz)
  r = Ref{Cint}(0)
  check(ccall((:nfft_toeplitz_is_fused, libnfft[]), Cint, (Ptr{Cvoid}, Ref{Cint}), t.handle, r))
  return r[] == 1
end

# calculateToeplitzKernel (Toeplitz.jl:86-93)
function calculateToeplitzKernel(shape::NTuple{D,Int}, tr::AbstractMatrix{T}; m=4, σ=2.0, window=:kaiser_bessel,
                                 toeplitz::GB300Toeplitz{T,D}=GB300Toeplitz(shape, T), kwargs...) where {T,D}
  p = AbstractNFFTs.plan_nfft(GB300Backend(), CuArray, Matrix{T}(tr), 2 .* shape; m, σ, window, kwargs...)
  λ = CuArray{Complex{T}}(undef, 2 .* shape)
  return calculateToeplitzKernel!(λ, p, toeplitz)
end

# calculateToeplitzKernel! (Toeplitz.jl:129-135)
function calculateToeplitzKernel!(λ::CuArray{Complex{T},D}, p::GB300NFFTPlan{T,D}, tr::Matrix{T},
                                  toeplitz::GB300Toeplitz{T,D}=GB300Toeplitz(p.N .÷ 2, T)) where {T,D}
  AbstractNFFTs.nodes!(p, tr)
  return calculateToeplitzKernel!(λ, p, toeplitz)
end

function calculateToeplitzKernel!(λ::CuArray{Complex{T},D}, p::GB300NFFTPlan{T,D}, t::GB300Toeplitz{T,D}) where {T,D}
  size(λ) == p.N == 2 .* t.shape || throw(DimensionMismatch("the kernel and the plan must have twice the image size"))
  bind_stream!(p)
  bind_stream!(t)
  check(ccall((:nfft_toeplitz_kernel, libnfft[]), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, CuPtr{Complex{T}}),
              t.handle, p.handle, λ))
  return λ
end

# calculateToeplitzKernel_explicit (Toeplitz.jl:142-164), sums in FP64
function calculateToeplitzKernel_explicit(shape::NTuple{D,Int}, tr::Matrix{T},
                                          t::GB300Toeplitz{T,D}=GB300Toeplitz(shape, T)) where {T,D}
  size(tr, 1) == D || throw(ArgumentError("Nodes x have dimension $(size(tr, 1)) != $D"))
  λ = CuArray{Complex{T}}(undef, 2 .* shape)
  kd = CuArray(tr)
  bind_stream!(t)
  check(ccall((:nfft_toeplitz_kernel_explicit, libnfft[]), Cint,
              (Ptr{Cvoid}, CuPtr{T}, Int64, Cint, CuPtr{Complex{T}}), t.handle, kd, size(tr, 2), 1, λ))
  return λ
end

# convolveToeplitzKernel! (Toeplitz.jl:230-244), y in place
function convolveToeplitzKernel!(y::CuArray{Complex{T},D}, λ::CuArray{Complex{T},D},
                                 t::GB300Toeplitz{T,D}=GB300Toeplitz(size(y), T)) where {T,D}
  size(λ) == 2 .* size(y) == 2 .* t.shape || throw(DimensionMismatch("the kernel must have twice the image size"))
  bind_stream!(t)
  check(ccall((:nfft_toeplitz_apply, libnfft[]), Cint, (Ptr{Cvoid}, CuPtr{Complex{T}}, CuPtr{Complex{T}}),
              t.handle, λ, y))
  return y
end

# ---------------------------------------------------------------- NFCT / NFST plans

const KIND_NDFT, KIND_NDCT, KIND_NDST, KIND_NNDFT = 0, 1, 2, 3

"""
    plan_nfct(CuArray, k, N; m, σ, window, ...)   /   plan_nfst(CuArray, k, N; ...)

NFCT / NFST plans (AbstractNFCTPlan / AbstractNFSTPlan) on the GPU NFFT of
size 2N of the even / odd extension (`nfft_tplan_*`); real data of type T.
The NFST input has N .- 1 points, as NDSTPlan.
"""
mutable struct GB300TrigPlan{T,D,KIND}
  handle::Ptr{Cvoid}
  N::NTuple{D,Int}
  J::Int
  k::Matrix{T}
end
const GB300NFCTPlan{T,D} = GB300TrigPlan{T,D,KIND_NDCT}
const GB300NFSTPlan{T,D} = GB300TrigPlan{T,D,KIND_NDST}

function trig_plan(kind::Int, k::Matrix{T}, N::NTuple{D,Int}; window::Symbol=:kaiser_bessel,
                   precompute=AbstractNFFTs.POLYNOMIAL, blocking::Bool=true, kwargs...) where {T,D}
  size(k, 1) == D || throw(ArgumentError("Nodes x have dimension $(size(k,1)) != $D"))
  m, σ, reltol = AbstractNFFTs.accuracyParams(; kwargs...)
  cp = CParams(m, σ, WINDOWS[window], Int(precompute), blocking, false, false, (0, 0, 0), 0, 0)
  Nc = Int64[N...; ones(Int64, 3 - D)]
  h = Ref{Ptr{Cvoid}}(C_NULL)
  check(ccall((:nfft_tplan_create, libnfft[]), Cint,
              (Ref{Ptr{Cvoid}}, Cint, Cint, Cint, Ptr{Int64}, Int64, Ref{CParams}, Ptr{Cvoid}),
              h, kind, T == Float32 ? 32 : 64, D, Nc, size(k, 2), cp, CUDA.stream().handle))
  p = GB300TrigPlan{T,D,kind}(h[], N, size(k, 2), k)
  finalizer(p) do q
    q.handle == C_NULL || ccall((:nfft_tplan_destroy, libnfft[]), Cint, (Ptr{Cvoid},), q.handle)
    q.handle = C_NULL
  end
  AbstractNFFTs.nodes!(p, k)
  return p
end

AbstractNFFTs.plan_nfct(::GB300Backend, ::Type{<:CuArray}, k::Matrix{T}, N::NTuple{D,Int}, rest...;
                        kwargs...) where {T<:Union{Float32,Float64},D} = trig_plan(KIND_NDCT, k, N; kwargs...)
AbstractNFFTs.plan_nfst(::GB300Backend, ::Type{<:CuArray}, k::Matrix{T}, N::NTuple{D,Int}, rest...;
                        kwargs...) where {T<:Union{Float32,Float64},D} = trig_plan(KIND_NDST, k, N; kwargs...)

AbstractNFFTs.size_in(p::GB300TrigPlan{T,D,KIND_NDCT}) where {T,D} = p.N
AbstractNFFTs.size_in(p::GB300TrigPlan{T,D,KIND_NDST}) where {T,D} = p.N .- 1
AbstractNFFTs.size_out(p::GB300TrigPlan) = (p.J,)

bind_stream!(p::GB300TrigPlan) =
  check(ccall((:nfft_tplan_set_stream, libnfft[]), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), p.handle, CUDA.stream().handle))

function AbstractNFFTs.nodes!(p::GB300TrigPlan{T}, k::Matrix{T}) where {T}
  size(k) == size(p.k) || throw(DimensionMismatch("nodes must be $(size(p.k))"))
  bind_stream!(p)
  check(ccall((:nfft_tplan_set_nodes, libnfft[]), Cint, (Ptr{Cvoid}, Ptr{T}, Cint), p.handle, k, 0))
  p.k = k
  return p
end

function LinearAlgebra.mul!(fHat::CuVector{T}, p::GB300TrigPlan{T,D}, f::CuArray{T,D}) where {T,D}
  size(f) == size_in(p) && length(fHat) == p.J || throw(DimensionMismatch("Data is not consistent with the plan"))
  bind_stream!(p)
  check(ccall((:nfft_tplan_forward, libnfft[]), Cint, (Ptr{Cvoid}, CuPtr{T}, CuPtr{T}), p.handle, f, fHat))
  return fHat
end

function LinearAlgebra.mul!(f::CuArray{T,D}, pl::Transpose{T,<:GB300TrigPlan{T,D}}, fHat::CuVector{T}) where {T,D}
  p = pl.parent
  size(f) == size_in(p) && length(fHat) == p.J || throw(DimensionMismatch("Data is not consistent with the plan"))
  bind_stream!(p)
  check(ccall((:nfft_tplan_transpose, libnfft[]), Cint, (Ptr{Cvoid}, CuPtr{T}, CuPtr{T}), p.handle, fHat, f))
  return f
end

# ---------------------------------------------------------------- NNFFT plans

"""
    plan_nnfft(CuArray, k, y; m, σ, window, ...)

Fast NNFFT (AbstractNNFFTPlan; the transform of NNDFTPlan): nodes k (D x J,
|k| <= 1/2), points y (D x N).  Spreading at y / N1, a forward NFFT of size
σ N1 at k / σ1 and a division by the window transform (`nfft_nnplan_*`).
"""
mutable struct GB300NNFFTPlan{T,D} <: AbstractNNFFTPlan{T,1,1}
  handle::Ptr{Cvoid}
  J::Int
  N::Int
  k::Matrix{T}
  y::Matrix{T}
end

function AbstractNFFTs.plan_nnfft(::GB300Backend, ::Type{<:CuArray}, k::Matrix{T}, y::Matrix{T}, rest...;
                                  window::Symbol=:kaiser_bessel, precompute=AbstractNFFTs.POLYNOMIAL,
                                  blocking::Bool=true, kwargs...) where {T<:Union{Float32,Float64}}
  D = size(k, 1)
  size(y, 1) == D || throw(ArgumentError("Nodes k have dimension $D != $(size(y, 1)) of the points y"))
  m, σ, reltol = AbstractNFFTs.accuracyParams(; kwargs...)
  cp = CParams(m, σ, WINDOWS[window], Int(precompute), blocking, false, false, (0, 0, 0), 0, 0)
  h = Ref{Ptr{Cvoid}}(C_NULL)
  check(ccall((:nfft_nnplan_create, libnfft[]), Cint,
              (Ref{Ptr{Cvoid}}, Cint, Cint, Int64, Int64, Ref{CParams}, Ptr{Cvoid}),
              h, T == Float32 ? 32 : 64, D, size(k, 2), size(y, 2), cp, CUDA.stream().handle))
  p = GB300NNFFTPlan{T,D}(h[], size(k, 2), size(y, 2), k, y)
  finalizer(p) do q
    q.handle == C_NULL || ccall((:nfft_nnplan_destroy, libnfft[]), Cint, (Ptr{Cvoid},), q.handle)
    q.handle = C_NULL
  end
  check(ccall((:nfft_nnplan_set_nodes, libnfft[]), Cint, (Ptr{Cvoid}, Ptr{T}, Ptr{T}, Cint), p.handle, k, y, 0))
  return p
end

AbstractNFFTs.size_in(p::GB300NNFFTPlan) = (p.N,)
AbstractNFFTs.size_out(p::GB300NNFFTPlan) = (p.J,)

bind_stream!(p::GB300NNFFTPlan) =
  check(ccall((:nfft_nnplan_set_stream, libnfft[]), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), p.handle, CUDA.stream().handle))

function LinearAlgebra.mul!(fHat::CuVector{Complex{T}}, p::GB300NNFFTPlan{T}, c::CuVector{Complex{T}}) where {T}
  length(c) == p.N && length(fHat) == p.J || throw(DimensionMismatch("Data is not consistent with the plan"))
  bind_stream!(p)
  check(ccall((:nfft_nnplan_forward, libnfft[]), Cint, (Ptr{Cvoid}, CuPtr{Complex{T}}, CuPtr{Complex{T}}),
              p.handle, c, fHat))
  return fHat
end

function LinearAlgebra.mul!(c::CuVector{Complex{T}}, pl::Adjoint{Complex{T},<:GB300NNFFTPlan{T}},
                            fHat::CuVector{Complex{T}}) where {T}
  p = pl.parent
  length(c) == p.N && length(fHat) == p.J || throw(DimensionMismatch("Data is not consistent with the plan"))
  bind_stream!(p)
  check(ccall((:nfft_nnplan_adjoint, libnfft[]), Cint, (Ptr{Cvoid}, CuPtr{Complex{T}}, CuPtr{Complex{T}}),
              p.handle, fHat, c))
  return c
end

# ---------------------------------------------------------------- direct transforms (src/direct.jl)

"""
    direct_mul!(out, kind, k, N, in; adjoint=false, y=nothing)

Exact NDFT / NDCT / NDST / NNDFT products on the GPU (`nfft_direct`, sums in
FP64): `kind` is KIND_NDFT, KIND_NDCT, KIND_NDST or KIND_NNDFT; `k` the D x J
nodes, `N` the plan size (NNDFT: `(size(y, 2),)`), `adjoint=true` for the
adjoint / transpose.
"""
function direct_mul!(out::CuArray, kind::Int, k::CuMatrix{T}, N::NTuple{D,Int}, x::CuArray;
                     adjoint::Bool=false, y::Union{Nothing,CuMatrix{T}}=nothing) where {T,D}
  cplx = eltype(x) <: Complex
  Nc = Int64[N...; ones(Int64, 4 - D)]
  yp = y === nothing ? CuPtr{T}(0) : pointer(y)
  check(ccall((:nfft_direct, libnfft[]), Cint,
              (Cint, Cint, Cint, Ptr{Int64}, Int64, CuPtr{T}, CuPtr{T}, Cint, Cint, CuPtr{Cvoid}, CuPtr{Cvoid},
               Ptr{Cvoid}),
              kind, T == Float32 ? 32 : 64, size(k, 1), Nc, size(k, 2), k, yp, adjoint, cplx, x, out,
              CUDA.stream().handle))
  return out
end

Base.show(io::IO, p::GB300NFFTPlan) =
  print(io, "GB300NFFTPlan with ", p.J, " sampling points for an input array of size", p.N,
        " and an output array of size", p.NOut, " with dims ", p.dims)

end # module
