"""
ChainRules for the GB300 backend: the rules of
AbstractNFFTs/ext/AbstractNFFTsChainRulesCoreExt.jl:31-61 for device
arrays, with the node gradient the reference leaves as NoTangent (:45, :61)
computed by the library's ∂k kernel (`nfft_grad_nodes`), which recomputes the
window and its derivative per tap instead of storing the sparse matrix B.

For a real loss L and complex cotangents (ChainRules' convention
ȳ = ∂L/∂Re y + i ∂L/∂Im y):
  y = nfft(k, x):            x̄ = nfft_adjoint(k, N, ȳ),
                             k̄[d, j] = Re(conj(ȳ[j]) ∂(A x)_j/∂k[d, j]);
  y = nfft_adjoint(k, N, x): x̄ = nfft(k, ȳ),
                             k̄[d, j] = Re(conj(x[j]) ∂(A ȳ)_j/∂k[d, j]).
"""
module NFFTGB300ChainRulesCoreExt

using NFFTGB300
using AbstractNFFTs
using CUDA
import ChainRulesCore

function ChainRulesCore.rrule(::typeof(AbstractNFFTs.nfft), k::AbstractMatrix{T},
                              x::CuArray{Complex{T},D}) where {T<:Union{Float32,Float64},D}
  kk = Matrix{T}(k)
  p = AbstractNFFTs.plan_nfft(NFFTGB300.GB300Backend(), CuArray, kk, size(x))
  y = p * x
  project_x = ChainRulesCore.ProjectTo(x)
  project_k = ChainRulesCore.ProjectTo(k)
  function nfft_pullback(ȳ)
    ȳc = CuArray{Complex{T}}(ChainRulesCore.unthunk(ȳ))
    x̄ = project_x(adjoint(p) * ȳc)
    dk = CUDA.zeros(T, size(kk))
    NFFTGB300.grad_nodes!(dk, p, x, ȳc)
    return ChainRulesCore.NoTangent(), project_k(Array(dk)), x̄
  end
  return y, nfft_pullback
end

function ChainRulesCore.rrule(::typeof(AbstractNFFTs.nfft_adjoint), k::AbstractMatrix{T}, N,
                              x::CuVector{Complex{T}}) where {T<:Union{Float32,Float64}}
  kk = Matrix{T}(k)
  p = AbstractNFFTs.plan_nfft(NFFTGB300.GB300Backend(), CuArray, kk, Tuple(N))
  y = adjoint(p) * x
  project_x = ChainRulesCore.ProjectTo(x)
  project_k = ChainRulesCore.ProjectTo(k)
  function nfft_adjoint_pullback(ȳ)
    ȳc = CuArray{Complex{T}}(ChainRulesCore.unthunk(ȳ))
    x̄ = project_x(p * ȳc)
    dk = CUDA.zeros(T, size(kk))
    NFFTGB300.grad_nodes!(dk, p, ȳc, x)
    return ChainRulesCore.NoTangent(), project_k(Array(dk)), ChainRulesCore.NoTangent(), x̄
  end
  return y, nfft_adjoint_pullback
end

end # module
