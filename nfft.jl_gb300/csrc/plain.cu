// The plain path (blocking = 0): one thread per node in input order, window
// values computed on the fly, gather straight from global memory and
// spreading with global atomics into a zeroed grid.  It restates NFFT.jl's
// non-blocking convolution (convolve_nonblocking!, src/convolution.jl:56-99;
// _convolve_transpose_nonblocking!, :164-212) and is the straightforward
// FP64 GPU comparator of the bin-sorted tiled kernels.
#include "nfft_internal.cuh"

namespace nfft {
namespace {

// Per-node setup shared by both kernels: grid indices and window values.
template <int D, typename T>
__device__ __forceinline__ void plain_setup(const Geom<T>& G, const T* cs, const T* k, int64_t j, int L,
                                            int idx[3][kMaxL], T w[3][kMaxL]) {
  for (int d = 0; d < D; ++d) {
    int t;
    T e;
    reduce_coord<T>(k[d + int64_t(D) * j], G.Nt[d], t, e);
    for (int l = 0; l < L; ++l) {
      idx[d][l] = wrap_any(t + G.sh[d] - G.m + 1 + l, G.Nt[d]);
      w[d][l] = tap_weight<T>(G, cs, e, l);
    }
  }
}

template <int D, typename T>
__global__ void __launch_bounds__(128) plain_interp_kernel(Geom<T> G, const T* __restrict__ k,
                                                           const T* __restrict__ g, T* __restrict__ fhat) {
  __shared__ T cs[kMaxDeg * kMaxL];
  const int L = 2 * G.m;
  if (G.mode == WIN_POLY) {
    for (int q = threadIdx.x; q < (2 * G.m + 1) * L; q += blockDim.x) cs[q] = G.coeffs[q];
  }
  __syncthreads();
  const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= G.M) return;
  int idx[3][kMaxL];
  T w[3][kMaxL];
  plain_setup<D, T>(G, cs, k, j, L, idx, w);
  T ar = 0, ai = 0;
  const int L1 = D > 1 ? L : 1, L2 = D > 2 ? L : 1;
  for (int c = 0; c < L2; ++c) {
    const T wz = D > 2 ? w[D > 2 ? 2 : 0][c] : T(1);
    const int64_t pz = D > 2 ? int64_t(idx[D > 2 ? 2 : 0][c]) * G.plane : 0;
    for (int b = 0; b < L1; ++b) {
      const T wyz = D > 1 ? wz * w[D > 1 ? 1 : 0][b] : wz;
      const int64_t py = pz + (D > 1 ? int64_t(idx[D > 1 ? 1 : 0][b]) * G.Nt[0] : 0);
      for (int a = 0; a < L; ++a) {
        const int64_t gi = py + idx[0][a];
        const T ww = wyz * w[0][a];
        ar += ww * g[2 * gi];
        ai += ww * g[2 * gi + 1];
      }
    }
  }
  fhat[2 * j] = ar;
  fhat[2 * j + 1] = ai;
}

template <int D, typename T>
__global__ void __launch_bounds__(128) plain_spread_kernel(Geom<T> G, const T* __restrict__ k,
                                                           const T* __restrict__ fhat, T* __restrict__ g) {
  __shared__ T cs[kMaxDeg * kMaxL];
  const int L = 2 * G.m;
  if (G.mode == WIN_POLY) {
    for (int q = threadIdx.x; q < (2 * G.m + 1) * L; q += blockDim.x) cs[q] = G.coeffs[q];
  }
  __syncthreads();
  const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= G.M) return;
  int idx[3][kMaxL];
  T w[3][kMaxL];
  plain_setup<D, T>(G, cs, k, j, L, idx, w);
  const T fr = fhat[2 * j], fi = fhat[2 * j + 1];
  const int L1 = D > 1 ? L : 1, L2 = D > 2 ? L : 1;
  for (int c = 0; c < L2; ++c) {
    const T wz = D > 2 ? w[D > 2 ? 2 : 0][c] : T(1);
    const int64_t pz = D > 2 ? int64_t(idx[D > 2 ? 2 : 0][c]) * G.plane : 0;
    for (int b = 0; b < L1; ++b) {
      const T wyz = D > 1 ? wz * w[D > 1 ? 1 : 0][b] : wz;
      const int64_t py = pz + (D > 1 ? int64_t(idx[D > 1 ? 1 : 0][b]) * G.Nt[0] : 0);
      for (int a = 0; a < L; ++a) {
        const int64_t gi = py + idx[0][a];
        const T ww = wyz * w[0][a];
        atomicAdd(g + 2 * gi, ww * fr);
        atomicAdd(g + 2 * gi + 1, ww * fi);
      }
    }
  }
}

template <typename T> int plain_interp_t(const nfft_plan* p, const void* g, void* fhat) {
  Geom<T> G = make_geom<T>(p);
  if (G.M == 0) return NFFT_OK;
  const unsigned nb = unsigned((G.M + 127) / 128);
  const T* k = static_cast<const T*>(p->k);
  const T* gp = static_cast<const T*>(g);
  T* fp = static_cast<T*>(fhat);
  switch (p->D) {
    case 1: plain_interp_kernel<1, T><<<nb, 128, 0, p->stream>>>(G, k, gp, fp); break;
    case 2: plain_interp_kernel<2, T><<<nb, 128, 0, p->stream>>>(G, k, gp, fp); break;
    default: plain_interp_kernel<3, T><<<nb, 128, 0, p->stream>>>(G, k, gp, fp); break;
  }
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

template <typename T> int plain_spread_t(const nfft_plan* p, const void* fhat, void* g) {
  Geom<T> G = make_geom<T>(p);
  const size_t gbytes = size_t(p->Nt[0] * p->Nt[1] * p->Nt[2]) * sizeof(T) * 2;
  NFFT_CUDA_TRY(cudaMemsetAsync(g, 0, gbytes, p->stream));
  if (G.M == 0) return NFFT_OK;
  const unsigned nb = unsigned((G.M + 127) / 128);
  const T* k = static_cast<const T*>(p->k);
  const T* fp = static_cast<const T*>(fhat);
  T* gp = static_cast<T*>(g);
  switch (p->D) {
    case 1: plain_spread_kernel<1, T><<<nb, 128, 0, p->stream>>>(G, k, fp, gp); break;
    case 2: plain_spread_kernel<2, T><<<nb, 128, 0, p->stream>>>(G, k, fp, gp); break;
    default: plain_spread_kernel<3, T><<<nb, 128, 0, p->stream>>>(G, k, fp, gp); break;
  }
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

}  // namespace

int launch_plain_interp(const nfft_plan* p, const void* g, int, void* fhat, int) {
  return p->precision == 32 ? plain_interp_t<float>(p, g, fhat) : plain_interp_t<double>(p, g, fhat);
}

int launch_plain_spread(const nfft_plan* p, const void* fhat, int, void* g, int) {
  return p->precision == 32 ? plain_spread_t<float>(p, fhat, g) : plain_spread_t<double>(p, fhat, g);
}

}  // namespace nfft
