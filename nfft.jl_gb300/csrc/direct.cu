// Direct (exact) transforms of src/direct.jl on the device:
//   NDFT   (:99-151)  fHat_j = sum_l f_l e^{-2 pi i k_j . n_l},  n_l = idx - N div 2
//   NDCT   (:153-199) fHat_j = sum_l f_l prod_d cos(2 pi k_dj n_dl), n = idx (0-based)
//   NDST   (:202-249) fHat_j = sum_l f_l prod_d sin(2 pi k_dj n_dl), n = idx + 1 (image N - 1)
//   NNDFT  (:252-287) fHat_j = sum_l f_l e^{-2 pi i k_j . y_l}
// and their adjoints / transposes (sign +, sums over the nodes).  O(M |N|)
// work: these are the exact references a user checks a fast plan against.
//
// GB300 form: one thread per output (node for the forward direction, image
// point for the adjoint); the inputs stream through shared memory in chunks
// of 256 (coordinates and values as FP64), phases by sincospi / cospi /
// sinpi in FP64 (exact argument reduction), sums in FP64.  When the outputs
// alone give too few CTAs to fill the GPU, the input range is split over
// blockIdx.y and the FP64 partial sums are added in a second, deterministic
// pass.
#include "nfft_internal.cuh"

namespace nfft {
namespace {

constexpr int kDirThreads = 256;
constexpr int kDirChunk = 256;
constexpr int kDirMaxD = 4;

struct DirGeom {
  int kind, D, adj, cplx;
  int64_t n_img, M;
  int64_t ext[kDirMaxD];  // image extents (NDST: N_d - 1; NNDFT: unused)
  int64_t off[kDirMaxD];  // coordinate of image index 0 along d
};

template <typename T>
__device__ __forceinline__ void image_coords(const DirGeom& G, const T* __restrict__ y, int64_t l,
                                             double (&c)[kDirMaxD]) {
#pragma unroll
  for (int d = 0; d < kDirMaxD; ++d) c[d] = 0.0;
  if (G.kind == NFFT_NNDFT) {
    for (int d = 0; d < G.D; ++d) c[d] = double(y[l * G.D + d]);
  } else {
    int64_t r = l;
    for (int d = 0; d < G.D; ++d) {
      const int64_t e = G.ext[d];
      const int64_t i = r % e;
      r /= e;
      c[d] = double(i + G.off[d]);
    }
  }
}

// kernel entry between node coordinates a and image coordinates b
__device__ __forceinline__ void entry(const DirGeom& G, const double (&a)[kDirMaxD], const double* b, int bstride,
                                      double& wr, double& wi) {
  if (G.kind == NFFT_NDFT || G.kind == NFFT_NNDFT) {
    double s = 0.0;
#pragma unroll
    for (int d = 0; d < kDirMaxD; ++d) s = fma(a[d], b[d * bstride], s);
    double sn, cs;
    sincospi(2.0 * s, &sn, &cs);
    wr = cs;
    wi = G.adj ? sn : -sn;
  } else if (G.kind == NFFT_NDCT) {
    double w = 1.0;
    for (int d = 0; d < G.D; ++d) w *= cospi(2.0 * a[d] * b[d * bstride]);
    wr = w;
    wi = 0.0;
  } else {
    double w = 1.0;
    for (int d = 0; d < G.D; ++d) w *= sinpi(2.0 * a[d] * b[d * bstride]);
    wr = w;
    wi = 0.0;
  }
}

// One thread per output; inputs [lo, hi) of split blockIdx.y.  FP64 results
// go to part (split s at part + s * n_out) or, with one split, to out in T.
template <typename T>
__global__ void __launch_bounds__(kDirThreads) direct_kernel(DirGeom G, const T* __restrict__ k,
                                                             const T* __restrict__ y, const T* __restrict__ in,
                                                             double2* __restrict__ part, T* __restrict__ out,
                                                             int64_t n_out, int64_t n_in, int64_t per_split) {
  __shared__ double sc[kDirMaxD][kDirChunk];
  __shared__ double sv[2][kDirChunk];
  const int64_t o = blockIdx.x * int64_t(kDirThreads) + threadIdx.x;
  const int64_t lo = blockIdx.y * per_split;
  const int64_t hi = lo + per_split < n_in ? lo + per_split : n_in;
  double mine[kDirMaxD];
#pragma unroll
  for (int d = 0; d < kDirMaxD; ++d) mine[d] = 0.0;
  if (o < n_out) {
    if (!G.adj) {
      for (int d = 0; d < G.D; ++d) mine[d] = double(k[o * G.D + d]);
    } else {
      image_coords<T>(G, y, o, mine);
    }
  }
  double ar = 0.0, ai = 0.0;
  for (int64_t b0 = lo; b0 < hi; b0 += kDirChunk) {
    const int cnt = int(hi - b0 < kDirChunk ? hi - b0 : kDirChunk);
    __syncthreads();
    for (int t = threadIdx.x; t < cnt; t += kDirThreads) {
      const int64_t b = b0 + t;
      double c[kDirMaxD];
      if (!G.adj) {
        image_coords<T>(G, y, b, c);
      } else {
#pragma unroll
        for (int d = 0; d < kDirMaxD; ++d) c[d] = d < G.D ? double(k[b * G.D + d]) : 0.0;
      }
#pragma unroll
      for (int d = 0; d < kDirMaxD; ++d) sc[d][t] = c[d];
      sv[0][t] = double(G.cplx ? in[2 * b] : in[b]);
      sv[1][t] = G.cplx ? double(in[2 * b + 1]) : 0.0;
    }
    __syncthreads();
    if (o < n_out) {
      for (int e = 0; e < cnt; ++e) {
        double wr, wi;
        if (!G.adj) {
          entry(G, mine, &sc[0][e], kDirChunk, wr, wi);
        } else {
          double a[kDirMaxD];
#pragma unroll
          for (int d = 0; d < kDirMaxD; ++d) a[d] = sc[d][e];
          entry(G, a, mine, 1, wr, wi);
        }
        const double vr = sv[0][e], vi = sv[1][e];
        ar = fma(vr, wr, fma(-vi, wi, ar));
        ai = fma(vr, wi, fma(vi, wr, ai));
      }
    }
  }
  if (o >= n_out) return;
  if (part) {
    part[blockIdx.y * n_out + o] = make_double2(ar, ai);
  } else if (G.cplx) {
    out[2 * o] = T(ar);
    out[2 * o + 1] = T(ai);
  } else {
    out[o] = T(ar);
  }
}

template <typename T>
__global__ void __launch_bounds__(kDirThreads) direct_reduce_kernel(const double2* __restrict__ part, int splits,
                                                                    int64_t n_out, int cplx, T* __restrict__ out) {
  const int64_t o = blockIdx.x * int64_t(kDirThreads) + threadIdx.x;
  if (o >= n_out) return;
  double ar = 0.0, ai = 0.0;
  for (int s = 0; s < splits; ++s) {
    const double2 v = part[s * n_out + o];
    ar += v.x;
    ai += v.y;
  }
  if (cplx) {
    out[2 * o] = T(ar);
    out[2 * o + 1] = T(ai);
  } else {
    out[o] = T(ar);
  }
}

template <typename T>
int run_direct(const DirGeom& G, const void* k, const void* y, const void* in, void* out, cudaStream_t s) {
  const int64_t n_out = G.adj ? G.n_img : G.M;
  const int64_t n_in = G.adj ? G.M : G.n_img;
  if (n_out == 0) return NFFT_OK;
  const int64_t out_ctas = (n_out + kDirThreads - 1) / kDirThreads;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t target = int64_t(sms) * 8;
  int64_t splits = out_ctas >= target ? 1 : (target + out_ctas - 1) / out_ctas;
  const int64_t max_splits = (n_in + kDirChunk - 1) / kDirChunk;
  if (splits > max_splits) splits = max_splits;
  if (splits < 1) splits = 1;
  if (splits > 65535) splits = 65535;
  int64_t per = (n_in + splits - 1) / splits;
  per = (per + kDirChunk - 1) / kDirChunk * kDirChunk;
  if (per < 1) per = kDirChunk;
  splits = (n_in + per - 1) / per;
  if (splits < 1) splits = 1;
  double2* part = nullptr;
  if (splits > 1)
    NFFT_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&part), size_t(splits) * n_out * sizeof(double2), s));
  const dim3 grid{unsigned(out_ctas), unsigned(splits), 1u};
  direct_kernel<T><<<grid, kDirThreads, 0, s>>>(G, static_cast<const T*>(k), static_cast<const T*>(y),
                                                 static_cast<const T*>(in), part, static_cast<T*>(out), n_out,
                                                 n_in, per);
  NFFT_LAUNCH_CHECK();
  if (part) {
    direct_reduce_kernel<T><<<unsigned(out_ctas), kDirThreads, 0, s>>>(part, int(splits), n_out, G.cplx,
                                                                        static_cast<T*>(out));
    NFFT_LAUNCH_CHECK();
    NFFT_CUDA_TRY(cudaFreeAsync(part, s));
  }
  return NFFT_OK;
}

}  // namespace
}  // namespace nfft

using namespace nfft;

extern "C" int nfft_direct(int kind, int precision, int D, const int64_t* N, int64_t M, const void* k, const void* y,
                           int adjoint, int complex_data, const void* in, void* out, void* stream) {
  if (kind < NFFT_NDFT || kind > NFFT_NNDFT) {
    set_error("unknown direct transform kind %d", kind);
    return NFFT_ERR_INVALID_ARG;
  }
  if (precision != 32 && precision != 64) {
    set_error("precision must be 32 or 64");
    return NFFT_ERR_INVALID_ARG;
  }
  if (D < 1 || D > kDirMaxD) {
    set_error("D = %d not supported by the direct transforms (1..%d)", D, kDirMaxD);
    return NFFT_ERR_INVALID_ARG;
  }
  if (!N || M < 0 || (M > 0 && !k)) {
    set_error("null argument or negative node count");
    return NFFT_ERR_INVALID_ARG;
  }
  if ((kind == NFFT_NDFT || kind == NFFT_NNDFT) && !complex_data) {
    set_error("the NDFT and the NNDFT take complex data");
    return NFFT_ERR_INVALID_ARG;
  }
  DirGeom G{};
  G.kind = kind;
  G.D = D;
  G.adj = adjoint ? 1 : 0;
  G.cplx = complex_data ? 1 : 0;
  G.M = M;
  if (kind == NFFT_NNDFT) {
    if (N[0] < 0 || (N[0] > 0 && !y)) {
      set_error("the NNDFT needs its D x N points y");
      return NFFT_ERR_INVALID_ARG;
    }
    G.n_img = N[0];
  } else {
    G.n_img = 1;
    for (int d = 0; d < D; ++d) {
      const int64_t n = N[d];
      const int64_t e = kind == NFFT_NDST ? n - 1 : n;
      if (n < 1 || e < 1) {
        set_error("N[%d] = %lld too small for this transform", d, (long long)n);
        return NFFT_ERR_INVALID_ARG;
      }
      G.ext[d] = e;
      G.off[d] = kind == NFFT_NDFT ? -(n / 2) : (kind == NFFT_NDST ? 1 : 0);
      G.n_img *= e;
    }
  }
  {
    const int64_t n_in = adjoint ? M : G.n_img, n_out = adjoint ? G.n_img : M;
    if ((n_in > 0 && !in) || (n_out > 0 && !out)) {
      set_error("null data pointer");
      return NFFT_ERR_INVALID_ARG;
    }
  }
  if (M == 0 || G.n_img == 0) {
    const int64_t n_out = adjoint ? G.n_img : M;
    const size_t bytes = size_t(n_out) * (precision / 8) * (complex_data ? 2 : 1);
    if (bytes) NFFT_CUDA_TRY(cudaMemsetAsync(out, 0, bytes, static_cast<cudaStream_t>(stream)));
    return NFFT_OK;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return precision == 32 ? run_direct<float>(G, k, y, in, out, s) : run_direct<double>(G, k, y, in, out, s);
}
