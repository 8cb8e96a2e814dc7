// Gather interpolation (convolve!): fHat[j] = sum over the (2m)^D window taps
// of prod_d phi_d * g[tap], src/convolution.jl:229-344 (blocked) and :56-99.
//
// One warp per node, nodes visited in bin-sorted order so that the warps of a
// CTA (and the CTAs resident on an SM) read overlapping grid neighbourhoods
// through L1/L2.  Lane layout: lane = ix + L*ry, ix the tap along dimension 1
// (contiguous grid addresses), ry a row slot; rows (taps along dimensions 2
// and 3) are stepped in groups of 32/L.  The D*2m window values are computed
// once per node, one per lane (Horner on the fitted polynomial, LUT or the
// window function), and exchanged with warp shuffles.
#include "nfft_internal.cuh"

namespace nfft {
namespace {

constexpr int kInterpThreads = 256;

template <typename T> __device__ __forceinline__ T shfl(T v, int src) { return __shfl_sync(0xFFFFFFFFu, v, src); }

// weight q of the node, q = d*L + l; lanes hold q (W0) and q+32 (W1)
template <int L, int D, typename T> __device__ __forceinline__ T wsel(T W0, T W1, int q) {
  if (D * L <= 32) return shfl(W0, q & 31);
  T a = shfl(W0, q & 31);
  T b = shfl(W1, q & 31);
  return q < 32 ? a : b;
}

template <typename T, int CG> struct GridVal;
template <typename T> struct GridVal<T, 2> {  // interleaved complex grid
  static __device__ __forceinline__ void load(const T* g, int64_t idx, T& re, T& im) {
    using C = typename Cplx<T>::type;
    C v = __ldg(reinterpret_cast<const C*>(g) + idx);
    re = v.x;
    im = v.y;
  }
};

template <int D, int L, typename T>
__global__ void __launch_bounds__(kInterpThreads) interp_warp_kernel(Geom<T> G, Nodes<T> Nd,
                                                                      const T* __restrict__ g,
                                                                      T* __restrict__ fhat) {
  constexpr int RY = (D == 1) ? 1 : (32 / L);           // rows per step
  constexpr int NSTEP = (D == 1) ? 1 : (L + RY - 1) / RY;  // steps over dimension-2 taps
  __shared__ T cs[kMaxDeg * kMaxL];
  if (G.mode == WIN_POLY) {
    const int n = (2 * G.m + 1) * L;
    for (int q = threadIdx.x; q < n; q += blockDim.x) cs[q] = G.coeffs[q];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int ix = lane % L;
  const int ry = lane / L;
  const bool xact = (D == 1) ? (lane < L) : (ry < RY);
  const int64_t warps_total = int64_t(gridDim.x) * (blockDim.x >> 5);
  const int m = G.m;
  for (int64_t i = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); i < Nd.M; i += warps_total) {
    // window values: lane q -> (d = q / L, l = q % L)
    T W0 = T(0), W1 = T(0);
    {
      const int q0 = lane;
      if (q0 < D * L) {
        const int d = q0 / L;
        W0 = tap_weight<T>(G, cs, Nd.te[int64_t(d) * Nd.M + i], q0 - d * L);
      }
      if (D * L > 32) {
        const int q1 = lane + 32;
        if (q1 < D * L) {
          const int d = q1 / L;
          W1 = tap_weight<T>(G, cs, Nd.te[int64_t(d) * Nd.M + i], q1 - d * L);
        }
      }
    }
    int t[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d) t[d] = Nd.ti[int64_t(d) * Nd.M + i];
    const int gx = G.small_grid ? wrap_any(t[0] - m + 1 + ix, G.Nt[0]) : wrap_once(t[0] - m + 1 + ix, G.Nt[0]);
    const T wx = wsel<L, D>(W0, W1, ix);
    T ar = T(0), ai = T(0);
    if constexpr (D == 1) {
      if (xact) {
        T vr, vi;
        GridVal<T, 2>::load(g, gx, vr, vi);
        ar = wx * vr;
        ai = wx * vi;
      }
    } else {
      int64_t rowoff[NSTEP];
      T wxy[NSTEP];
#pragma unroll
      for (int s = 0; s < NSTEP; ++s) {
        const int iy = s * RY + ry;
        const bool ok = xact && iy < L;
        const int iyc = ok ? iy : 0;
        const int gy = G.small_grid ? wrap_any(t[1] - m + 1 + iyc, G.Nt[1]) : wrap_once(t[1] - m + 1 + iyc, G.Nt[1]);
        rowoff[s] = int64_t(gy) * G.Nt[0] + gx;
        const T wy = wsel<L, D>(W0, W1, L + iyc);
        wxy[s] = ok ? wx * wy : T(0);
      }
      if constexpr (D == 2) {
#pragma unroll
        for (int s = 0; s < NSTEP; ++s) {
          T vr, vi;
          GridVal<T, 2>::load(g, rowoff[s], vr, vi);
          ar = fma(wxy[s], vr, ar);
          ai = fma(wxy[s], vi, ai);
        }
      } else {
#pragma unroll
        for (int iz = 0; iz < L; ++iz) {
          const T wz = wsel<L, D>(W0, W1, 2 * L + iz);
          const int gz = G.small_grid ? wrap_any(t[2] - m + 1 + iz, G.Nt[2]) : wrap_once(t[2] - m + 1 + iz, G.Nt[2]);
          const int64_t pz = int64_t(gz) * G.plane;
#pragma unroll
          for (int s = 0; s < NSTEP; ++s) {
            T vr, vi;
            GridVal<T, 2>::load(g, pz + rowoff[s], vr, vi);
            const T w = wxy[s] * wz;
            ar = fma(w, vr, ar);
            ai = fma(w, vi, ai);
          }
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ar += __shfl_xor_sync(0xFFFFFFFFu, ar, o);
      ai += __shfl_xor_sync(0xFFFFFFFFu, ai, o);
    }
    if (lane == 0) {
      const int64_t j = Nd.perm[i];
      fhat[2 * j] = ar;
      fhat[2 * j + 1] = ai;
    }
  }
}

template <int D, int L, typename T>
int interp_dispatch_c(const nfft_plan* p, const void* g, int, void* fhat, int) {
  Geom<T> G = make_geom<T>(p);
  Nodes<T> Nd = make_nodes<T>(p);
  if (Nd.M == 0) return NFFT_OK;
  const int64_t warps = Nd.M;
  int64_t blocks = (warps + (kInterpThreads / 32) - 1) / (kInterpThreads / 32);
  const int64_t cap = 152 * 64;
  if (blocks > cap) blocks = cap;
  const T* gp = static_cast<const T*>(g);
  T* fp = static_cast<T*>(fhat);
  interp_warp_kernel<D, L, T><<<unsigned(blocks), kInterpThreads, 0, p->stream>>>(G, Nd, gp, fp);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

template <int D, typename T>
int interp_dispatch_l(const nfft_plan* p, const void* g, int g_real, void* fhat, int fhat_real) {
  switch (p->m) {
    case 2: return interp_dispatch_c<D, 4, T>(p, g, g_real, fhat, fhat_real);
    case 3: return interp_dispatch_c<D, 6, T>(p, g, g_real, fhat, fhat_real);
    case 4: return interp_dispatch_c<D, 8, T>(p, g, g_real, fhat, fhat_real);
    case 5: return interp_dispatch_c<D, 10, T>(p, g, g_real, fhat, fhat_real);
    case 6: return interp_dispatch_c<D, 12, T>(p, g, g_real, fhat, fhat_real);
    case 7: return interp_dispatch_c<D, 14, T>(p, g, g_real, fhat, fhat_real);
    case 8: return interp_dispatch_c<D, 16, T>(p, g, g_real, fhat, fhat_real);
  }
  set_error("m = %d not supported (2..8)", p->m);
  return NFFT_ERR_UNSUPPORTED;
}

template <typename T> int interp_dispatch(const nfft_plan* p, const void* g, int g_real, void* fhat, int fhat_real) {
  switch (p->D) {
    case 1: return interp_dispatch_l<1, T>(p, g, g_real, fhat, fhat_real);
    case 2: return interp_dispatch_l<2, T>(p, g, g_real, fhat, fhat_real);
    case 3: return interp_dispatch_l<3, T>(p, g, g_real, fhat, fhat_real);
  }
  return NFFT_ERR_UNSUPPORTED;
}

}  // namespace

int launch_interp(const nfft_plan* p, const void* g, int g_real, void* fhat, int fhat_real) {
  return p->precision == 32 ? interp_dispatch<float>(p, g, g_real, fhat, fhat_real)
                            : interp_dispatch<double>(p, g, g_real, fhat, fhat_real);
}

}  // namespace nfft
