// Node gradient of the forward NFFT (no reference counterpart; the reference
// rrules give NoTangent for k, AbstractNFFTs/ext/AbstractNFFTsChainRulesCoreExt.jl:45,61).
//
// With y_j = sum_taps prod_d phi_d(x_d) g[tap] (x_d = k_d*Ntilde_d - tap_d the
// distance in grid units), dy_j/dk_{d,j} = Ntilde_d * sum_taps phi_d'(x_d)
// prod_{d' != d} phi_{d'}(x_{d'}) g[tap].  The kernel recomputes window values
// and their derivatives per tap (nothing like the sparse matrix B is stored)
// and reads the forward grid g (apodized, padded and transformed image).
// Output: dk[d, j] = Re(conj(w_j) * dy_j/dk_{d,j}).
#include "nfft_internal.cuh"

namespace nfft {
namespace {

constexpr int kGradThreads = 256;

template <typename T> __device__ __forceinline__ T shfl(T v, int src) { return __shfl_sync(0xFFFFFFFFu, v, src); }

// d phi / d x at distance x (grid units) for the exact Kaiser-Bessel and
// Gaussian windows (src/windowFunctions.jl:21-34, :60-68).
template <typename T> __device__ __forceinline__ T window_exact_deriv(int window, T x, int m, T sigma) {
  const T PI = T(3.14159265358979323846);
  const T mm = T(m);
  T ax = x < T(0) ? -x : x;
  if (ax >= mm) return T(0);
  if (window == NFFT_WINDOW_GAUSS) {
    T b = mm / PI;
    return T(1) / sqrt(PI * b) * exp(-(x * x) / b) * (T(-2) * x / b);
  }
  // Kaiser-Bessel: phi = sinh(b s) / (pi s), s = sqrt(m^2 - x^2), ds/dx = -x/s
  T b = PI * (T(2) - T(1) / sigma);
  T s = sqrt(mm * mm - x * x);
  T dphids = (b * cosh(b * s) * s - sinh(b * s)) / (PI * s * s);
  return dphids * (-x / s);
}

// Window value and derivative with respect to the node offset e.
template <typename T>
__device__ __forceinline__ void tap_weight_deriv(const Geom<T>& G, const T* cs, T e, int l, T& w, T& dw) {
  if (G.mode == WIN_POLY || (G.mode == WIN_EXACT && G.window != NFFT_WINDOW_KAISER_BESSEL &&
                             G.window != NFFT_WINDOW_GAUSS)) {
    const int deg = 2 * G.m + 1;
    const T* c = cs + l * deg;
    T t = e - T(0.5);
    T r = c[deg - 1], dr = T(0);
    for (int i = deg - 2; i >= 0; --i) {
      dr = fma(dr, t, r);
      r = fma(r, t, c[i]);
    }
    w = (G.mode == WIN_POLY) ? r : window_exact<T>(G.window, e + T(G.m - 1 - l), G.m, G.sigma);
    dw = dr;
  } else if (G.mode == WIN_LINEAR) {
    T x = e + T(G.m - 1 - l);
    T sgn = x < T(0) ? T(-1) : T(1);
    T u = (x < T(0) ? -x : x) * G.lut_scale;
    const T umax = T(G.m) * G.lut_scale;
    if (u > umax) u = umax;
    T fi = floor(u);
    int i = int(fi);
    T a = u - fi;
    T v0 = __ldg(G.lut + i), v1 = __ldg(G.lut + i + 1);
    w = v0 + a * (v1 - v0);
    dw = (v1 - v0) * G.lut_scale * sgn;
  } else {
    T x = e + T(G.m - 1 - l);
    w = window_exact<T>(G.window, x, G.m, G.sigma);
    dw = window_exact_deriv<T>(G.window, x, G.m, G.sigma);
  }
}

template <int L, int D, typename T> __device__ __forceinline__ T wsel(T W0, T W1, int q) {
  if (D * L <= 32) return shfl(W0, q & 31);
  T a = shfl(W0, q & 31);
  T b = shfl(W1, q & 31);
  return q < 32 ? a : b;
}

template <int D, int L, typename T>
__global__ void __launch_bounds__(kGradThreads) grad_nodes_kernel(Geom<T> G, Nodes<T> Nd,
                                                                   const typename Cplx<T>::type* __restrict__ g,
                                                                   const typename Cplx<T>::type* __restrict__ wv,
                                                                   T* __restrict__ dk) {
  using C = typename Cplx<T>::type;
  constexpr int RY = (D == 1) ? 1 : (32 / L);
  constexpr int NSTEP = (D == 1) ? 1 : (L + RY - 1) / RY;
  __shared__ T cs[kMaxDeg * kMaxL];
  {
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
    T W0 = 0, W1 = 0, V0 = 0, V1 = 0;  // weights and derivatives
    if (lane < D * L) {
      const int d = lane / L;
      tap_weight_deriv<T>(G, cs, Nd.frac4[4 * i + d], lane - d * L, W0, V0);
    }
    if (D * L > 32 && lane + 32 < D * L) {
      const int q = lane + 32, d = q / L;
      tap_weight_deriv<T>(G, cs, Nd.frac4[4 * i + d], q - d * L, W1, V1);
    }
    const int4 nd = Nd.node4[i];
    const int t[3] = {nd.x, nd.y, nd.z};
    const int gx = G.small_grid ? wrap_any(t[0] + G.sh[0] - m + 1 + ix, G.Nt[0]) : wrap_once(t[0] + G.sh[0] - m + 1 + ix, G.Nt[0]);
    const T wx = wsel<L, D>(W0, W1, ix), dwx = wsel<L, D>(V0, V1, ix);
    T sr[D], si[D];
#pragma unroll
    for (int d = 0; d < D; ++d) sr[d] = si[d] = T(0);
    if constexpr (D == 1) {
      if (xact) {
        C v = g[gx];
        sr[0] = dwx * v.x;
        si[0] = dwx * v.y;
      }
    } else {
#pragma unroll
      for (int s = 0; s < NSTEP; ++s) {
        const int iy = s * RY + ry;
        const bool ok = xact && iy < L;
        const int iyc = ok ? iy : 0;
        const int gy = G.small_grid ? wrap_any(t[1] + G.sh[1] - m + 1 + iyc, G.Nt[1]) : wrap_once(t[1] + G.sh[1] - m + 1 + iyc, G.Nt[1]);
        const int64_t row = int64_t(gy) * G.Nt[0] + gx;
        // shuffles run on every lane; inactive rows are zeroed afterwards
        const T wy_all = wsel<L, D>(W0, W1, L + iyc);
        const T dwy_all = wsel<L, D>(V0, V1, L + iyc);
        const T wy = ok ? wy_all : T(0);
        const T dwy = ok ? dwy_all : T(0);
        if constexpr (D == 2) {
          C v = g[row];
          const T a = dwx * wy, b = wx * dwy;
          sr[0] += a * v.x; si[0] += a * v.y;
          sr[1] += b * v.x; si[1] += b * v.y;
        } else {
          for (int iz = 0; iz < L; ++iz) {
            const T wz = wsel<L, D>(W0, W1, 2 * L + iz), dwz = wsel<L, D>(V0, V1, 2 * L + iz);
            const int gz = G.small_grid ? wrap_any(t[2] + G.sh[2] - m + 1 + iz, G.Nt[2]) : wrap_once(t[2] + G.sh[2] - m + 1 + iz, G.Nt[2]);
            C v = g[int64_t(gz) * G.plane + row];
            const T a = dwx * wy * wz, b = wx * dwy * wz, c = wx * wy * dwz;
            sr[0] += a * v.x; si[0] += a * v.y;
            sr[1] += b * v.x; si[1] += b * v.y;
            sr[2] += c * v.x; si[2] += c * v.y;
          }
        }
      }
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        sr[d] += __shfl_xor_sync(0xFFFFFFFFu, sr[d], o);
        si[d] += __shfl_xor_sync(0xFFFFFFFFu, si[d], o);
      }
    }
    if (lane == 0) {
      const int64_t j = nd.w;
      const C w = wv[j];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        // Re(conj(w) * Ntilde_d * S_d)
        dk[int64_t(d) + int64_t(D) * j] = T(G.Nt[d]) * (w.x * sr[d] + w.y * si[d]);
      }
    }
  }
}

template <int D, int L, typename T> int grad_c(const nfft_plan* p, const void* g, const void* w, void* dk) {
  Geom<T> G = make_geom<T>(p);
  Nodes<T> Nd = make_nodes<T>(p);
  if (Nd.M == 0) return NFFT_OK;
  using C = typename Cplx<T>::type;
  int64_t blocks = (Nd.M + 7) / 8;
  if (blocks > 152 * 64) blocks = 152 * 64;
  grad_nodes_kernel<D, L, T><<<unsigned(blocks), kGradThreads, 0, p->stream>>>(
      G, Nd, static_cast<const C*>(g), static_cast<const C*>(w), static_cast<T*>(dk));
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

template <int D, typename T> int grad_l(const nfft_plan* p, const void* g, const void* w, void* dk) {
  switch (p->m) {
    case 2: return grad_c<D, 4, T>(p, g, w, dk);
    case 3: return grad_c<D, 6, T>(p, g, w, dk);
    case 4: return grad_c<D, 8, T>(p, g, w, dk);
    case 5: return grad_c<D, 10, T>(p, g, w, dk);
    case 6: return grad_c<D, 12, T>(p, g, w, dk);
    case 7: return grad_c<D, 14, T>(p, g, w, dk);
    case 8: return grad_c<D, 16, T>(p, g, w, dk);
  }
  set_error("m = %d not supported (2..8)", p->m);
  return NFFT_ERR_UNSUPPORTED;
}

template <typename T> int grad_d(const nfft_plan* p, const void* g, const void* w, void* dk) {
  switch (p->D) {
    case 1: return grad_l<1, T>(p, g, w, dk);
    case 2: return grad_l<2, T>(p, g, w, dk);
    case 3: return grad_l<3, T>(p, g, w, dk);
  }
  return NFFT_ERR_UNSUPPORTED;
}

}  // namespace

int launch_grad_nodes(const nfft_plan* p, const void* g, const void* w, void* dk) {
  return p->precision == 32 ? grad_d<float>(p, g, w, dk) : grad_d<double>(p, g, w, dk);
}

}  // namespace nfft
