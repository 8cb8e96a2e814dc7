// Fast cosine / sine transforms at nonequispaced nodes (the AbstractNFFTs
// NFCT / NFST plan types, AbstractNFFTs/src/interface.jl:73-90; the
// reference computes them only directly, src/direct.jl:153-249, or through
// its NFFT3 wrapper) on this library's NFFT:
//   NFCT  fHat_j = sum_{n in [0,N)} f_n prod_d cos(2 pi k_dj n_d)
//   NFST  fHat_j = sum_{n in [1,N-1]} f_n prod_d sin(2 pi k_dj n_d)   (input N - 1)
// With cos t = (e^{it} + e^{-it})/2 and sin t = (e^{it} - e^{-it})/(2i), both
// are the NFFT, on an image of size 2N, of an even (NFCT) or odd (NFST)
// extension of f:
//   NFCT  F_n = f_|n| prod_d (n_d = 0 ? 1 : 1/2),  |n_d| < N_d;
//   NFST  F_n = f_(|n|-1) prod_d (sign(n_d) i / 2), 1 <= |n_d| < N_d;
// F = 0 elsewhere (n_d = -N_d, and n_d = 0 for the NFST); fHat = Re NFFT(F).
// The transposes fold the adjoint NFFT G (size 2N) of the real node values:
//   NFCT  f_n = 2^-D sum_{s in {+1,-1}^D} Re G_{s n}
//   NFST  f_n = Re[(2i)^-D sum_s (prod_d s_d) G_{s n}].
// Extension, real part and folding are one small kernel each; the NFFT is
// the blocked GB300 plan.
#include "nfft_internal.cuh"

struct nfft_tplan {
  nfft_plan* p = nullptr;     // NFFT plan of size 2N
  int kind = NFFT_NDCT;
  int precision = 32;
  int D = 0;
  int64_t N[3] = {1, 1, 1};   // plan size (NFST input: N - 1)
  int64_t M = 0;
  void* ext = nullptr;        // complex image of size 2N
  void* nodevals = nullptr;   // complex M
};

namespace nfft {
namespace {

template <typename T> using Cx = typename Cplx<T>::type;

struct TGeom {
  int kind, D;
  int N[3];      // plan size per dim
  int E[3];      // real image extent per dim (N, or N - 1 for the NFST)
  int64_t n_ext, n_real;
};

unsigned blocks_of(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return unsigned(b < 1 ? 1 : b);
}

// the extended complex image F (size 2N, NFFT layout: index = n + N) of real f
template <typename T>
__global__ void __launch_bounds__(256) extend_kernel(TGeom G, const T* __restrict__ f, Cx<T>* __restrict__ F) {
  for (int64_t q = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; q < G.n_ext; q += int64_t(gridDim.x) * blockDim.x) {
    int64_t r = q, a = 0, stride = 1;
    bool zero = false;
    int neg = 0, halves = 0;
    for (int d = 0; d < G.D; ++d) {
      const int two = 2 * G.N[d];
      const int n = int(r % two) - G.N[d];
      r /= two;
      int ad = n < 0 ? -n : n;
      if (n == -G.N[d]) zero = true;
      if (G.kind == NFFT_NDST) {
        if (n == 0) zero = true;
        ad -= 1;
        if (n < 0) ++neg;
        ++halves;
      } else if (n != 0) {
        ++halves;
      }
      a += int64_t(ad < 0 ? 0 : ad) * stride;
      stride *= G.E[d];
    }
    Cx<T> v;
    v.x = T(0);
    v.y = T(0);
    if (!zero) {
      const T val = f[a] * T(1.0 / double(1 << halves));
      if (G.kind == NFFT_NDCT) {
        v.x = val;
      } else {
        // prod_d (sign_d i) = (-1)^neg i^D
        const T sv = (neg & 1) ? -val : val;
        switch (G.D & 3) {
          case 1: v.y = sv; break;   // i
          case 2: v.x = -sv; break;  // -1
          case 3: v.y = -sv; break;  // -i
          default: v.x = sv; break;
        }
      }
    }
    F[q] = v;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) real_part_kernel(const Cx<T>* __restrict__ c, T* __restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    out[i] = c[i].x;
}

template <typename T>
__global__ void __launch_bounds__(256) to_complex_kernel(const T* __restrict__ v, Cx<T>* __restrict__ c, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    Cx<T> z;
    z.x = v[i];
    z.y = T(0);
    c[i] = z;
  }
}

// f_n from the adjoint NFFT G of the real node values (see the file comment)
template <typename T>
__global__ void __launch_bounds__(256) fold_kernel(TGeom G, const Cx<T>* __restrict__ Gimg, T* __restrict__ f) {
  for (int64_t q = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; q < G.n_real; q += int64_t(gridDim.x) * blockDim.x) {
    int n[3] = {0, 0, 0};
    int64_t r = q;
    for (int d = 0; d < G.D; ++d) {
      n[d] = int(r % G.E[d]) + (G.kind == NFFT_NDST ? 1 : 0);
      r /= G.E[d];
    }
    double sr = 0.0, si = 0.0;
    const int combos = 1 << G.D;
    for (int s = 0; s < combos; ++s) {
      int64_t idx = 0, stride = 1;
      int neg = 0;
      for (int d = 0; d < G.D; ++d) {
        const bool minus = (s >> d) & 1;
        neg += minus ? 1 : 0;
        idx += int64_t((minus ? -n[d] : n[d]) + G.N[d]) * stride;
        stride *= 2 * G.N[d];
      }
      const Cx<T> v = Gimg[idx];
      const double sign = (G.kind == NFFT_NDST && (neg & 1)) ? -1.0 : 1.0;
      sr += sign * double(v.x);
      si += sign * double(v.y);
    }
    double out = sr;
    if (G.kind == NFFT_NDST) {
      // Re[(-i)^D (sr + i si)]: (-i)^1 = -i, (-i)^2 = -1, (-i)^3 = i
      switch (G.D & 3) {
        case 1: out = si; break;
        case 2: out = -sr; break;
        case 3: out = -si; break;
        default: out = sr; break;
      }
    }
    f[q] = T(out / double(combos));
  }
}

TGeom make_tgeom(const nfft_tplan* q) {
  TGeom G{};
  G.kind = q->kind;
  G.D = q->D;
  G.n_ext = 1;
  G.n_real = 1;
  for (int d = 0; d < 3; ++d) {
    G.N[d] = d < q->D ? int(q->N[d]) : 1;
    G.E[d] = d < q->D ? int(q->kind == NFFT_NDST ? q->N[d] - 1 : q->N[d]) : 1;
  }
  for (int d = 0; d < q->D; ++d) {
    G.n_ext *= 2 * G.N[d];
    G.n_real *= G.E[d];
  }
  return G;
}

template <typename T> int tforward(nfft_tplan* q, const void* f, void* fhat) {
  nfft_plan* p = q->p;
  const TGeom G = make_tgeom(q);
  extend_kernel<T><<<blocks_of(G.n_ext), 256, 0, p->stream>>>(G, static_cast<const T*>(f),
                                                              static_cast<Cx<T>*>(q->ext));
  NFFT_LAUNCH_CHECK();
  if (int rc = nfft_forward(p, q->ext, q->nodevals)) return rc;
  if (q->M > 0) {
    real_part_kernel<T><<<blocks_of(q->M), 256, 0, p->stream>>>(static_cast<const Cx<T>*>(q->nodevals),
                                                                static_cast<T*>(fhat), q->M);
    NFFT_LAUNCH_CHECK();
  }
  return NFFT_OK;
}

template <typename T> int ttranspose(nfft_tplan* q, const void* fhat, void* f) {
  nfft_plan* p = q->p;
  const TGeom G = make_tgeom(q);
  if (q->M > 0) {
    to_complex_kernel<T><<<blocks_of(q->M), 256, 0, p->stream>>>(static_cast<const T*>(fhat),
                                                                 static_cast<Cx<T>*>(q->nodevals), q->M);
    NFFT_LAUNCH_CHECK();
  }
  if (int rc = nfft_adjoint(p, q->nodevals, q->ext)) return rc;
  fold_kernel<T><<<blocks_of(G.n_real), 256, 0, p->stream>>>(G, static_cast<const Cx<T>*>(q->ext),
                                                             static_cast<T*>(f));
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

}  // namespace
}  // namespace nfft

using namespace nfft;

extern "C" {

int nfft_tplan_create(nfft_tplan** out, int kind, int precision, int D, const int64_t* N, int64_t M,
                      const nfft_params* params, void* stream) {
  if (!out || !N || !params) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  *out = nullptr;
  if (kind != NFFT_NDCT && kind != NFFT_NDST) {
    set_error("kind must be NFFT_NDCT (NFCT) or NFFT_NDST (NFST)");
    return NFFT_ERR_INVALID_ARG;
  }
  if (D < 1 || D > 3) {
    set_error("D = %d not supported (1..3)", D);
    return NFFT_ERR_INVALID_ARG;
  }
  for (int d = 0; d < D; ++d)
    if (N[d] < (kind == NFFT_NDST ? 2 : 1) || N[d] > (int64_t(1) << 27)) {
      set_error("N[%d] = %lld out of range", d, (long long)N[d]);
      return NFFT_ERR_INVALID_ARG;
    }
  if (M < 0) {
    set_error("negative node count");
    return NFFT_ERR_INVALID_ARG;
  }
  auto* q = new nfft_tplan();
  q->kind = kind;
  q->precision = precision;
  q->D = D;
  q->M = M;
  int64_t N2[3] = {1, 1, 1};
  int64_t n_ext = 1;
  for (int d = 0; d < D; ++d) {
    q->N[d] = N[d];
    N2[d] = 2 * N[d];
    n_ext *= N2[d];
  }
  int rc = nfft_plan_create(&q->p, precision, D, N2, M, params, stream);
  const size_t cs = size_t(precision / 4);
  if (!rc && cudaMalloc(&q->ext, size_t(n_ext) * cs) != cudaSuccess) {
    set_error("cudaMalloc of the extended image failed");
    rc = NFFT_ERR_ALLOC;
  }
  if (!rc && cudaMalloc(&q->nodevals, size_t(M > 0 ? M : 1) * cs) != cudaSuccess) {
    set_error("cudaMalloc of the node values failed");
    rc = NFFT_ERR_ALLOC;
  }
  if (rc) {
    nfft_tplan_destroy(q);
    return rc;
  }
  *out = q;
  return NFFT_OK;
}

int nfft_tplan_destroy(nfft_tplan* q) {
  if (!q) return NFFT_OK;
  cudaFree(q->ext);
  cudaFree(q->nodevals);
  nfft_plan_destroy(q->p);
  delete q;
  return NFFT_OK;
}

int nfft_tplan_set_stream(nfft_tplan* q, void* stream) {
  if (!q) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  return nfft_set_stream(q->p, stream);
}

int nfft_tplan_set_nodes(nfft_tplan* q, const void* k, int k_on_device) {
  if (!q) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  return nfft_set_nodes(q->p, k, k_on_device);
}

int nfft_tplan_forward(nfft_tplan* q, const void* f, void* fhat) {
  if (!q || !f || (!fhat && q->M > 0)) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  return q->precision == 32 ? tforward<float>(q, f, fhat) : tforward<double>(q, f, fhat);
}

int nfft_tplan_transpose(nfft_tplan* q, const void* fhat, void* f) {
  if (!q || !f || (!fhat && q->M > 0)) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  return q->precision == 32 ? ttranspose<float>(q, fhat, f) : ttranspose<double>(q, fhat, f);
}

}  // extern "C"
