// Fast NNFFT, nonequispaced in both domains (the transform of NNDFTPlan,
// src/direct.jl:252-287; AbstractNNFFTPlan, AbstractNFFTs/src/interface.jl):
//   fHat_j = sum_l c_l exp(-2 pi i k_j . y_l),  k_j in [-1/2, 1/2)^D, y_l anywhere.
// Computed with two plans of this library (the method of Elbel and Steidl):
//   1. spread c at u_l = y_l / N1 (convolve_transpose! of a plan P1 of size N1)
//      onto its oversampled grid of Ntilde1 = sigma N1 points, with
//      N1_d = 2 ceil(max |y_d| + m / sigma) + 2 so that no window wraps around;
//   2. the grid in centred order is the image of a plan P2 of size Ntilde1:
//      its forward NFFT at the nodes k_j / sigma1 (sigma1 = Ntilde1 / N1) gives
//      F(k_j) = sum_n G_n exp(-2 pi i n k_j / sigma1)
//             ~ phi-hat_1(k_j N1) sum_l c_l exp(-2 pi i k_j . y_l)
//      (Poisson summation; phi-hat_1 is P1's window transform, product over d);
//   3. fHat_j = F(k_j) / phi-hat_1(k_j N1).
// The adjoint runs the same steps backwards: scale by 1 / phi-hat_1, adjoint
// NFFT of P2, back to grid order, gather (convolve!) of P1 at u.  The error
// is that of an NFFT with the plans' m and sigma on both sides.
#include "nfft_internal.cuh"

#include <cmath>
#include <cstring>
#include <vector>

struct nfft_nnplan {
  int precision = 32;
  int D = 0;
  int64_t M = 0, Ny = 0;
  nfft_params prm{};
  cudaStream_t stream = nullptr;
  nfft_plan* p1 = nullptr;   // size N1, nodes y / N1
  nfft_plan* p2 = nullptr;   // size Ntilde1, nodes k / sigma1
  int64_t N1[3] = {1, 1, 1};
  int64_t Nt1[3] = {1, 1, 1};
  void* img = nullptr;       // P2's image (Ntilde1 complex)
  void* invhat = nullptr;    // 1 / phi-hat_1(k_j N1), M reals (T)
  void* tmp = nullptr;       // M complex
  bool has_nodes = false;
};

namespace nfft {
namespace {

template <typename T> using Cx = typename Cplx<T>::type;

unsigned nn_blocks(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return unsigned(b < 1 ? 1 : b);
}

// dst = src shifted by half the (even) extent along every dimension: grid
// order <-> centred image order (its own inverse)
template <typename T>
__global__ void __launch_bounds__(256) half_shift_kernel(int n0, int n1, int n2, const Cx<T>* __restrict__ src,
                                                         Cx<T>* __restrict__ dst) {
  const int64_t total = int64_t(n0) * n1 * n2;
  for (int64_t q = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; q < total; q += int64_t(gridDim.x) * blockDim.x) {
    int x = int(q % n0);
    const int64_t r = q / n0;
    int y = int(r % n1), z = int(r / n1);
    x = x + n0 / 2 >= n0 ? x + n0 / 2 - n0 : x + n0 / 2;
    y = n1 > 1 ? (y + n1 / 2 >= n1 ? y + n1 / 2 - n1 : y + n1 / 2) : y;
    z = n2 > 1 ? (z + n2 / 2 >= n2 ? z + n2 / 2 - n2 : z + n2 / 2) : z;
    dst[q] = src[x + int64_t(n0) * (y + int64_t(n1) * z)];
  }
}

template <typename T>
__global__ void __launch_bounds__(256) scale_kernel(const Cx<T>* __restrict__ in, const T* __restrict__ s,
                                                    Cx<T>* __restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    Cx<T> v = in[i];
    const T w = s[i];
    v.x *= w;
    v.y *= w;
    out[i] = v;
  }
}

template <typename T> int nn_forward(nfft_nnplan* q, const void* c, void* f) {
  nfft_plan* p1 = q->p1;
  if (int rc = nfft_convolve_transpose(p1, c, 0, p1->grid, 0)) return rc;
  half_shift_kernel<T><<<nn_blocks(p1->Nt[0] * p1->Nt[1] * p1->Nt[2]), 256, 0, q->stream>>>(
      int(p1->Nt[0]), int(p1->Nt[1]), int(p1->Nt[2]), static_cast<const Cx<T>*>(p1->grid), static_cast<Cx<T>*>(q->img));
  NFFT_LAUNCH_CHECK();
  if (int rc = nfft_forward(q->p2, q->img, f)) return rc;
  if (q->M > 0) {
    scale_kernel<T><<<nn_blocks(q->M), 256, 0, q->stream>>>(static_cast<const Cx<T>*>(f),
                                                           static_cast<const T*>(q->invhat), static_cast<Cx<T>*>(f),
                                                           q->M);
    NFFT_LAUNCH_CHECK();
  }
  return NFFT_OK;
}

template <typename T> int nn_adjoint(nfft_nnplan* q, const void* f, void* c) {
  nfft_plan* p1 = q->p1;
  if (q->M > 0) {
    scale_kernel<T><<<nn_blocks(q->M), 256, 0, q->stream>>>(static_cast<const Cx<T>*>(f),
                                                           static_cast<const T*>(q->invhat),
                                                           static_cast<Cx<T>*>(q->tmp), q->M);
    NFFT_LAUNCH_CHECK();
  }
  if (int rc = nfft_adjoint(q->p2, q->tmp, q->img)) return rc;
  half_shift_kernel<T><<<nn_blocks(p1->Nt[0] * p1->Nt[1] * p1->Nt[2]), 256, 0, q->stream>>>(
      int(p1->Nt[0]), int(p1->Nt[1]), int(p1->Nt[2]), static_cast<const Cx<T>*>(q->img), static_cast<Cx<T>*>(p1->grid));
  NFFT_LAUNCH_CHECK();
  return nfft_convolve(p1, p1->grid, 0, c, 0);
}

void free_plans(nfft_nnplan* q) {
  nfft_plan_destroy(q->p1);
  nfft_plan_destroy(q->p2);
  q->p1 = q->p2 = nullptr;
  cudaFree(q->img);
  cudaFree(q->invhat);
  cudaFree(q->tmp);
  q->img = q->invhat = q->tmp = nullptr;
}

}  // namespace
}  // namespace nfft

using namespace nfft;

extern "C" {

int nfft_nnplan_create(nfft_nnplan** out, int precision, int D, int64_t M, int64_t Ny, const nfft_params* params,
                       void* stream) {
  if (!out || !params) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  *out = nullptr;
  if (precision != 32 && precision != 64) {
    set_error("precision must be 32 or 64");
    return NFFT_ERR_INVALID_ARG;
  }
  if (D < 1 || D > 3 || M < 0 || Ny < 0) {
    set_error("D = %d, M = %lld, N = %lld not supported", D, (long long)M, (long long)Ny);
    return NFFT_ERR_INVALID_ARG;
  }
  auto* q = new nfft_nnplan();
  q->precision = precision;
  q->D = D;
  q->M = M;
  q->Ny = Ny;
  q->prm = *params;
  q->prm.compensated = 0;
  q->prm.timing = 0;
  q->stream = static_cast<cudaStream_t>(stream);
  *out = q;
  return NFFT_OK;
}

int nfft_nnplan_destroy(nfft_nnplan* q) {
  if (!q) return NFFT_OK;
  free_plans(q);
  delete q;
  return NFFT_OK;
}

int nfft_nnplan_set_stream(nfft_nnplan* q, void* stream) {
  if (!q) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  q->stream = static_cast<cudaStream_t>(stream);
  int rc = q->p1 ? nfft_set_stream(q->p1, stream) : NFFT_OK;
  if (!rc && q->p2) rc = nfft_set_stream(q->p2, stream);
  return rc;
}

int nfft_nnplan_set_nodes(nfft_nnplan* q, const void* k, const void* y, int on_device) {
  if (!q || (!k && q->M > 0) || (!y && q->Ny > 0)) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  const int D = q->D;
  const size_t rs = q->precision == 32 ? 4 : 8;
  const size_t nk = size_t(D) * q->M, ny = size_t(D) * q->Ny;
  std::vector<unsigned char> kb(nk * rs), yb(ny * rs);
  if (on_device) {
    if (nk) NFFT_CUDA_TRY(cudaMemcpy(kb.data(), k, nk * rs, cudaMemcpyDeviceToHost));
    if (ny) NFFT_CUDA_TRY(cudaMemcpy(yb.data(), y, ny * rs, cudaMemcpyDeviceToHost));
  } else {
    if (nk) memcpy(kb.data(), k, nk * rs);
    if (ny) memcpy(yb.data(), y, ny * rs);
  }
  auto val = [&](const std::vector<unsigned char>& b, size_t i) {
    return q->precision == 32 ? double(reinterpret_cast<const float*>(b.data())[i])
                              : reinterpret_cast<const double*>(b.data())[i];
  };
  for (size_t i = 0; i < nk; ++i) {
    const double v = val(kb, i);
    if (!(std::fabs(v) <= 0.5)) {
      set_error("Nodes k need to be within the range [-1/2, 1/2]");
      return NFFT_ERR_NODE_OUT_OF_RANGE;
    }
  }
  double ymax[3] = {0, 0, 0};
  for (size_t i = 0; i < ny; ++i) {
    const double v = val(yb, i);
    if (!std::isfinite(v)) {
      set_error("points y must be finite");
      return NFFT_ERR_INVALID_ARG;
    }
    ymax[i % D] = std::fmax(ymax[i % D], std::fabs(v));
  }
  const int m = q->prm.m > 0 ? q->prm.m : 4;
  const double sigma = q->prm.sigma > 0 ? q->prm.sigma : 2.0;
  int64_t N1[3] = {1, 1, 1};
  for (int d = 0; d < D; ++d) N1[d] = 2 * int64_t(std::ceil(ymax[d] + m / sigma)) + 2;
  bool same = q->p1 != nullptr;
  for (int d = 0; d < D; ++d) same = same && N1[d] == q->N1[d];
  q->has_nodes = false;
  if (!same) {
    free_plans(q);
    for (int d = 0; d < 3; ++d) q->N1[d] = N1[d];
    int rc = nfft_plan_create(&q->p1, q->precision, D, N1, q->Ny, &q->prm, q->stream);
    if (!rc) {
      for (int d = 0; d < 3; ++d) q->Nt1[d] = q->p1->Nt[d];
      rc = nfft_plan_create(&q->p2, q->precision, D, q->Nt1, q->M, &q->prm, q->stream);
    }
    if (!rc) {
      const size_t cs = 2 * rs;
      const int64_t ng = q->Nt1[0] * q->Nt1[1] * q->Nt1[2];
      if (cudaMalloc(&q->img, size_t(ng) * cs) != cudaSuccess ||
          cudaMalloc(&q->invhat, size_t(q->M > 0 ? q->M : 1) * rs) != cudaSuccess ||
          cudaMalloc(&q->tmp, size_t(q->M > 0 ? q->M : 1) * cs) != cudaSuccess) {
        set_error("cudaMalloc of the NNFFT buffers failed");
        rc = NFFT_ERR_ALLOC;
      }
    }
    if (rc) {  // leave no half-built plan behind
      free_plans(q);
      return rc;
    }
  }
  // P1 nodes u = y / N1, P2 nodes k / sigma1, window transforms in FP64
  std::vector<unsigned char> u(ny * rs), k2(nk * rs), ih(size_t(q->M) * rs);
  auto put = [&](std::vector<unsigned char>& b, size_t i, double v) {
    if (q->precision == 32) reinterpret_cast<float*>(b.data())[i] = float(v);
    else reinterpret_cast<double*>(b.data())[i] = v;
  };
  double s1[3];
  for (int d = 0; d < D; ++d) s1[d] = double(q->Nt1[d]) / double(q->N1[d]);
  for (size_t i = 0; i < ny; ++i) put(u, i, val(yb, i) / double(q->N1[i % D]));
  for (size_t i = 0; i < nk; ++i) put(k2, i, val(kb, i) / s1[i % D]);
  const double sig1 = q->p1->sigma;
  for (int64_t j = 0; j < q->M; ++j) {
    double h = 1.0;
    for (int d = 0; d < D; ++d)
      h *= window_hat(q->prm.window, val(kb, size_t(j) * D + d) * double(q->N1[d]), double(q->Nt1[d]), m, sig1);
    put(ih, size_t(j), 1.0 / h);
  }
  if (int rc = nfft_set_nodes(q->p1, u.data(), 0)) return rc;
  if (int rc = nfft_set_nodes(q->p2, k2.data(), 0)) return rc;
  if (q->M > 0) NFFT_CUDA_TRY(cudaMemcpy(q->invhat, ih.data(), ih.size(), cudaMemcpyHostToDevice));
  q->has_nodes = true;
  return NFFT_OK;
}

int nfft_nnplan_forward(nfft_nnplan* q, const void* c, void* fhat) {
  if (!q || (!c && q->Ny > 0) || (!fhat && q->M > 0)) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  if (!q->has_nodes) {
    set_error("plan has no nodes");
    return NFFT_ERR_NO_NODES;
  }
  return q->precision == 32 ? nn_forward<float>(q, c, fhat) : nn_forward<double>(q, c, fhat);
}

int nfft_nnplan_adjoint(nfft_nnplan* q, const void* fhat, void* c) {
  if (!q || (!c && q->Ny > 0) || (!fhat && q->M > 0)) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  if (!q->has_nodes) {
    set_error("plan has no nodes");
    return NFFT_ERR_NO_NODES;
  }
  return q->precision == 32 ? nn_adjoint<float>(q, fhat, c) : nn_adjoint<double>(q, fhat, c);
}

}  // extern "C"
