// NFFTTools' Toeplitz tools on the GPU (NFFTTools/src/Toeplitz.jl): the
// Gram operator A^H A of an NFFT plan as a convolution with a kernel lambda on
// the twice-oversampled image grid.
//   calculateToeplitzKernel(!) (:86-93, :129-135): lambda = FFT(fftshift(
//       adjoint(p) * ones(J))) with p a plan of size 2N holding the nodes;
//   calculateToeplitzKernel_explicit (:142-164): the same from the exact sums
//       E[n] = sum_j exp(2 pi i k_j . n), n_d = idx_d - 1 - N_d on the 2N grid;
//   convolveToeplitzKernel! (:230-244): y <- crop(IFFT(lambda . FFT(pad(y)))),
//       y in the corner of a zero 2N grid, IFFT normalised by 1/|2N|.
//
// GB300 form of the convolution: on power-of-two grids 64..1024 (D = 2, 3) the
// pruned line FFTs of fft.cu with the product fused into the last axis' pass
// (fused_toeplitz: each 1-D pass reads only the nonzero input and writes only
// what the next pass reads, lambda is read once); elsewhere (D = 1, other
// sizes, or on request) corner pad, cuFFT over the 2N grid, product, cuFFT
// back, crop -- the reference's own sequence.
// fftshift + FFT: the grid sizes 2N_d are even, so FFT(fftshift(x))[k] =
// (-1)^(k_1 + ... + k_D) FFT(x)[k]; the shift is a sign pattern applied after
// an in-place cuFFT.
#include "nfft_internal.cuh"

#include <vector>

struct nfft_toeplitz {
  nfft_plan* t = nullptr;    // transform-only plan: N image, Ntilde = 2N, unit deconvolution factors
  int fft_mode = 0;          // 0: fused where the sizes allow, 1: cuFFT
  cufftHandle fft = 0;       // full 2N-grid transform (lazy)
  bool fft_ok = false;
  void* ones = nullptr;      // J complex ones for calculateToeplitzKernel
  int64_t ones_len = 0;
  void* kbuf = nullptr;      // nodes copied from the host for the explicit kernel
  size_t kbuf_bytes = 0;
  cudaEvent_t ev = nullptr;  // orders the NFFT plan's stream before this object's
};

namespace nfft {
namespace {

template <typename T> using Cx = typename Cplx<T>::type;

struct Box {
  int N[3], Nt[3];
};

unsigned grid_blocks(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return unsigned(b < 1 ? 1 : b);
}

// zero 2N grid with the image y in its corner
template <typename T>
__global__ void __launch_bounds__(256) pad_corner_kernel(Box B, const Cx<T>* __restrict__ y, Cx<T>* __restrict__ g,
                                                         int64_t ng) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < ng; i += int64_t(gridDim.x) * blockDim.x) {
    const int x = int(i % B.Nt[0]);
    const int64_t r = i / B.Nt[0];
    const int yy = int(r % B.Nt[1]), z = int(r / B.Nt[1]);
    Cx<T> v;
    v.x = T(0);
    v.y = T(0);
    if (x < B.N[0] && yy < B.N[1] && z < B.N[2]) v = y[x + int64_t(B.N[0]) * (yy + int64_t(B.N[1]) * z)];
    g[i] = v;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) crop_corner_kernel(Box B, const Cx<T>* __restrict__ g, Cx<T>* __restrict__ y,
                                                          int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int x = int(i % B.N[0]);
    const int64_t r = i / B.N[0];
    const int yy = int(r % B.N[1]), z = int(r / B.N[1]);
    y[i] = g[x + int64_t(B.Nt[0]) * (yy + int64_t(B.Nt[1]) * z)];
  }
}

template <typename T>
__global__ void __launch_bounds__(256) product_kernel(Cx<T>* __restrict__ g, const Cx<T>* __restrict__ lam, T scale,
                                                      int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const Cx<T> a = g[i], l = __ldg(lam + i);
    Cx<T> r;
    r.x = scale * (a.x * l.x - a.y * l.y);
    r.y = scale * (a.x * l.y + a.y * l.x);
    g[i] = r;
  }
}

// (-1)^(k_1 + k_2 + k_3): the fftshift of the even-sized grid, after its FFT
template <typename T>
__global__ void __launch_bounds__(256) shift_sign_kernel(Box B, Cx<T>* __restrict__ g, int64_t ng) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < ng; i += int64_t(gridDim.x) * blockDim.x) {
    const int x = int(i % B.Nt[0]);
    const int64_t r = i / B.Nt[0];
    const int yy = int(r % B.Nt[1]), z = int(r / B.Nt[1]);
    if ((x + yy + z) & 1) {
      Cx<T> v = g[i];
      v.x = -v.x;
      v.y = -v.y;
      g[i] = v;
    }
  }
}

template <typename T> __global__ void __launch_bounds__(256) fill_ones_kernel(Cx<T>* __restrict__ a, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    Cx<T> v;
    v.x = T(1);
    v.y = T(0);
    a[i] = v;
  }
}

// E[idx] = sum_j exp(2 pi i k_j . n), n_d = idx_d - N_d (getMatrixElement,
// Toeplitz.jl:152-164, with the sign folded: -(N_d + 1 - idx_d) for 1-based
// idx).  Thread per grid point, nodes staged through shared memory as FP64,
// phases by sincospi in FP64 (exact argument reduction), sums in FP64.
constexpr int kExplicitChunk = 256;
template <typename T>
__global__ void __launch_bounds__(256) explicit_kernel(Box B, int D, const T* __restrict__ k, int64_t M,
                                                       Cx<T>* __restrict__ out, int64_t ng) {
  __shared__ double sk[3][kExplicitChunk];
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  double n[3] = {0.0, 0.0, 0.0};
  if (i < ng) {
    const int x = int(i % B.Nt[0]);
    const int64_t r = i / B.Nt[0];
    n[0] = double(x - B.N[0]);
    if (D > 1) n[1] = double(int(r % B.Nt[1]) - B.N[1]);
    if (D > 2) n[2] = double(int(r / B.Nt[1]) - B.N[2]);
  }
  double re = 0.0, im = 0.0;
  for (int64_t j0 = 0; j0 < M; j0 += kExplicitChunk) {
    const int cnt = int(M - j0 < kExplicitChunk ? M - j0 : kExplicitChunk);
    __syncthreads();
    for (int t = threadIdx.x; t < cnt * D; t += blockDim.x) {
      const int j = t / D, d = t % D;
      sk[d][j] = double(k[(j0 + j) * D + d]);
    }
    for (int t = threadIdx.x; t < cnt; t += blockDim.x)
      for (int d = D; d < 3; ++d) sk[d][t] = 0.0;
    __syncthreads();
    for (int j = 0; j < cnt; ++j) {
      const double ph = 2.0 * (sk[0][j] * n[0] + sk[1][j] * n[1] + sk[2][j] * n[2]);
      double s, c;
      sincospi(ph, &s, &c);
      re += c;
      im += s;
    }
  }
  if (i < ng) {
    Cx<T> v;
    v.x = T(re);
    v.y = T(im);
    out[i] = v;
  }
}

Box make_box(const nfft_plan* t) {
  Box B;
  for (int d = 0; d < 3; ++d) {
    B.N[d] = int(t->N[d]);
    B.Nt[d] = int(t->Nt[d]);
  }
  return B;
}

int64_t grid_count(const nfft_plan* t) { return t->Nt[0] * t->Nt[1] * t->Nt[2]; }
int64_t image_count(const nfft_plan* t) { return t->N[0] * t->N[1] * t->N[2]; }

int fft_check(cufftResult r, const char* what) {
  if (r == CUFFT_SUCCESS) return NFFT_OK;
  set_error("cuFFT %s failed (%d)", what, int(r));
  return NFFT_ERR_CUFFT;
}

// the full 2N-grid cuFFT plan (column-major: dimension 1 fastest)
int ensure_fft(nfft_toeplitz* q) {
  if (q->fft_ok) return NFFT_OK;
  const nfft_plan* t = q->t;
  int n[3];
  for (int d = 0; d < t->D; ++d) n[d] = int(t->Nt[t->D - 1 - d]);
  const cufftType type = t->precision == 32 ? CUFFT_C2C : CUFFT_Z2Z;
  if (int rc = fft_check(cufftPlanMany(&q->fft, t->D, n, nullptr, 1, 0, nullptr, 1, 0, type, 1), "plan"))
    return rc;
  q->fft_ok = true;
  return fft_check(cufftSetStream(q->fft, t->stream), "set stream");
}

int exec_fft(nfft_toeplitz* q, void* g, int dir) {
  if (q->t->precision == 32)
    return fft_check(cufftExecC2C(q->fft, static_cast<cufftComplex*>(g), static_cast<cufftComplex*>(g), dir),
                     "exec");
  return fft_check(
      cufftExecZ2Z(q->fft, static_cast<cufftDoubleComplex*>(g), static_cast<cufftDoubleComplex*>(g), dir), "exec");
}

template <typename T> int apply_cufft(nfft_toeplitz* q, const void* lam, void* y) {
  nfft_plan* t = q->t;
  const Box B = make_box(t);
  const int64_t ng = grid_count(t), ni = image_count(t);
  Cx<T>* g = static_cast<Cx<T>*>(t->grid);
  if (int rc = ensure_fft(q)) return rc;
  pad_corner_kernel<T><<<grid_blocks(ng), 256, 0, t->stream>>>(B, static_cast<const Cx<T>*>(y), g, ng);
  NFFT_LAUNCH_CHECK();
  if (int rc = exec_fft(q, g, CUFFT_FORWARD)) return rc;
  product_kernel<T><<<grid_blocks(ng), 256, 0, t->stream>>>(g, static_cast<const Cx<T>*>(lam), T(1.0 / double(ng)),
                                                            ng);
  NFFT_LAUNCH_CHECK();
  if (int rc = exec_fft(q, g, CUFFT_INVERSE)) return rc;
  crop_corner_kernel<T><<<grid_blocks(ni), 256, 0, t->stream>>>(B, g, static_cast<Cx<T>*>(y), ni);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

// lambda <- FFT(fftshift(lambda)) in place on the 2N grid
template <typename T> int shift_fft(nfft_toeplitz* q, void* lam) {
  nfft_plan* t = q->t;
  if (int rc = ensure_fft(q)) return rc;
  if (int rc = exec_fft(q, lam, CUFFT_FORWARD)) return rc;
  const int64_t ng = grid_count(t);
  shift_sign_kernel<T><<<grid_blocks(ng), 256, 0, t->stream>>>(make_box(t), static_cast<Cx<T>*>(lam), ng);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

template <typename T> int kernel_from_plan(nfft_toeplitz* q, nfft_plan* p, void* lam) {
  const int64_t need = p->M > 0 ? p->M : 1;
  if (q->ones_len < need) {
    cudaFree(q->ones);
    q->ones = nullptr;
    q->ones_len = 0;
    if (cudaMalloc(&q->ones, size_t(need) * sizeof(Cx<T>)) != cudaSuccess) {
      set_error("cudaMalloc of %lld ones failed", (long long)need);
      return NFFT_ERR_ALLOC;
    }
    q->ones_len = need;
  }
  fill_ones_kernel<T><<<grid_blocks(need), 256, 0, p->stream>>>(static_cast<Cx<T>*>(q->ones), need);
  NFFT_LAUNCH_CHECK();
  if (int rc = nfft_adjoint(p, q->ones, lam)) return rc;
  if (p->stream != q->t->stream) {
    NFFT_CUDA_TRY(cudaEventRecord(q->ev, p->stream));
    NFFT_CUDA_TRY(cudaStreamWaitEvent(q->t->stream, q->ev, 0));
  }
  return shift_fft<T>(q, lam);
}

template <typename T> int kernel_explicit(nfft_toeplitz* q, const void* k, int64_t M, void* lam) {
  nfft_plan* t = q->t;
  const int64_t ng = grid_count(t);
  const unsigned blocks = unsigned((ng + 255) / 256);
  explicit_kernel<T><<<blocks, 256, 0, t->stream>>>(make_box(t), t->D, static_cast<const T*>(k), M,
                                                    static_cast<Cx<T>*>(lam), ng);
  NFFT_LAUNCH_CHECK();
  return shift_fft<T>(q, lam);
}

}  // namespace
}  // namespace nfft

using namespace nfft;

extern "C" {

int nfft_toeplitz_create(nfft_toeplitz** out, int precision, int D, const int64_t* N, int fft_mode, void* stream) {
  if (!out || !N) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  *out = nullptr;
  if (precision != 32 && precision != 64) {
    set_error("precision must be 32 or 64");
    return NFFT_ERR_INVALID_ARG;
  }
  if (D < 1 || D > 3) {
    set_error("D = %d not supported (1..3)", D);
    return NFFT_ERR_INVALID_ARG;
  }
  if (fft_mode != 0 && fft_mode != 1) {
    set_error("fft_mode must be 0 (fused where possible) or 1 (cuFFT)");
    return NFFT_ERR_INVALID_ARG;
  }
  for (int d = 0; d < D; ++d)
    if (N[d] < 1 || N[d] > (int64_t(1) << 28)) {
      set_error("image size N[%d] = %lld out of range", d, (long long)N[d]);
      return NFFT_ERR_INVALID_ARG;
    }
  auto* q = new nfft_toeplitz();
  auto* t = new nfft_plan();
  q->t = t;
  q->fft_mode = fft_mode;
  t->precision = precision;
  t->real_size = precision == 32 ? 4 : 8;
  t->D = D;
  for (int d = 0; d < D; ++d) {
    t->N[d] = N[d];
    t->Nt[d] = 2 * N[d];
  }
  t->stream = static_cast<cudaStream_t>(stream);
  const size_t cs = 2 * t->real_size;
  int rc = NFFT_OK;
  if (cudaMalloc(&t->grid, size_t(grid_count(t)) * cs) != cudaSuccess) {
    set_error("cudaMalloc of the %lld-point grid failed", (long long)grid_count(t));
    rc = NFFT_ERR_ALLOC;
  }
  if (!rc) {
    // unit factors for the fused passes' deconvolution slots (+ the "one" entry)
    const int64_t nf = t->N[0] + t->N[1] + t->N[2] + 1;
    std::vector<unsigned char> h(size_t(nf) * t->real_size);
    for (int64_t i = 0; i < nf; ++i) {
      if (precision == 32) reinterpret_cast<float*>(h.data())[i] = 1.f;
      else reinterpret_cast<double*>(h.data())[i] = 1.0;
    }
    if (cudaMalloc(&t->inv, h.size()) != cudaSuccess) {
      set_error("cudaMalloc of the unit factors failed");
      rc = NFFT_ERR_ALLOC;
    } else if (cudaMemcpy(t->inv, h.data(), h.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
      set_error("copy of the unit factors failed");
      rc = NFFT_ERR_CUDA;
    }
  }
  if (!rc && fft_mode == 0) rc = fused_fft_init(t);
  if (!rc && cudaEventCreateWithFlags(&q->ev, cudaEventDisableTiming) != cudaSuccess) {
    set_error("cudaEventCreate failed");
    rc = NFFT_ERR_CUDA;
  }
  if (rc) {
    nfft_toeplitz_destroy(q);
    return rc;
  }
  *out = q;
  return NFFT_OK;
}

int nfft_toeplitz_destroy(nfft_toeplitz* q) {
  if (!q) return NFFT_OK;
  if (q->fft_ok) cufftDestroy(q->fft);
  cudaFree(q->ones);
  cudaFree(q->kbuf);
  if (q->ev) cudaEventDestroy(q->ev);
  nfft_plan_destroy(q->t);
  delete q;
  return NFFT_OK;
}

int nfft_toeplitz_set_stream(nfft_toeplitz* q, void* stream) {
  if (!q) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  q->t->stream = static_cast<cudaStream_t>(stream);
  if (q->fft_ok) return fft_check(cufftSetStream(q->fft, q->t->stream), "set stream");
  return NFFT_OK;
}

int nfft_toeplitz_is_fused(const nfft_toeplitz* q, int* fused) {
  if (!q || !fused) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  *fused = q->t->fused_fft ? 1 : 0;
  return NFFT_OK;
}

int nfft_toeplitz_apply(nfft_toeplitz* q, const void* lambda, void* y) {
  if (!q || !lambda || !y) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  nfft_plan* t = q->t;
  if (t->fused_fft) return fused_toeplitz(t, lambda, 1.0 / double(grid_count(t)), y);
  return t->precision == 32 ? apply_cufft<float>(q, lambda, y) : apply_cufft<double>(q, lambda, y);
}

int nfft_toeplitz_kernel(nfft_toeplitz* q, nfft_plan* p, void* lambda) {
  if (!q || !p || !lambda) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  const nfft_plan* t = q->t;
  if (p->precision != t->precision) {
    set_error("plan precision %d does not match the Toeplitz object's %d", p->precision, t->precision);
    return NFFT_ERR_INVALID_ARG;
  }
  if (p->D != t->D) {
    set_error("plan dimension %d does not match the Toeplitz object's %d", p->D, t->D);
    return NFFT_ERR_DIM_MISMATCH;
  }
  for (int d = 0; d < t->D; ++d)
    if (p->N[d] != t->Nt[d]) {
      set_error("the plan's N[%d] = %lld must be twice the image size (%lld)", d, (long long)p->N[d],
                (long long)t->Nt[d]);
      return NFFT_ERR_DIM_MISMATCH;
    }
  if (!p->has_nodes) {
    set_error("plan has no nodes");
    return NFFT_ERR_NO_NODES;
  }
  return t->precision == 32 ? kernel_from_plan<float>(q, p, lambda) : kernel_from_plan<double>(q, p, lambda);
}

int nfft_toeplitz_kernel_explicit(nfft_toeplitz* q, const void* k, int64_t M, int k_on_device, void* lambda) {
  if (!q || !lambda || (!k && M > 0) || M < 0) {
    set_error("null argument or negative node count");
    return NFFT_ERR_INVALID_ARG;
  }
  nfft_plan* t = q->t;
  const void* kd = k;
  if (M > 0 && !k_on_device) {
    const size_t bytes = size_t(M) * t->D * t->real_size;
    if (q->kbuf_bytes < bytes) {
      cudaFree(q->kbuf);
      q->kbuf = nullptr;
      q->kbuf_bytes = 0;
      if (cudaMalloc(&q->kbuf, bytes) != cudaSuccess) {
        set_error("cudaMalloc of %zu node bytes failed", bytes);
        return NFFT_ERR_ALLOC;
      }
      q->kbuf_bytes = bytes;
    }
    NFFT_CUDA_TRY(cudaMemcpyAsync(q->kbuf, k, bytes, cudaMemcpyHostToDevice, t->stream));
    kd = q->kbuf;
  }
  return t->precision == 32 ? kernel_explicit<float>(q, kd, M, lambda) : kernel_explicit<double>(q, kd, M, lambda);
}

}  // extern "C"
