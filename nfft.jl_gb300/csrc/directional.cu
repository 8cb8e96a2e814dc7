// Directional plans: the NFFT along a contiguous range of dimensions dims
// of a D-dimensional array, every other index a batch column
// (src/directional.jl, NFFTPlan with dims, src/implementation.jl:73-104).
// NOut replaces the dims range of N by the node count J; the reference
// forces precompute = LINEAR and runs unblocked loops.
//
// GB300 form: the data is (pre, transform dims, post) with pre the
// contiguous inner index.  Every (pre, post) index pair is a column: an image
// of the transform dims.  The core plan bins the nodes once, and the columns
// are transformed together:
//   pad + apodize  grid column c = a + pre b holds image column (a, b) at
//                  (n + Ntilde - N/2) mod Ntilde, times prod 1/phi-hat; for
//                  pre > 1 a shared-memory transposition (pre <-> image index)
//   FFT            cuFFT along dims, batched over the contiguous grid columns
//   gather         the core plan's tiled gather, all columns per launch, into
//                  node values in column order, transposed to (pre, node, post)
//   spread         node values transposed to column order, then the core
//                  plan's atomic-free tiled spreader, all columns per launch
//   crop + apodize (transposing for pre > 1)
// Plans without nodes (and pre > 1 with NFFT_GB300_DIRECTIONAL_TILED=0) keep
// the grid in (pre, grid, post) order and run one thread per (pre, node, post)
// with global atomics for the spread (the reference's unblocked
// convolve_transpose! of src/directional.jl:107-154).
// The window follows src/directional.jl:82-92: xscale = k * Ntilde in T,
// c = floor(xscale), taps c-m+1 .. c+m, LUT linear interpolation at
// |xscale - l| * LUTSize/m.  A core plan over the transform dims supplies the
// LUT and the deconvolution factors.
#include "nfft_internal.cuh"

#include <algorithm>
#include <vector>

struct nfft_dplan {
  nfft_plan* core = nullptr;       // plan over the transform dims (tables only)
  int precision = 32;
  int D = 0, R = 0;                // array rank, number of transform dims
  int lo = 0;                      // first transform dim (0-based)
  int64_t N[3] = {1, 1, 1};
  int64_t Nt[3] = {1, 1, 1};       // oversampled along dims, N elsewhere
  int64_t M = 0;
  int64_t pre = 1, post = 1;       // column counts before / after dims
  int64_t Rn = 1, Rnt = 1;         // points of one column: image / grid
  cudaStream_t stream = nullptr;
  void* k = nullptr;               // R x M nodes (T), user order
  void* grid = nullptr;            // pre x Rnt x post complex
  cufftHandle fft = 0;
  bool fft_ok = false;
  bool fft_loop = false;           // one exec per post column block
  void* fft_work = nullptr;
  bool has_nodes = false;
  // tiled: grid columns contiguous (column c = a + pre b), the core plan's
  // tiled gather / atomic-free spreader run over all columns
  bool tiled = false;
  int64_t ncols = 1;               // pre x post
  void* sorted = nullptr;          // tiled: bin-sorted node values of a launch's columns (M x <= 65535 complex)
  void* vals = nullptr;            // tiled, pre > 1: node values in column order (M x ncols complex)
};

namespace nfft {
namespace {

template <typename T> struct DGeom {
  int R, m;
  int64_t pre, post, M, Rn, Rnt;
  int N[3], Nt[3];                 // transform dims only
  T lut_scale;
  const T* lut;
  const T* inv[3];
};

template <typename T> DGeom<T> make_dgeom(const nfft_dplan* q) {
  DGeom<T> G{};
  G.R = q->R;
  G.m = q->core->m;
  G.pre = q->pre;
  G.post = q->post;
  G.M = q->M;
  G.Rn = q->Rn;
  G.Rnt = q->Rnt;
  const T* inv = static_cast<const T*>(q->core->inv);
  int64_t off = 0;
  for (int d = 0; d < 3; ++d) {
    G.N[d] = d < q->R ? int(q->N[q->lo + d]) : 1;
    G.Nt[d] = d < q->R ? int(q->Nt[q->lo + d]) : 1;
    G.inv[d] = inv + off;
    if (d < q->R) off += G.N[d];
  }
  // singleton dims read the "one" entry stored after the factors
  for (int d = q->R; d < 3; ++d) G.inv[d] = inv + off;
  G.lut_scale = T(q->core->lut_size / q->core->m);
  G.lut = static_cast<const T*>(q->core->lut);
  return G;
}

unsigned blocks_for(int64_t work) {
  int64_t b = (work + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  return unsigned(b < 1 ? 1 : b);
}

template <typename T>
__global__ void __launch_bounds__(256) dpad_kernel(DGeom<T> G, const typename Cplx<T>::type* __restrict__ f,
                                                   typename Cplx<T>::type* __restrict__ g) {
  using C = typename Cplx<T>::type;
  const int64_t total = G.pre * G.Rnt * G.post;
  for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < total; q += int64_t(gridDim.x) * blockDim.x) {
    const int64_t a = q % G.pre;
    const int64_t r = q / G.pre;
    int64_t gt = r % G.Rnt;
    const int64_t b = r / G.Rnt;
    int64_t nl = 0, stride = 1;
    bool in = true;
    T w = T(1);
    for (int d = 0; d < G.R; ++d) {
      const int gd = int(gt % G.Nt[d]);
      gt /= G.Nt[d];
      const int nd = wrap_once(gd + G.N[d] / 2, G.Nt[d]);  // image index of grid point gd
      in = in && nd < G.N[d];
      if (nd < G.N[d]) {
        w *= __ldg(G.inv[d] + nd);
        nl += nd * stride;
      }
      stride *= G.N[d];
    }
    C v;
    v.x = T(0);
    v.y = T(0);
    if (in) {
      const C s = f[a + G.pre * (nl + G.Rn * b)];
      v.x = s.x * w;
      v.y = s.y * w;
    }
    g[q] = v;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) dcrop_kernel(DGeom<T> G, const typename Cplx<T>::type* __restrict__ g,
                                                    typename Cplx<T>::type* __restrict__ f) {
  using C = typename Cplx<T>::type;
  const int64_t total = G.pre * G.Rn * G.post;
  for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < total; q += int64_t(gridDim.x) * blockDim.x) {
    const int64_t a = q % G.pre;
    const int64_t r = q / G.pre;
    int64_t nt = r % G.Rn;
    const int64_t b = r / G.Rn;
    int64_t gl = 0, stride = 1;
    T w = T(1);
    for (int d = 0; d < G.R; ++d) {
      const int nd = int(nt % G.N[d]);
      nt /= G.N[d];
      gl += int64_t(wrap_once(nd - G.N[d] / 2, G.Nt[d])) * stride;
      w *= __ldg(G.inv[d] + nd);
      stride *= G.Nt[d];
    }
    const C s = g[a + G.pre * (gl + G.Rnt * b)];
    C v;
    v.x = s.x * w;
    v.y = s.y * w;
    f[q] = v;
  }
}

// Grid offset within a column (uncentred oversampled grid) and apodization
// factor of image point n of the transform dims.
template <typename T> __device__ __forceinline__ int64_t dgrid_point(const DGeom<T>& G, int64_t n, T& w) {
  int64_t gl = 0, stride = 1;
  w = T(1);
  for (int d = 0; d < G.R; ++d) {
    const int nd = int(n % G.N[d]);
    n /= G.N[d];
    gl += int64_t(wrap_once(nd - G.N[d] / 2, G.Nt[d])) * stride;
    w *= __ldg(G.inv[d] + nd);
    stride *= G.Nt[d];
  }
  return gl;
}

// Transposition between the user layout X[a + pre (n + nn b)] (pre index a
// contiguous) and the column layout Y[map(n) + ystride (a + pre b)] through a
// 32 x 32 shared-memory tile, both sides coalesced.  GRID: n is an image
// point, map(n) its grid offset, values scaled by its apodization factor
// (pad: X -> Y into a zeroed grid; crop: Y -> X); otherwise map(n) = n
// (node values).  Block 32 x 8; grid (n tiles, a tiles, post).
template <typename T, bool TO_Y, bool GRID>
__global__ void __launch_bounds__(256) dtranspose_kernel(DGeom<T> G, const typename Cplx<T>::type* __restrict__ src,
                                                         typename Cplx<T>::type* __restrict__ dst, int64_t nn,
                                                         int64_t ystride) {
  using C = typename Cplx<T>::type;
  __shared__ C tile[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int64_t n0 = int64_t(blockIdx.x) * 32, a0 = int64_t(blockIdx.y) * 32;
  // the n of this thread on the column side, with its grid offset and factor
  const int64_t nc = n0 + tx;
  T w = T(1);
  int64_t yoff = nc;
  if (GRID && nc < nn) yoff = dgrid_point(G, nc, w);
  for (int64_t b = blockIdx.z; b < G.post; b += gridDim.z) {
    const int64_t xbase = G.pre * nn * b, cbase = G.pre * b;
    if (TO_Y) {
#pragma unroll
      for (int i = 0; i < 4; ++i) {  // X rows n, coalesced over a
        const int64_t n = n0 + ty + 8 * i, a = a0 + tx;
        if (n < nn && a < G.pre) tile[ty + 8 * i][tx] = src[xbase + a + G.pre * n];
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < 4; ++i) {  // Y columns a, coalesced over n
        const int64_t a = a0 + ty + 8 * i;
        if (nc < nn && a < G.pre) {
          C v = tile[tx][ty + 8 * i];
          v.x *= w;
          v.y *= w;
          dst[yoff + ystride * (cbase + a)] = v;
        }
      }
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) {  // Y columns a, coalesced over n
        const int64_t a = a0 + ty + 8 * i;
        if (nc < nn && a < G.pre) {
          C v = src[yoff + ystride * (cbase + a)];
          v.x *= w;
          v.y *= w;
          tile[tx][ty + 8 * i] = v;
        }
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < 4; ++i) {  // X rows n, coalesced over a
        const int64_t n = n0 + ty + 8 * i, a = a0 + tx;
        if (n < nn && a < G.pre) dst[xbase + a + G.pre * n] = tile[ty + 8 * i][tx];
      }
    }
    __syncthreads();
  }
}

template <typename T, bool TO_Y, bool GRID>
int dtranspose(nfft_dplan* q, const DGeom<T>& G, const void* src, void* dst, int64_t nn, int64_t ystride) {
  using C = typename Cplx<T>::type;
  if (nn == 0) return NFFT_OK;
  const int64_t nt = (nn + 31) / 32, at = (q->pre + 31) / 32;
  if (at > 65535) {
    set_error("directional plan: %lld columns before dims exceed the transposition grid", (long long)q->pre);
    return NFFT_ERR_UNSUPPORTED;
  }
  if (nt > 0x7fffffffLL) return NFFT_ERR_UNSUPPORTED;
  const unsigned gz = unsigned(q->post < 65535 ? q->post : 65535);
  dtranspose_kernel<T, TO_Y, GRID><<<dim3(unsigned(nt), unsigned(at), gz), 256, 0, q->stream>>>(
      G, static_cast<const C*>(src), static_cast<C*>(dst), nn, ystride);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

// Window values and first grid index of node j along transform dim d.
template <typename T, int L>
__device__ __forceinline__ void dnode_weights(const DGeom<T>& G, T x, int d, int& c0, T (&w)[L]) {
  const T xs = x * T(G.Nt[d]);
  const T fc = floor(xs);
  c0 = int(fc) - G.m + 1;
  const T e = xs - fc;
  const T umax = T(G.m) * G.lut_scale;
#pragma unroll
  for (int l = 0; l < L; ++l) {
    const T dist = e + T(G.m - 1 - l);
    T u = (dist < T(0) ? -dist : dist) * G.lut_scale;
    if (u > umax) u = umax;
    const T fi = floor(u);
    const int i = int(fi);
    const T v0 = __ldg(G.lut + i), v1 = __ldg(G.lut + i + 1);
    w[l] = v0 + (u - fi) * (v1 - v0);
  }
}

// One thread per (pre index, node, post index); R = number of transform dims.
template <typename T, int R, int L, bool ADJ>
__global__ void __launch_bounds__(256) dconv_kernel(DGeom<T> G, const T* __restrict__ k,
                                                    const typename Cplx<T>::type* __restrict__ src,
                                                    typename Cplx<T>::type* __restrict__ dst) {
  using C = typename Cplx<T>::type;
  const int64_t total = G.pre * G.M * G.post;
  for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < total; q += int64_t(gridDim.x) * blockDim.x) {
    const int64_t a = q % G.pre;
    const int64_t r = q / G.pre;
    const int64_t j = r % G.M;
    const int64_t b = r / G.M;
    T w[R][L];
    int c0[R];
#pragma unroll
    for (int d = 0; d < R; ++d) dnode_weights<T, L>(G, __ldg(k + R * j + d), d, c0[d], w[d]);
    const int64_t colbase = a + G.pre * G.Rnt * b;
    T ar = T(0), ai = T(0);
    C v;
    if (ADJ) v = src[q];  // fHat[pre, j, post] has the same flat index q
    // taps: innermost dimension 0
    const int n1 = R > 1 ? L : 1, n2 = R > 2 ? L : 1;
    for (int t2 = 0; t2 < n2; ++t2) {
      const int i2 = R > 2 ? wrap_any(c0[R > 2 ? 2 : 0] + t2, G.Nt[2]) : 0;
      const T w2 = R > 2 ? w[R > 2 ? 2 : 0][t2] : T(1);
      for (int t1 = 0; t1 < n1; ++t1) {
        const int i1 = R > 1 ? wrap_any(c0[R > 1 ? 1 : 0] + t1, G.Nt[1]) : 0;
        const T w12 = w2 * (R > 1 ? w[R > 1 ? 1 : 0][t1] : T(1));
        const int64_t rowbase = int64_t(i1) * G.Nt[0] + int64_t(i2) * G.Nt[0] * G.Nt[1];
#pragma unroll
        for (int t0 = 0; t0 < L; ++t0) {
          const int i0 = wrap_any(c0[0] + t0, G.Nt[0]);
          const T ww = w12 * w[0][t0];
          const int64_t gi = colbase + G.pre * (rowbase + i0);
          if (ADJ) {
            T* gp = reinterpret_cast<T*>(dst + gi);
            atomicAdd(gp, ww * v.x);
            atomicAdd(gp + 1, ww * v.y);
          } else {
            const C s = src[gi];
            ar = fma(ww, s.x, ar);
            ai = fma(ww, s.y, ai);
          }
        }
      }
    }
    if (!ADJ) {
      C o;
      o.x = ar;
      o.y = ai;
      dst[q] = o;
    }
  }
}

template <typename T> int dcheck_nodes(nfft_dplan* q) {
  int flag = 0;
  int* dflag = q->core->dflag;
  NFFT_CUDA_TRY(cudaMemsetAsync(dflag, 0, sizeof(int), q->stream));
  int rc = launch_check_nodes(q->core, q->k, dflag);
  if (rc) return rc;
  NFFT_CUDA_TRY(cudaMemcpyAsync(&flag, dflag, sizeof(int), cudaMemcpyDeviceToHost, q->stream));
  NFFT_CUDA_TRY(cudaStreamSynchronize(q->stream));
  if (flag) {
    set_error("Nodes k need to be within the range [-1/2, 1/2)");
    return NFFT_ERR_NODE_OUT_OF_RANGE;
  }
  return NFFT_OK;
}

template <typename T, int R, int L>
int dconv_launch(nfft_dplan* q, const void* src, void* dst, bool adj) {
  using C = typename Cplx<T>::type;
  DGeom<T> G = make_dgeom<T>(q);
  const int64_t work = q->pre * q->M * q->post;
  if (work == 0) return NFFT_OK;
  if (adj)
    dconv_kernel<T, R, L, true><<<blocks_for(work), 256, 0, q->stream>>>(
        G, static_cast<const T*>(q->k), static_cast<const C*>(src), static_cast<C*>(dst));
  else
    dconv_kernel<T, R, L, false><<<blocks_for(work), 256, 0, q->stream>>>(
        G, static_cast<const T*>(q->k), static_cast<const C*>(src), static_cast<C*>(dst));
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

template <typename T, int R> int dconv_l(nfft_dplan* q, const void* src, void* dst, bool adj) {
  switch (q->core->m) {
    case 2: return dconv_launch<T, R, 4>(q, src, dst, adj);
    case 3: return dconv_launch<T, R, 6>(q, src, dst, adj);
    case 4: return dconv_launch<T, R, 8>(q, src, dst, adj);
    case 5: return dconv_launch<T, R, 10>(q, src, dst, adj);
    case 6: return dconv_launch<T, R, 12>(q, src, dst, adj);
    case 7: return dconv_launch<T, R, 14>(q, src, dst, adj);
    case 8: return dconv_launch<T, R, 16>(q, src, dst, adj);
  }
  set_error("m = %d not supported (2..8)", q->core->m);
  return NFFT_ERR_UNSUPPORTED;
}

template <typename T> int dconv(nfft_dplan* q, const void* src, void* dst, bool adj) {
  switch (q->R) {
    case 1: return dconv_l<T, 1>(q, src, dst, adj);
    case 2: return dconv_l<T, 2>(q, src, dst, adj);
    case 3: return dconv_l<T, 3>(q, src, dst, adj);
  }
  return NFFT_ERR_UNSUPPORTED;
}

int dexec_fft(nfft_dplan* q, int dir) {
  const int64_t step = q->pre * q->Rnt;
  const int64_t n = q->fft_loop ? q->post : 1;
  for (int64_t b = 0; b < n; ++b) {
    cufftResult r;
    if (q->precision == 32) {
      auto* g = static_cast<cufftComplex*>(q->grid) + b * step;
      r = cufftExecC2C(q->fft, g, g, dir);
    } else {
      auto* g = static_cast<cufftDoubleComplex*>(q->grid) + b * step;
      r = cufftExecZ2Z(q->fft, g, g, dir);
    }
    if (r != CUFFT_SUCCESS) {
      set_error("cuFFT exec failed (%d)", int(r));
      return NFFT_ERR_CUFFT;
    }
  }
  return NFFT_OK;
}

// All columns' gather (tiled) from the contiguous grid columns into
// node values out[j + M c], at most 65535 columns per launch.
template <typename T> int dgather_cols(nfft_dplan* q, void* out) {
  using C = typename Cplx<T>::type;
  int rc = NFFT_OK;
  for (int64_t c0 = 0; c0 < q->ncols && !rc; c0 += 65535) {
    const int nc = int(q->ncols - c0 < 65535 ? q->ncols - c0 : 65535);
    rc = launch_interp_cols(q->core, static_cast<const C*>(q->grid) + c0 * q->Rnt, static_cast<C*>(out) + c0 * q->M,
                            nc, q->Rnt, q->M);
  }
  return rc;
}

// All columns' spread (tiled, atomic-free) of node values in[j + M c] into
// the contiguous grid columns (the spreader zeroes them).
template <typename T> int dspread_cols(nfft_dplan* q, const void* in) {
  using C = typename Cplx<T>::type;
  int rc = NFFT_OK;
  for (int64_t c0 = 0; c0 < q->ncols && !rc; c0 += 65535) {
    const int nc = int(q->ncols - c0 < 65535 ? q->ncols - c0 : 65535);
    rc = launch_spread_cols(q->core, static_cast<const C*>(in) + c0 * q->M, static_cast<C*>(q->grid) + c0 * q->Rnt, nc,
                            q->M, q->Rnt, q->sorted);
  }
  return rc;
}

template <typename T> int dforward(nfft_dplan* q, const void* f, void* fhat) {
  using C = typename Cplx<T>::type;
  DGeom<T> G = make_dgeom<T>(q);
  int rc = NFFT_OK;
  if (q->tiled && q->pre > 1) {  // transposing pad into zeroed grid columns
    NFFT_CUDA_TRY(cudaMemsetAsync(q->grid, 0, 2 * sizeof(T) * size_t(q->ncols * q->Rnt), q->stream));
    if ((rc = dtranspose<T, true, true>(q, G, f, q->grid, q->Rn, q->Rnt))) return rc;
  } else {  // pre == 1: the layouts agree
    dpad_kernel<T><<<blocks_for(q->pre * q->Rnt * q->post), 256, 0, q->stream>>>(G, static_cast<const C*>(f),
                                                                                 static_cast<C*>(q->grid));
    NFFT_LAUNCH_CHECK();
  }
  if ((rc = dexec_fft(q, CUFFT_FORWARD))) return rc;
  if (!q->tiled) return dconv<T>(q, q->grid, fhat, false);
  if (q->pre == 1) return dgather_cols<T>(q, fhat);
  if ((rc = dgather_cols<T>(q, q->vals))) return rc;
  return dtranspose<T, false, false>(q, G, q->vals, fhat, q->M, q->M);
}

template <typename T> int dadjoint(nfft_dplan* q, const void* fhat, void* f) {
  using C = typename Cplx<T>::type;
  DGeom<T> G = make_dgeom<T>(q);
  int rc = NFFT_OK;
  if (q->tiled && q->pre > 1) {
    if ((rc = dtranspose<T, true, false>(q, G, fhat, q->vals, q->M, q->M))) return rc;
    rc = dspread_cols<T>(q, q->vals);
  } else if (q->tiled) {
    rc = dspread_cols<T>(q, fhat);
  } else {
    NFFT_CUDA_TRY(cudaMemsetAsync(q->grid, 0, 2 * sizeof(T) * size_t(q->pre * q->Rnt * q->post), q->stream));
    rc = dconv<T>(q, fhat, q->grid, true);
  }
  if (rc) return rc;
  if ((rc = dexec_fft(q, CUFFT_INVERSE))) return rc;
  if (q->tiled && q->pre > 1) return dtranspose<T, false, true>(q, G, q->grid, f, q->Rn, q->Rnt);
  dcrop_kernel<T><<<blocks_for(q->pre * q->Rn * q->post), 256, 0, q->stream>>>(G, static_cast<const C*>(q->grid),
                                                                              static_cast<C*>(f));
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

}  // namespace
}  // namespace nfft

using namespace nfft;

extern "C" int nfft_dplan_destroy(nfft_dplan* q) {
  if (!q) return NFFT_OK;
  if (q->fft_ok) cufftDestroy(q->fft);
  cudaFree(q->fft_work);
  cudaFree(q->grid);
  cudaFree(q->k);
  cudaFree(q->sorted);
  cudaFree(q->vals);
  if (q->core) nfft_plan_destroy(q->core);
  delete q;
  return NFFT_OK;
}

extern "C" int nfft_dplan_create(nfft_dplan** out, int precision, int D, const int64_t* N, int dim_lo, int dim_hi,
                                 int64_t M, const nfft_params* params, void* stream) {
  if (!out || !N || !params) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  *out = nullptr;
  if (precision != 32 && precision != 64) {
    set_error("precision must be 32 or 64");
    return NFFT_ERR_INVALID_ARG;
  }
  if (D < 1 || D > 3 || dim_lo < 0 || dim_hi < dim_lo || dim_hi >= D) {
    set_error("dims %d:%d do not fit a %d-dimensional array", dim_lo + 1, dim_hi + 1, D);
    return NFFT_ERR_INVALID_ARG;
  }
  for (int d = 0; d < D; ++d)
    if (N[d] < 1) {
      set_error("N must be positive");
      return NFFT_ERR_INVALID_ARG;
    }
  auto* q = new nfft_dplan();
  q->precision = precision;
  q->D = D;
  q->R = dim_hi - dim_lo + 1;
  q->lo = dim_lo;
  q->M = M;
  q->stream = static_cast<cudaStream_t>(stream);
  for (int d = 0; d < D; ++d) q->N[d] = N[d];
  // the core plan: the transform dims, LINEAR window (src/implementation.jl:80-82)
  nfft_params prm = *params;
  prm.precompute = NFFT_PRECOMPUTE_LINEAR;
  q->tiled = M > 0;
  if (dim_lo > 0) {
    const char* e = getenv("NFFT_GB300_DIRECTIONAL_TILED");
    if (e && e[0] == '0') q->tiled = false;
  }
  prm.blocking = q->tiled ? 1 : 0;
  prm.compensated = 0;
  prm.timing = 0;
  int64_t Nc[3] = {1, 1, 1};
  for (int d = 0; d < q->R; ++d) Nc[d] = N[dim_lo + d];
  int rc = nfft_plan_create(&q->core, precision, q->R, Nc, M, &prm, stream);
  if (rc) {
    delete q;
    return rc;
  }
  for (int d = 0; d < D; ++d) q->Nt[d] = (d >= dim_lo && d <= dim_hi) ? q->core->Nt[d - dim_lo] : N[d];
  for (int d = 0; d < dim_lo; ++d) q->pre *= N[d];
  for (int d = dim_hi + 1; d < D; ++d) q->post *= N[d];
  for (int d = dim_lo; d <= dim_hi; ++d) {
    q->Rn *= q->N[d];
    q->Rnt *= q->Nt[d];
  }
  const size_t rs = precision == 32 ? 4 : 8;
  const int64_t total = q->pre * q->Rnt * q->post;
  if (cudaMalloc(&q->grid, 2 * rs * size_t(total)) != cudaSuccess) {
    nfft_dplan_destroy(q);
    set_error("cudaMalloc of the directional grid failed");
    return NFFT_ERR_ALLOC;
  }
  q->ncols = q->pre * q->post;
  if (q->tiled) {
    const int64_t per = q->ncols < 65535 ? q->ncols : 65535;
    if (cudaMalloc(&q->sorted, 2 * rs * size_t(M) * size_t(per)) != cudaSuccess ||
        (q->pre > 1 && cudaMalloc(&q->vals, 2 * rs * size_t(M) * size_t(q->ncols)) != cudaSuccess)) {
      nfft_dplan_destroy(q);
      set_error("cudaMalloc of the column node values failed");
      return NFFT_ERR_ALLOC;
    }
  }
  // cuFFT along the transform dims (C order: reversed), columns batched
  int n[3];
  for (int d = 0; d < q->R; ++d) n[d] = int(q->Nt[dim_hi - d]);
  const cufftType type = precision == 32 ? CUFFT_C2C : CUFFT_Z2Z;
  size_t ws = 0;
  cufftResult r = cufftCreate(&q->fft);
  if (r == CUFFT_SUCCESS) {
    q->fft_ok = true;
    r = cufftSetAutoAllocation(q->fft, 0);
  }
  if (r == CUFFT_SUCCESS) {
    if (q->pre == 1 || q->tiled) {  // contiguous grid columns
      if (q->ncols > 0x7fffffffLL) r = CUFFT_INVALID_SIZE;
      else r = cufftMakePlanMany(q->fft, q->R, n, n, 1, int(q->Rnt), n, 1, int(q->Rnt), type, int(q->ncols), &ws);
    } else {
      q->fft_loop = q->post > 1;
      r = cufftMakePlanMany(q->fft, q->R, n, n, int(q->pre), 1, n, int(q->pre), 1, type, int(q->pre), &ws);
    }
  }
  if (r == CUFFT_SUCCESS && ws > 0 && cudaMalloc(&q->fft_work, ws) != cudaSuccess) r = CUFFT_ALLOC_FAILED;
  if (r == CUFFT_SUCCESS && ws > 0) r = cufftSetWorkArea(q->fft, q->fft_work);
  if (r == CUFFT_SUCCESS) r = cufftSetStream(q->fft, q->stream);
  if (r != CUFFT_SUCCESS) {
    nfft_dplan_destroy(q);
    set_error("cuFFT plan of the directional transform failed (%d)", int(r));
    return NFFT_ERR_CUFFT;
  }
  *out = q;
  return NFFT_OK;
}

extern "C" int nfft_dplan_set_nodes(nfft_dplan* q, const void* k, int k_on_device) {
  if (!q || (!k && q->M > 0)) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  const size_t rs = q->precision == 32 ? 4 : 8;
  const size_t bytes = rs * size_t(q->R) * size_t(q->M);
  q->has_nodes = false;
  if (!q->k && cudaMalloc(&q->k, bytes ? bytes : 16) != cudaSuccess) {
    set_error("cudaMalloc of the nodes failed");
    return NFFT_ERR_ALLOC;
  }
  if (bytes)
    NFFT_CUDA_TRY(cudaMemcpyAsync(q->k, k, bytes, k_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                  q->stream));
  int rc = q->precision == 32 ? dcheck_nodes<float>(q) : dcheck_nodes<double>(q);
  if (rc) return rc;
  if (q->tiled && (rc = nfft_set_nodes(q->core, q->k, 1))) return rc;
  q->has_nodes = true;
  return NFFT_OK;
}

extern "C" int nfft_dplan_set_stream(nfft_dplan* q, void* stream) {
  if (!q) return NFFT_ERR_INVALID_ARG;
  q->stream = static_cast<cudaStream_t>(stream);
  if (cufftSetStream(q->fft, q->stream) != CUFFT_SUCCESS) {
    set_error("cufftSetStream failed");
    return NFFT_ERR_CUFFT;
  }
  return nfft_set_stream(q->core, stream);
}

extern "C" int nfft_dplan_forward(nfft_dplan* q, const void* f, void* fhat) {
  if (!q || !f || (!fhat && q->M > 0)) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  if (!q->has_nodes) {
    set_error("plan has no nodes");
    return NFFT_ERR_NO_NODES;
  }
  return q->precision == 32 ? dforward<float>(q, f, fhat) : dforward<double>(q, f, fhat);
}

extern "C" int nfft_dplan_adjoint(nfft_dplan* q, const void* fhat, void* f) {
  if (!q || !f || (!fhat && q->M > 0)) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  if (!q->has_nodes) {
    set_error("plan has no nodes");
    return NFFT_ERR_NO_NODES;
  }
  return q->precision == 32 ? dadjoint<float>(q, fhat, f) : dadjoint<double>(q, fhat, f);
}
