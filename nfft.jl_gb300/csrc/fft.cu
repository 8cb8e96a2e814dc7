// Pruned grid FFT fused with the deconvolution (D = 2, 3; every Ntilde_d a
// power of two in [64, 1024]).  Replaces, on the transform path,
//   forward:  fill!(tmpVec, 0); deconvolve!; fft!      (src/implementation.jl:159-161)
//   adjoint:  bfft!; deconvolve_transpose!             (:182-183)
// by line FFTs that touch only what the zero padding leaves nonzero:
//   forward  X: one kernel reads the image rows, applies the separable
//               deconvolution factors, places each row into its zero-padded
//               length-Ntilde_0 line and transforms it (only image rows, y and
//               z inside the image);
//            Y: lines along y of the image z-slices, input read only at the
//               image rows (the others are zero), all outputs written;
//            Z: lines along z of every (x, y), input read only at the image
//               slices, all outputs written.
//   adjoint  Z', Y': the same lines backwards, writing only the outputs the
//               next step reads; X': transforms the image rows and writes the
//               cropped, deconvolved image.
// The grid ends up (forward) or is read (adjoint) exactly as the unpruned
// transform of the zero-padded grid.  Each CTA transforms W lines held in a
// shared-memory tile [position][line] (row pitch W+1: transfers along a line
// and butterflies across lines are both free of bank conflicts), loaded with
// asynchronous copies (cp.async, the whole tile in flight at once), with
// radix-8 Stockham passes (a final radix-2 or radix-4 pass for 128, 256,
// 1024) computed in registers; twiddles come from a per-length table
// exp(-2 pi i q / n) built on the host in FP64.  Unnormalised, forward sign
// -1 / backward +1, like FFTW's fft!/bfft!.
#include "nfft_internal.cuh"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace nfft {
namespace {

#ifndef NFFT_FFT_FOURSTEP
#define NFFT_FFT_FOURSTEP 1
#endif
#ifndef NFFT_FFT_THREADS
#define NFFT_FFT_THREADS 256
#endif
constexpr int kFftThreads = NFFT_FFT_THREADS;

template <typename T> using Cx = typename Cplx<T>::type;

template <typename C> __device__ __forceinline__ C c_add(C a, C b) {
  a.x += b.x;
  a.y += b.y;
  return a;
}
template <typename C> __device__ __forceinline__ C c_sub(C a, C b) {
  a.x -= b.x;
  a.y -= b.y;
  return a;
}
template <typename C> __device__ __forceinline__ C c_mul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
// a * (S i), S = -1 (forward) or +1 (backward)
template <int S, typename C> __device__ __forceinline__ C c_mul_si(C a) {
  C r;
  r.x = S > 0 ? -a.y : a.y;
  r.y = S > 0 ? a.x : -a.x;
  return r;
}

// In-register DFTs of length 2, 4, 8 with kernel exp(S 2 pi i t q / R),
// outputs in natural order.
template <int S, typename C> __device__ __forceinline__ void dft2(C (&v)[2]) {
  const C a = v[0];
  v[0] = c_add(a, v[1]);
  v[1] = c_sub(a, v[1]);
}
template <int S, typename C> __device__ __forceinline__ void dft4(C (&u)[4]) {
  const C c0 = c_add(u[0], u[2]), c1 = c_sub(u[0], u[2]);
  const C d0 = c_add(u[1], u[3]), d1 = c_mul_si<S>(c_sub(u[1], u[3]));
  u[0] = c_add(c0, d0);
  u[2] = c_sub(c0, d0);
  u[1] = c_add(c1, d1);
  u[3] = c_sub(c1, d1);
}
template <int S, typename C> __device__ __forceinline__ void dft8(C (&v)[8]) {
  using T = decltype(v[0].x);
  const T h = T(0.70710678118654752440084436210485);  // 1/sqrt(2)
  C a[4], b[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    a[t] = c_add(v[t], v[t + 4]);
    b[t] = c_sub(v[t], v[t + 4]);
  }
  // b[t] *= w^t, w = exp(S i pi / 4) = h (1 + S i)
  {
    const C s1 = c_mul_si<S>(b[1]);
    b[1].x = h * (b[1].x + s1.x);
    b[1].y = h * (b[1].y + s1.y);
    b[2] = c_mul_si<S>(b[2]);
    const C s3 = c_mul_si<S>(b[3]);
    b[3].x = h * (s3.x - b[3].x);
    b[3].y = h * (s3.y - b[3].y);
  }
  dft4<S>(a);
  dft4<S>(b);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    v[2 * q] = a[q];
    v[2 * q + 1] = b[q];
  }
}
template <int S, int R, typename C> __device__ __forceinline__ void dft(C (&v)[R]) {
  if constexpr (R == 8) dft8<S>(v);
  else if constexpr (R == 4) dft4<S>(v);
  else dft2<S>(v);
}

// One Stockham pass over the W lines of length N in buf[pos * (W + 1) + w]:
// butterfly j of line w loads positions j + r N/R, twiddles by
// (j mod NS) r / (NS R) turns, transforms, and stores at
// (j div NS) NS R + (j mod NS) + r NS.
template <typename T, int S, int N, int W, int R, int NS>
__device__ __forceinline__ void fft_pass(Cx<T>* buf, const Cx<T>* __restrict__ tw) {
  using C = Cx<T>;
  constexpr int NB = N / R;
  constexpr int TOT = NB * W;
  constexpr int BPT = (TOT + kFftThreads - 1) / kFftThreads;
  constexpr int P = W + 1;
  C v[BPT][R];
#pragma unroll
  for (int b = 0; b < BPT; ++b) {
    const int t = threadIdx.x + b * kFftThreads;
    if (TOT % kFftThreads == 0 || t < TOT) {
      const int w = t % W, j = t / W;
#pragma unroll
      for (int r = 0; r < R; ++r) v[b][r] = buf[(j + r * NB) * P + w];
    }
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < BPT; ++b) {
    const int t = threadIdx.x + b * kFftThreads;
    if (TOT % kFftThreads == 0 || t < TOT) {
      const int w = t % W, j = t / W;
      const int k = j & (NS - 1);
      if constexpr (NS > 1) {
        constexpr int STEP = N / (NS * R);
#pragma unroll
        for (int r = 1; r < R; ++r) {
          C tt = __ldg(tw + ((k * r * STEP) & (N - 1)));
          if constexpr (S > 0) tt.y = -tt.y;
          v[b][r] = c_mul(v[b][r], tt);
        }
      }
      dft<S, R>(v[b]);
      const int base = (j - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) buf[(base + r * NS) * P + w] = v[b][r];
    }
  }
  __syncthreads();
}

template <typename T, int S, int N, int W, int NS = 1>
__device__ __forceinline__ void fft_lines(Cx<T>* buf, const Cx<T>* __restrict__ tw) {
  if constexpr (NS < N) {
    constexpr int REM = N / NS;
    constexpr int R = REM % 8 == 0 ? 8 : REM;
    fft_pass<T, S, N, W, R, NS>(buf, tw);
    fft_lines<T, S, N, W, NS * R>(buf, tw);
  }
}

// 8- or 16-byte asynchronous global -> shared copy (cp.async, sm_80+): a
// tile's loads are all in flight at once, without register staging.
template <typename C> __device__ __forceinline__ void cp_async_elem(C* smem, const C* gmem) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  if constexpr (sizeof(C) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Pull one 128-byte line toward L2 ahead of its use (no register is held).
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];\n" ::"l"(p)); }

#ifndef NFFT_TOE_PREFETCH
#define NFFT_TOE_PREFETCH 1
#endif

// Move the W x n tile elements q = threadIdx.x + i * kFftThreads through
// registers in batches of up to 8: every load of a batch is issued before
// its stores, so a thread keeps a batch of global (or shared) loads in flight
// instead of one load-store round trip per element.
template <typename C, int ITEMS, typename Load, typename Store>
__device__ __forceinline__ void staged_copy(Load ld, Store st) {
  constexpr int CH = ITEMS < 8 ? ITEMS : 8;
  static_assert(ITEMS % CH == 0, "tile items per thread");
#pragma unroll 1
  for (int c0 = 0; c0 < ITEMS; c0 += CH) {
    C v[CH];
#pragma unroll
    for (int i = 0; i < CH; ++i) v[i] = ld(int(threadIdx.x) + (c0 + i) * kFftThreads);
#pragma unroll
    for (int i = 0; i < CH; ++i) st(int(threadIdx.x) + (c0 + i) * kFftThreads, v[i]);
  }
}

// CTAs per SM the register allocation must allow: 3 for the forward FP32
// kernels up to 512 (a few spilled bytes, measured faster), 2 for the
// backward ones (whose spills at 3 cost more than the occupancy gains),
// 1 for the largest lines.
template <typename T, int N, bool FWD> constexpr int fft_min_blocks() {
  if (kFftThreads > 256) return 1;
  return (sizeof(T) == 4 ? N <= 512 : N <= 256) ? ((sizeof(T) == 4 && FWD) ? 3 : 2) : 1;
}

struct FftGeom {
  int N[3], Nt[3];
  int64_t plane;  // Nt0 * Nt1
};

template <typename T> struct Inv3 {
  const T* d[3];
};

// forward X: image rows -> deconvolved, zero-padded, transformed grid rows
template <typename T, int NX, int W>
__global__ void __launch_bounds__(kFftThreads, fft_min_blocks<T, NX, true>()) fft_x_pad_kernel(FftGeom G, Inv3<T> inv, const Cx<T>* __restrict__ f,
                                                                Cx<T>* __restrict__ g, const Cx<T>* __restrict__ tw, void* const* slot) {
  using C = Cx<T>;
  if (slot) f = static_cast<const C*>(slot[0]);  // image pointer read from device memory
  extern __shared__ __align__(16) unsigned char fft_smem[];
  C* buf = reinterpret_cast<C*>(fft_smem);
  constexpr int P = W + 1;
  const int64_t rows = int64_t(G.N[1]) * G.N[2];
  const int64_t r0 = int64_t(blockIdx.x) * W;
  const int N0 = G.N[0], h0 = G.N[0] / 2;
  constexpr int ITEMS = NX * W / kFftThreads;
  // per row: the y / z deconvolution factor and the grid row offset
  __shared__ T s_row[W];
  __shared__ int64_t s_goff[W];
  if (threadIdx.x < W) {
    const int64_t r = r0 + threadIdx.x;
    T s = T(0);
    int64_t go = 0;
    if (r < rows) {
      const int y = int(r % G.N[1]), z = int(r / G.N[1]);
      s = __ldg(inv.d[1] + y) * __ldg(inv.d[2] + z);
      go = int64_t(NX) * (wrap_once(y - G.N[1] / 2, G.Nt[1]) +
                          int64_t(G.Nt[1]) * wrap_once(z - G.N[2] / 2, G.Nt[2]));
    }
    s_row[threadIdx.x] = s;
    s_goff[threadIdx.x] = go;
  }
  __syncthreads();
  // raw image values land asynchronously; padding positions are zeroed
#pragma unroll 4
  for (int i = 0; i < ITEMS; ++i) {
    const int q = int(threadIdx.x) + i * kFftThreads;
    const int pos = q % NX, w = q / NX;
    const int nx = wrap_once(pos + h0, NX);
    if (r0 + w < rows && nx < N0) {
      cp_async_elem(buf + pos * P + w, f + nx + int64_t(N0) * (r0 + w));
    } else {
      C z;
      z.x = T(0);
      z.y = T(0);
      buf[pos * P + w] = z;
    }
  }
  cp_async_wait_all();
  __syncthreads();
  // deconvolution factors (each thread scales the elements it copied)
#pragma unroll 4
  for (int i = 0; i < ITEMS; ++i) {
    const int q = int(threadIdx.x) + i * kFftThreads;
    const int pos = q % NX, w = q / NX;
    const int nx = wrap_once(pos + h0, NX);
    if (nx < N0) {
      const T sc = __ldg(inv.d[0] + nx) * s_row[w];
      C v = buf[pos * P + w];
      v.x *= sc;
      v.y *= sc;
      buf[pos * P + w] = v;
    }
  }
  __syncthreads();
  fft_lines<T, -1, NX, W>(buf, tw);
  staged_copy<C, ITEMS>([&](int q) { return buf[(q % NX) * P + q / NX]; },
                        [&](int q, C v) {
                          if (r0 + q / NX < rows) g[s_goff[q / NX] + q % NX] = v;
                        });
}

// adjoint X': grid rows of the image -> transformed, cropped, deconvolved image rows
template <typename T, int NX, int W>
__global__ void __launch_bounds__(kFftThreads, fft_min_blocks<T, NX, false>()) fft_x_crop_kernel(FftGeom G, Inv3<T> inv, const Cx<T>* __restrict__ g,
                                                                 Cx<T>* __restrict__ f, const Cx<T>* __restrict__ tw, void* const* slot) {
  if (slot) f = static_cast<Cx<T>*>(slot[0]);  // image pointer read from device memory
  using C = Cx<T>;
  extern __shared__ __align__(16) unsigned char fft_smem[];
  C* buf = reinterpret_cast<C*>(fft_smem);
  constexpr int P = W + 1;
  const int64_t rows = int64_t(G.N[1]) * G.N[2];
  const int64_t r0 = int64_t(blockIdx.x) * W;
  const int N0 = G.N[0], h0 = G.N[0] / 2;
  constexpr int ITEMS = NX * W / kFftThreads;
  __shared__ T s_row[W];
  __shared__ int64_t s_goff[W];
  if (threadIdx.x < W) {
    const int64_t r = r0 + threadIdx.x;
    T s = T(0);
    int64_t go = 0;
    if (r < rows) {
      const int y = int(r % G.N[1]), z = int(r / G.N[1]);
      s = __ldg(inv.d[1] + y) * __ldg(inv.d[2] + z);
      go = int64_t(NX) * (wrap_once(y - G.N[1] / 2, G.Nt[1]) +
                          int64_t(G.Nt[1]) * wrap_once(z - G.N[2] / 2, G.Nt[2]));
    }
    s_row[threadIdx.x] = s;
    s_goff[threadIdx.x] = go;
  }
  __syncthreads();
#pragma unroll 4
  for (int i = 0; i < ITEMS; ++i) {
    const int q = int(threadIdx.x) + i * kFftThreads;
    const int pos = q % NX, w = q / NX;
    if (r0 + w < rows) {
      cp_async_elem(buf + pos * P + w, g + s_goff[w] + pos);
    } else {
      C z;
      z.x = T(0);
      z.y = T(0);
      buf[pos * P + w] = z;
    }
  }
  cp_async_wait_all();
  __syncthreads();
  fft_lines<T, 1, NX, W>(buf, tw);
  staged_copy<C, ITEMS>([&](int q) { return buf[(q % NX) * P + q / NX]; },
                        [&](int q, C v) {
                          const int pos = q % NX, w = q / NX;
                          const int nx = wrap_once(pos + h0, NX);
                          if (r0 + w < rows && nx < N0) {
                            const T s = __ldg(inv.d[0] + nx) * s_row[w];
                            v.x *= s;
                            v.y *= s;
                            f[nx + int64_t(N0) * (r0 + w)] = v;
                          }
                        });
}

// Lines of length NL along an axis with element stride `stride`; a CTA takes
// W consecutive x of one outer index.  The outer index o runs over the image
// positions of a pruned outer dimension (outer_N > 0: grid index
// (o - outer_N/2) mod outer_Nt) or over all grid positions (outer_N = 0).
// FWD: input read only at the line's image positions (the rest is zero), all
// outputs written.  Otherwise: all inputs read, only image positions written.
struct LineGeom {
  int64_t stride;       // elements between consecutive line positions
  int64_t outer_stride; // elements between consecutive outer grid indices
  int tiles_x;          // Nt0 / W
  int n_img;            // image length along the line
  int outer_N, outer_Nt;
};

template <typename T, int NL, int W, bool FWD>
__global__ void __launch_bounds__(kFftThreads, fft_min_blocks<T, NL, FWD>()) fft_lines_kernel(LineGeom L, Cx<T>* __restrict__ g,
                                                                const Cx<T>* __restrict__ tw) {
  using C = Cx<T>;
  extern __shared__ __align__(16) unsigned char fft_smem[];
  C* buf = reinterpret_cast<C*>(fft_smem);
  constexpr int P = W + 1;
  const int tile = blockIdx.x % L.tiles_x;
  const int o = blockIdx.x / L.tiles_x;
  const int go = L.outer_N > 0 ? wrap_once(o - L.outer_N / 2, L.outer_Nt) : o;
  C* base = g + int64_t(go) * L.outer_stride + int64_t(tile) * W;
  const int head = L.n_img - L.n_img / 2;   // image positions [0, head) and [NL - n_img/2, NL)
  const int tail0 = NL - L.n_img / 2;
  // thread -> fixed column w, positions p0, p0 + PS, ...
  constexpr int PS = kFftThreads / W;
  const int w = threadIdx.x % W, p0 = threadIdx.x / W;
  const C* src = base + w + int64_t(p0) * L.stride;
  const int64_t step = int64_t(PS) * L.stride;
#pragma unroll 4
  for (int pos = p0; pos < NL; pos += PS, src += step) {
    if (!FWD || pos < head || pos >= tail0) {
      cp_async_elem(buf + pos * P + w, src);
    } else {
      C z;
      z.x = T(0);
      z.y = T(0);
      buf[pos * P + w] = z;
    }
  }
  cp_async_wait_all();
  __syncthreads();
  fft_lines<T, FWD ? -1 : 1, NL, W>(buf, tw);
  C* dst = base + w + int64_t(p0) * L.stride;
#pragma unroll 4
  for (int pos = p0; pos < NL; pos += PS, dst += step)
    if (FWD || pos < head || pos >= tail0) *dst = buf[pos * P + w];
}

// Toeplitz convolution along the last axis with the shared-memory Stockham
// passes (FP64, and FP32 lines of 1024): pruned load, forward FFT, product
// with lambda times `scale`, backward FFT, pruned store.
template <typename T, int NL, int W>
__global__ void __launch_bounds__(kFftThreads, fft_min_blocks<T, NL, false>()) fft_toeplitz_lines_kernel(
    LineGeom L, Cx<T>* __restrict__ g, const Cx<T>* __restrict__ lam, T scale, const Cx<T>* __restrict__ tw) {
  using C = Cx<T>;
  extern __shared__ __align__(16) unsigned char fft_smem[];
  C* buf = reinterpret_cast<C*>(fft_smem);
  constexpr int P = W + 1;
  const int tile = blockIdx.x % L.tiles_x;
  const int o = blockIdx.x / L.tiles_x;
  const int go = L.outer_N > 0 ? wrap_once(o - L.outer_N / 2, L.outer_Nt) : o;
  const int64_t off = int64_t(go) * L.outer_stride + int64_t(tile) * W;
  C* base = g + off;
  const int head = L.n_img - L.n_img / 2;
  const int tail0 = NL - L.n_img / 2;
  if (NFFT_TOE_PREFETCH)
    for (int r = threadIdx.x; r < NL; r += kFftThreads) prefetch_l2(lam + off + int64_t(r) * L.stride);
  constexpr int PS = kFftThreads / W;
  const int w = threadIdx.x % W, p0 = threadIdx.x / W;
  const int64_t step = int64_t(PS) * L.stride;
  const C* src = base + w + int64_t(p0) * L.stride;
#pragma unroll 4
  for (int pos = p0; pos < NL; pos += PS, src += step) {
    if (pos < head || pos >= tail0) {
      cp_async_elem(buf + pos * P + w, src);
    } else {
      C z;
      z.x = T(0);
      z.y = T(0);
      buf[pos * P + w] = z;
    }
  }
  cp_async_wait_all();
  __syncthreads();
  fft_lines<T, -1, NL, W>(buf, tw);
  const C* lsrc = lam + off + w + int64_t(p0) * L.stride;
#pragma unroll 4
  for (int pos = p0; pos < NL; pos += PS, lsrc += step) {
    C l = __ldg(lsrc);
    l.x *= scale;
    l.y *= scale;
    buf[pos * P + w] = c_mul(buf[pos * P + w], l);
  }
  __syncthreads();
  fft_lines<T, 1, NL, W>(buf, tw);
  C* dst = base + w + int64_t(p0) * L.stride;
#pragma unroll 4
  for (int pos = p0; pos < NL; pos += PS, dst += step)
    if (pos < head || pos >= tail0) *dst = buf[pos * P + w];
}

#ifndef NFFT_FFT_W32
#define NFFT_FFT_W32 16
#endif
#ifndef NFFT_FFT_W64
#define NFFT_FFT_W64 8
#endif
template <typename T> constexpr int lines_per_cta() { return sizeof(T) == 4 ? NFFT_FFT_W32 : NFFT_FFT_W64; }

template <int NL, typename T> size_t fft_smem_bytes() {
  return size_t(NL) * (lines_per_cta<T>() + 1) * sizeof(Cx<T>);
}


// ---------------------------------------------------------------------------
// FP32 lines of length N <= 512: four-step FFT in registers.  N = R1 R2;
// pass 1 loads the R1 points n = R2 n1 + n2 of a line straight from global
// memory into registers, transforms them (DFT of length R1), applies the
// twiddles exp(S 2 pi i n2 k1 / N) and writes them to shared memory; pass 2
// reads the R2 values of one k1, transforms them (DFT of length R2) and
// writes X[k1 + R1 k2] straight to global memory.  A point crosses shared
// memory once (16 bytes of shared traffic against 64 for the Stockham
// passes), which keeps the kernel on the HBM side of its bounds.

// cos(2 pi j / 32)
__host__ __device__ constexpr double cos32(int j) {
  switch (j & 31) {
    case 0: return 1.0;
    case 1: case 31: return 0.9807852804032304491261822;
    case 2: case 30: return 0.9238795325112867561281832;
    case 3: case 29: return 0.8314696123025452370787884;
    case 4: case 28: return 0.7071067811865475244008444;
    case 5: case 27: return 0.5555702330196022247428308;
    case 6: case 26: return 0.3826834323650897717284600;
    case 7: case 25: return 0.1950903220161282678482849;
    case 8: case 24: return 0.0;
    case 9: case 23: return -0.1950903220161282678482849;
    case 10: case 22: return -0.3826834323650897717284600;
    case 11: case 21: return -0.5555702330196022247428308;
    case 12: case 20: return -0.7071067811865475244008444;
    case 13: case 19: return -0.8314696123025452370787884;
    case 14: case 18: return -0.9238795325112867561281832;
    case 15: case 17: return -0.9807852804032304491261822;
    default: return -1.0;  // 16
  }
}

// In-register DFT of length R (2..32), natural order, kernel exp(S 2 pi i t q / R):
// radix 2/4/8 directly, 16 and 32 by an even/odd split.
template <int S, int R, typename C> __device__ __forceinline__ void dft_reg(C (&v)[R]) {
  using T = decltype(v[0].x);
  if constexpr (R <= 8) {
    dft<S, R>(v);
  } else {
    C e[R / 2], o[R / 2];
#pragma unroll
    for (int t = 0; t < R / 2; ++t) {
      e[t] = v[2 * t];
      o[t] = v[2 * t + 1];
    }
    dft_reg<S, R / 2>(e);
    dft_reg<S, R / 2>(o);
#pragma unroll
    for (int k = 0; k < R / 2; ++k) {
      const int j = k * (32 / R);
      const T c = T(cos32(j)), sn = T(S) * T(cos32(j - 8));
      C t;
      t.x = o[k].x * c - o[k].y * sn;
      t.y = o[k].x * sn + o[k].y * c;
      v[k] = c_add(e[k], t);
      v[k + R / 2] = c_sub(e[k], t);
    }
  }
}

template <int N> struct Split4 {
  static constexpr int R1 = N == 64 ? 8 : N == 128 ? 8 : N == 256 ? 16 : 16;
  static constexpr int R2 = N / R1;
};

// v[k1] *= exp(S 2 pi i n2 k1 / N) for k1 >= 1 (table of exp(-2 pi i q / N))
template <int S, int N, int R1, typename C>
__device__ __forceinline__ void twiddle4(C (&v)[R1], int n2, const C* __restrict__ tw) {
  if (n2 == 0) return;
#pragma unroll
  for (int k1 = 1; k1 < R1; ++k1) {
    C tt = __ldg(tw + ((n2 * k1) & (N - 1)));
    if constexpr (S > 0) tt.y = -tt.y;
    v[k1] = c_mul(v[k1], tt);
  }
}

constexpr int kW4 = 16;  // lines per CTA

// Split of the fused Toeplitz pass (fft4_toeplitz_kernel): 512 = 32 x 16, so
// the 16-point pass carries the twiddles and the kernel product (no spills
// at two CTAs per SM; 16 x 32 spills).
#ifndef NFFT_TOE_R1_512
#define NFFT_TOE_R1_512 32
#endif
#ifndef NFFT_TOE_MINB
#define NFFT_TOE_MINB 2
#endif
template <int N> struct ToeSplit {
  static constexpr int R1 = N == 512 ? NFFT_TOE_R1_512 : Split4<N>::R1;
  static constexpr int R2 = N / R1;
};

template <int NL, bool FWD>
__global__ void __launch_bounds__(256, FWD ? 3 : 2) fft4_lines_kernel(LineGeom L, float2* __restrict__ g,
                                                                      const float2* __restrict__ tw) {
  using C = float2;
  constexpr int R1 = Split4<NL>::R1, R2 = Split4<NL>::R2, W = kW4, P = W + 1, S = FWD ? -1 : 1;
  extern __shared__ __align__(16) unsigned char fft_smem[];
  C* y = reinterpret_cast<C*>(fft_smem);
  const int tile = blockIdx.x % L.tiles_x;
  const int o = blockIdx.x / L.tiles_x;
  const int go = L.outer_N > 0 ? wrap_once(o - L.outer_N / 2, L.outer_Nt) : o;
  C* base = g + int64_t(go) * L.outer_stride + int64_t(tile) * W;
  const int head = L.n_img - L.n_img / 2, tail0 = NL - L.n_img / 2;
  constexpr int T1 = W * R2, B1 = (T1 + 255) / 256;
#pragma unroll
  for (int b = 0; b < B1; ++b) {
    const int task = int(threadIdx.x) + b * 256;
    if (T1 % 256 == 0 || task < T1) {
      const int w = task % W, n2 = task / W;
      C v[R1];
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1) {
        const int n = R2 * n1 + n2;
        v[n1].x = 0.f;
        v[n1].y = 0.f;
        if (!FWD || n < head || n >= tail0) v[n1] = base[w + int64_t(n) * L.stride];
      }
      dft_reg<S, R1>(v);
      twiddle4<S, NL, R1>(v, n2, tw);
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) y[(n2 * R1 + k1) * P + w] = v[k1];
    }
  }
  __syncthreads();
  constexpr int T2 = W * R1, B2 = (T2 + 255) / 256;
#pragma unroll
  for (int b = 0; b < B2; ++b) {
    const int task = int(threadIdx.x) + b * 256;
    if (T2 % 256 == 0 || task < T2) {
      const int w = task % W, k1 = task / W;
      C v[R2];
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) v[n2] = y[(n2 * R1 + k1) * P + w];
      dft_reg<S, R2>(v);
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) {
        const int pos = k1 + R1 * k2;
        if (FWD || pos < head || pos >= tail0) base[w + int64_t(pos) * L.stride] = v[k2];
      }
    }
  }
}

// Marks, for every block of kW4 x columns and every y of the (centred)
// grid, the 8-position z groups that the padded tile of some bin with nodes
// covers: bin tile t spans x [o0 - m - 1, o0 + bx + m), y and z
// [o - m, o + b + m) around its origin o (+ the grid shift sh, modulo Ntilde).
__global__ void zmask_kernel(const int32_t* __restrict__ tstart, int nt0, int nt1, int nt2, int bx, int by, int bz,
                             int m, int Nt0, int Nt1, int Nt2, int sh0, int sh1, int sh2, int tiles_x,
                             unsigned long long* __restrict__ zmask) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= int64_t(nt0) * nt1 * nt2 || tstart[t + 1] == tstart[t]) return;
  const int tx = int(t % nt0), ty = int((t / nt0) % nt1), tz = int(t / (int64_t(nt0) * nt1));
  const int ox = tx * bx + sh0, oy = ty * by + sh1, oz = tz * bz + sh2;
  unsigned long long bits = 0;
  for (int z = oz - m; z < oz + bz + m; ++z) bits |= 1ull << (wrap_any(z, Nt2) >> 3);
  const int x0 = ox - m - 1, x1 = ox + bx + m - 1;
  for (int y = oy - m; y < oy + by + m; ++y) {
    unsigned long long* row = zmask + int64_t(wrap_any(y, Nt1)) * tiles_x;
    for (int x = x0;; x += kW4) {
      const int xc = x < x1 ? x : x1;
      atomicOr(row + wrap_any(xc, Nt0) / kW4, bits);
      if (xc == x1) break;
    }
  }
}

// The same four-step line FFT with the CTA's W x NL tile staged in shared
// memory first: every thread issues its share of 16-byte cp.async copies of
// the tile at once (the forward copies only the image rows), so a CTA has
// its whole tile in flight without holding it in registers.  The tile is
// row-major [position][W columns] without padding and the FFT runs in place:
// the R1-point DFTs of column w, offset n2 write their outputs to the rows
// they read (row R2 k1 + n2), and the R2-point DFTs of k1 read rows
// R2 k1 .. R2 k1 + R2 - 1; half-warps cover the 16 columns of one row in every
// access, so no access has a bank conflict.  W x NL x 8 bytes of shared
// memory (64 KB at NL = 512).
//
// MASK = 2 (z lines): bit b of zmask[y * tiles_x + x tile] says whether grid
// positions z in [8 b, 8 b + 8) of those lines lie in the padded tile of some
// bin with nodes.  The forward writes only those positions (the gather reads
// nothing else; a line block with no such position is skipped), the inverse
// reads only those (the spreading wrote nothing else into the zeroed grid)
// and skips blocks with none: their lines are zero, and so is their
// transform, which the zeroed grid already holds.  MASK = 0: no mask.
template <int NL, bool FWD, int MASK>
__global__ void __launch_bounds__(256, 3) fft4_lines_staged_kernel(LineGeom L, float2* __restrict__ g,
                                                                   const float2* __restrict__ tw,
                                                                   const unsigned long long* __restrict__ zmask) {
  using C = float2;
  constexpr int R1 = Split4<NL>::R1, R2 = Split4<NL>::R2, W = kW4, S = FWD ? -1 : 1;
  static_assert(W == 16, "a row of the tile is 8 16-byte chunks");
  extern __shared__ __align__(16) unsigned char fft_smem[];
  C* buf = reinterpret_cast<C*>(fft_smem);
  const int tile = blockIdx.x % L.tiles_x;
  const int o = blockIdx.x / L.tiles_x;
  const int go = L.outer_N > 0 ? wrap_once(o - L.outer_N / 2, L.outer_Nt) : o;
  C* base = g + int64_t(go) * L.outer_stride + int64_t(tile) * W;
  const int head = L.n_img - L.n_img / 2, tail0 = NL - L.n_img / 2;
  const unsigned long long live = MASK == 2 ? __ldg(zmask + int64_t(o) * L.tiles_x + tile) : ~0ull;
  if (MASK == 2 && live == 0) return;  // nothing of these lines is read (forward) or non-zero (inverse)
  auto used = [&](int pos) { return MASK != 2 || ((live >> (pos >> 3)) & 1ull) != 0; };
  // stage the tile: NL rows of W complex values (8 chunks of 16 bytes)
  for (int c = threadIdx.x; c < NL * 8; c += 256) {
    const int row = c >> 3, part = c & 7;
    if ((!FWD || row < head || row >= tail0) && (FWD || used(row))) {
      const unsigned dst = static_cast<unsigned>(__cvta_generic_to_shared(buf + row * W + 2 * part));
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst),
                   "l"(base + int64_t(row) * L.stride + 2 * part)
                   : "memory");
    }
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
  // R1-point DFTs in place: thread (w, n2) owns rows R2 n1 + n2 of column w
  constexpr int T1 = W * R2, B1 = (T1 + 255) / 256;
#pragma unroll
  for (int b = 0; b < B1; ++b) {
    const int task = int(threadIdx.x) + b * 256;
    if (T1 % 256 == 0 || task < T1) {
      const int w = task % W, n2 = task / W;
      C v[R1];
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1) {
        const int n = R2 * n1 + n2;
        v[n1].x = 0.f;
        v[n1].y = 0.f;
        if ((!FWD || n < head || n >= tail0) && (FWD || used(n))) v[n1] = buf[n * W + w];
      }
      dft_reg<S, R1>(v);
      twiddle4<S, NL, R1>(v, n2, tw);
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) buf[(R2 * k1 + n2) * W + w] = v[k1];
    }
  }
  __syncthreads();
  // R2-point DFTs: thread (w, k1) reads rows R2 k1 .. R2 k1 + R2 - 1
  constexpr int T2 = W * R1, B2 = (T2 + 255) / 256;
#pragma unroll
  for (int b = 0; b < B2; ++b) {
    const int task = int(threadIdx.x) + b * 256;
    if (T2 % 256 == 0 || task < T2) {
      const int w = task % W, k1 = task / W;
      C v[R2];
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) v[n2] = buf[(R2 * k1 + n2) * W + w];
      dft_reg<S, R2>(v);
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) {
        const int pos = k1 + R1 * k2;
        if ((FWD && used(pos)) || (!FWD && (pos < head || pos >= tail0))) base[w + int64_t(pos) * L.stride] = v[k2];
      }
    }
  }
}

// x lines of the image rows: forward pad + deconvolution + FFT (FWD), or
// backward FFT + crop + deconvolution.
template <int NX, bool FWD>
__global__ void __launch_bounds__(256, FWD ? 3 : 2) fft4_x_kernel(FftGeom G, Inv3<float> inv,
                                                                  const float2* __restrict__ src,
                                                                  float2* __restrict__ dst,
                                                                  const float2* __restrict__ tw,
                                                                  void* const* slot) {
  using C = float2;
  constexpr int R1 = Split4<NX>::R1, R2 = Split4<NX>::R2, W = kW4, PR = R1 + 1, PW = R2 * PR, S = FWD ? -1 : 1;
  if (slot) {  // the image pointer is read from device memory (graph replays with new arrays)
    if (FWD) src = static_cast<const float2*>(slot[0]);
    else dst = static_cast<float2*>(slot[0]);
  }
  extern __shared__ __align__(16) unsigned char fft_smem[];
  C* y = reinterpret_cast<C*>(fft_smem);
  __shared__ float s_row[W];
  __shared__ int64_t s_goff[W];
  const int64_t rows = int64_t(G.N[1]) * G.N[2];
  const int64_t r0 = int64_t(blockIdx.x) * W;
  const int N0 = G.N[0], h0 = G.N[0] / 2;
  if (threadIdx.x < W) {
    const int64_t r = r0 + threadIdx.x;
    float sc = 0.f;
    int64_t goff = 0;
    if (r < rows) {
      const int yy = int(r % G.N[1]), zz = int(r / G.N[1]);
      sc = __ldg(inv.d[1] + yy) * __ldg(inv.d[2] + zz);
      goff = int64_t(NX) * (wrap_once(yy - G.N[1] / 2, G.Nt[1]) +
                            int64_t(G.Nt[1]) * wrap_once(zz - G.N[2] / 2, G.Nt[2]));
    }
    s_row[threadIdx.x] = sc;
    s_goff[threadIdx.x] = goff;
  }
  __syncthreads();
  constexpr int T1 = W * R2, B1 = (T1 + 255) / 256;
#pragma unroll
  for (int b = 0; b < B1; ++b) {
    const int task = int(threadIdx.x) + b * 256;
    if (T1 % 256 == 0 || task < T1) {
      const int n2 = task % R2, w = task / R2;
      const bool live = r0 + w < rows;
      C v[R1];
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1) {
        const int n = R2 * n1 + n2;
        v[n1].x = 0.f;
        v[n1].y = 0.f;
        if (FWD) {
          const int nx = wrap_once(n + h0, NX);
          if (live && nx < N0) {
            const C a = src[nx + int64_t(N0) * (r0 + w)];
            const float sc = __ldg(inv.d[0] + nx) * s_row[w];
            v[n1].x = a.x * sc;
            v[n1].y = a.y * sc;
          }
        } else if (live) {
          v[n1] = src[s_goff[w] + n];
        }
      }
      dft_reg<S, R1>(v);
      twiddle4<S, NX, R1>(v, n2, tw);
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) y[w * PW + n2 * PR + k1] = v[k1];
    }
  }
  __syncthreads();
  constexpr int T2 = W * R1, B2 = (T2 + 255) / 256;
#pragma unroll
  for (int b = 0; b < B2; ++b) {
    const int task = int(threadIdx.x) + b * 256;
    if (T2 % 256 == 0 || task < T2) {
      const int k1 = task % R1, w = task / R1;
      if (r0 + w < rows) {
        C v[R2];
#pragma unroll
        for (int n2 = 0; n2 < R2; ++n2) v[n2] = y[w * PW + n2 * PR + k1];
        dft_reg<S, R2>(v);
#pragma unroll
        for (int k2 = 0; k2 < R2; ++k2) {
          const int pos = k1 + R1 * k2;
          if (FWD) {
            dst[s_goff[w] + pos] = v[k2];
          } else {
            const int nx = wrap_once(pos + h0, NX);
            if (nx < N0) {
              const float sc = __ldg(inv.d[0] + nx) * s_row[w];
              C out;
              out.x = v[k2].x * sc;
              out.y = v[k2].y * sc;
              dst[nx + int64_t(N0) * (r0 + w)] = out;
            }
          }
        }
      }
    }
  }
}

// Toeplitz convolution along the last axis (NFFTTools' convolveToeplitzKernel!):
// forward FFT of the line's image positions, product with the kernel lambda
// times `scale`, backward FFT, write back the image positions -- the
// transformed line never leaves the CTA.  N = R1 R2 with n = R2 n1 + n2 and
// k = k1 + R1 k2:
//   pass 1 (thread per n2): length-R1 DFT over n1 of the image positions;
//   pass 2 (thread per k1): twiddle e^{-2 pi i n2 k1/N}, length-R2 DFT over
//     n2 (now X[k1 + R1 k2]), product with lambda, backward length-R2 DFT
//     over k2, twiddle e^{+2 pi i k1 n2/N} -- the same table entries as the
//     forward twiddle, loaded once; it reads and writes the same shared-memory
//     slots, so no barrier separates the halves;
//   pass 3 (thread per n2): backward length-R1 DFT, image positions written.
// Both twiddles sit in the pass over R2 points, which keeps the pass over R1
// points free of table loads.  The image occupies positions [0, N/4) and
// [3N/4, N) (the grid is twice the image), i.e. n1 in [0, R1/4) and
// [3R1/4, R1) -- compile-time in the unrolled loops.
template <int NL>
__global__ void __launch_bounds__(256, NFFT_TOE_MINB) fft4_toeplitz_kernel(LineGeom L, float2* __restrict__ g,
                                                                           const float2* __restrict__ lam, float scale,
                                                                           const float2* __restrict__ tw) {
  using C = float2;
  constexpr int R1 = ToeSplit<NL>::R1, R2 = ToeSplit<NL>::R2, W = kW4, P = W + 1;
  static_assert(R1 % 4 == 0, "image quarter of the R1 index");
  extern __shared__ __align__(16) unsigned char fft_smem[];
  C* y = reinterpret_cast<C*>(fft_smem);
  const int tile = blockIdx.x % L.tiles_x;
  const int o = blockIdx.x / L.tiles_x;
  const int go = L.outer_N > 0 ? wrap_once(o - L.outer_N / 2, L.outer_Nt) : o;
  const int64_t off = int64_t(go) * L.outer_stride + int64_t(tile) * W;
  C* base = g + off;
  const C* lbase = lam + off;
  if (NFFT_TOE_PREFETCH && NL >= 512) {
    // the CTA's kernel tile (NL rows of W values = one 128-byte line each)
    // streams into L2 while pass 1 loads and transforms; pass 2 reads it
    // there (measured: 512-point lines 4 % faster, 256-point lines slower)
    for (int r = threadIdx.x; r < NL; r += 256) prefetch_l2(lbase + int64_t(r) * L.stride);
  }
  constexpr int T1 = W * R2, B1 = (T1 + 255) / 256;
#pragma unroll
  for (int b = 0; b < B1; ++b) {
    const int task = int(threadIdx.x) + b * 256;
    if (T1 % 256 == 0 || task < T1) {
      const int w = task % W, n2 = task / W;
      C v[R1];
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1) {
        v[n1].x = 0.f;
        v[n1].y = 0.f;
        if (n1 < R1 / 4 || n1 >= 3 * R1 / 4) v[n1] = base[w + int64_t(R2 * n1 + n2) * L.stride];
      }
      dft_reg<-1, R1>(v);
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) y[(n2 * R1 + k1) * P + w] = v[k1];
    }
  }
  __syncthreads();
  constexpr int T2 = W * R1, B2 = (T2 + 255) / 256;
#pragma unroll
  for (int b = 0; b < B2; ++b) {
    const int task = int(threadIdx.x) + b * 256;
    if (T2 % 256 == 0 || task < T2) {
      const int w = task % W, k1 = task / W;
      C v[R2], t[R2];
      t[0].x = 1.f;
      t[0].y = 0.f;
#pragma unroll
      for (int n2 = 1; n2 < R2; ++n2) t[n2] = __ldg(tw + ((n2 * k1) & (NL - 1)));
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) v[n2] = c_mul(y[(n2 * R1 + k1) * P + w], t[n2]);
      dft_reg<-1, R2>(v);
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) {
        C l = __ldg(lbase + w + int64_t(k1 + R1 * k2) * L.stride);
        l.x *= scale;
        l.y *= scale;
        v[k2] = c_mul(v[k2], l);
      }
      dft_reg<1, R2>(v);
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) {
        C c = t[n2];
        c.y = -c.y;
        y[(n2 * R1 + k1) * P + w] = c_mul(v[n2], c);
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < B1; ++b) {
    const int task = int(threadIdx.x) + b * 256;
    if (T1 % 256 == 0 || task < T1) {
      const int w = task % W, n2 = task / W;
      C v[R1];
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) v[k1] = y[(n2 * R1 + k1) * P + w];
      dft_reg<1, R1>(v);
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1)
        if (n1 < R1 / 4 || n1 >= 3 * R1 / 4) base[w + int64_t(R2 * n1 + n2) * L.stride] = v[n1];
    }
  }
}

template <int N> size_t fft4_smem_bytes() { return size_t(N) * (kW4 + 1) * sizeof(float2); }

FftGeom make_fft_geom(const nfft_plan* p) {
  FftGeom G{};
  for (int d = 0; d < 3; ++d) {
    G.N[d] = int(p->N[d]);
    G.Nt[d] = int(p->Nt[d]);
  }
  G.plane = p->Nt[0] * p->Nt[1];
  return G;
}

template <typename T> Inv3<T> make_inv3(const nfft_plan* p) {
  const T* inv = static_cast<const T*>(p->cur_center ? p->inv_c : p->inv);
  const T* one = inv + (p->N[0] + (p->D > 1 ? p->N[1] : 0) + (p->D > 2 ? p->N[2] : 0));
  Inv3<T> I;
  I.d[0] = inv;
  I.d[1] = p->D > 1 ? inv + p->N[0] : one;
  I.d[2] = p->D > 2 ? inv + p->N[0] + p->N[1] : one;
  return I;
}

template <typename K> int set_smem(K kern, size_t bytes) {
  NFFT_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
  return NFFT_OK;
}

template <typename T, int NX> int x_pass_t(nfft_plan* p, const void* src, void* dst, bool fwd, void* const* slot) {
  using C = Cx<T>;
  if constexpr (sizeof(T) == 4 && NX <= 512 && NFFT_FFT_FOURSTEP) {
    const size_t smem = size_t(kW4) * Split4<NX>::R2 * (Split4<NX>::R1 + 1) * sizeof(float2);
    const unsigned blocks = unsigned((p->N[1] * p->N[2] + kW4 - 1) / kW4);
    const float2* tw = static_cast<const float2*>(p->fft_tw[0]);
    auto kern = fwd ? fft4_x_kernel<NX, true> : fft4_x_kernel<NX, false>;
    if (int rc = set_smem(kern, smem)) return rc;
    kern<<<blocks, 256, smem, p->stream>>>(make_fft_geom(p), make_inv3<float>(p), static_cast<const float2*>(src),
                                           static_cast<float2*>(dst), tw, slot);
    NFFT_LAUNCH_CHECK();
    return NFFT_OK;
  }
  constexpr int W = lines_per_cta<T>();
  const size_t smem = fft_smem_bytes<NX, T>();
  const int64_t rows = p->N[1] * p->N[2];
  const unsigned blocks = unsigned((rows + W - 1) / W);
  const C* tw = static_cast<const C*>(p->fft_tw[0]);
  if (fwd) {
    auto kern = fft_x_pad_kernel<T, NX, W>;
    if (int rc = set_smem(kern, smem)) return rc;
    kern<<<blocks, kFftThreads, smem, p->stream>>>(make_fft_geom(p), make_inv3<T>(p), static_cast<const C*>(src),
                                                   static_cast<C*>(dst), tw, slot);
  } else {
    auto kern = fft_x_crop_kernel<T, NX, W>;
    if (int rc = set_smem(kern, smem)) return rc;
    kern<<<blocks, kFftThreads, smem, p->stream>>>(make_fft_geom(p), make_inv3<T>(p), static_cast<const C*>(src),
                                                   static_cast<C*>(dst), tw, slot);
  }
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

// Line geometry of a pass along `axis` (1: y, 2: z) with W lines per CTA.
LineGeom make_line_geom(const nfft_plan* p, int axis, int W, int64_t* outer_count) {
  LineGeom L{};
  L.tiles_x = int(p->Nt[0] / W);
  L.n_img = int(p->N[axis]);
  if (axis == 1) {  // y lines of the image z-slices (D = 3) or of the single plane (D = 2)
    L.stride = p->Nt[0];
    L.outer_stride = p->Nt[0] * p->Nt[1];
    L.outer_N = p->D == 3 ? int(p->N[2]) : 0;
    L.outer_Nt = int(p->Nt[2]);
    *outer_count = p->D == 3 ? p->N[2] : 1;
  } else {          // z lines of every (x, y)
    L.stride = p->Nt[0] * p->Nt[1];
    L.outer_stride = p->Nt[0];
    L.outer_N = 0;
    L.outer_Nt = int(p->Nt[1]);
    *outer_count = p->Nt[1];
  }
  return L;
}

// The plan's z-line mask (see fft4_lines_staged_kernel), rebuilt when the
// nodes, the tile shape or the grid shift changed; null when it does not
// apply (not a 3-D FP32 binned plan on the staged path, z longer than 512,
// NFFT_GB300_FFT_PRUNE=0) or would have to be built inside a stream capture.
// Either pass may run with or without it: the passes agree on every value
// the gather reads and on every value of the inverse.
static const unsigned long long* zmask_for(nfft_plan* p) {
  if (!p->fft_prune || p->D != 3 || p->precision != 32 || !p->prm.blocking || !p->tile_start || !p->has_nodes)
    return nullptr;
  if (p->Nt[2] > 512 || p->Nt[2] % 8 != 0 || p->Nt[0] % kW4 != 0) return nullptr;
  int sh[3];
  for (int d = 0; d < 3; ++d) sh[d] = p->cur_center ? int(p->sh[d]) : 0;
  const int64_t key = (((p->nodes_version * 1024 + p->bs[0]) * 1024 + p->bs[1]) * 1024 + p->bs[2]) * 8 +
                      (sh[0] != 0) * 4 + (sh[1] != 0) * 2 + (sh[2] != 0);
  if (p->zmask && p->zmask_key == key) return static_cast<const unsigned long long*>(p->zmask);
  // (no allocation or rebuild inside a stream capture: unmasked passes then)
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(p->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return nullptr;
  const int tiles_x = int(p->Nt[0] / kW4);
  const size_t bytes = sizeof(unsigned long long) * size_t(tiles_x) * size_t(p->Nt[1]);
  if (!p->zmask && cudaMalloc(&p->zmask, bytes) != cudaSuccess) {
    p->zmask = nullptr;
    p->fft_prune = false;
    cudaGetLastError();
    return nullptr;
  }
  if (cudaMemsetAsync(p->zmask, 0, bytes, p->stream) != cudaSuccess) return nullptr;
  const int64_t nt = p->ntiles_total;
  if (nt > 0) {
    ::nfft::g_launches.fetch_add(1, std::memory_order_relaxed);
    zmask_kernel<<<unsigned((nt + 255) / 256), 256, 0, p->stream>>>(
        p->tile_start, int(p->ntiles[0]), int(p->ntiles[1]), int(p->ntiles[2]), int(p->bs[0]), int(p->bs[1]),
        int(p->bs[2]), p->m, int(p->Nt[0]), int(p->Nt[1]), int(p->Nt[2]), sh[0], sh[1], sh[2], tiles_x,
        static_cast<unsigned long long*>(p->zmask));
  }
  if (cudaGetLastError() != cudaSuccess) return nullptr;
  p->zmask_key = key;
  return static_cast<const unsigned long long*>(p->zmask);
}

template <typename T, int NL> int line_pass_t(nfft_plan* p, int axis, bool fwd) {
  using C = Cx<T>;
  const C* tw = static_cast<const C*>(p->fft_tw[axis]);
  C* g = static_cast<C*>(p->grid);
  int64_t outer_count;
  if constexpr (sizeof(T) == 4 && NL <= 512 && NFFT_FFT_FOURSTEP) {
    const LineGeom L = make_line_geom(p, axis, kW4, &outer_count);
    const unsigned blocks4 = unsigned(outer_count * L.tiles_x);
    if (p->fft_staged) {  // tile staged by cp.async, in-place four-step
      const size_t smem_s = size_t(NL) * kW4 * sizeof(float2);
      const unsigned long long* zm = axis == 2 ? zmask_for(p) : nullptr;
      // (the y passes take no mask: the row bitmap costs more than it saves)
      auto ks = zm && axis == 2 ? (fwd ? fft4_lines_staged_kernel<NL, true, 2> : fft4_lines_staged_kernel<NL, false, 2>)
                                : (fwd ? fft4_lines_staged_kernel<NL, true, 0> : fft4_lines_staged_kernel<NL, false, 0>);
      if (int rc = set_smem(ks, smem_s)) return rc;
      ks<<<blocks4, 256, smem_s, p->stream>>>(L, g, tw, zm);
      NFFT_LAUNCH_CHECK();
      return NFFT_OK;
    }
    const size_t smem4 = fft4_smem_bytes<NL>();
    auto kern = fwd ? fft4_lines_kernel<NL, true> : fft4_lines_kernel<NL, false>;
    if (int rc = set_smem(kern, smem4)) return rc;
    kern<<<blocks4, 256, smem4, p->stream>>>(L, g, tw);
    NFFT_LAUNCH_CHECK();
    return NFFT_OK;
  }
  constexpr int W = lines_per_cta<T>();
  const size_t smem = fft_smem_bytes<NL, T>();
  const LineGeom L = make_line_geom(p, axis, W, &outer_count);
  const unsigned blocks = unsigned(outer_count * L.tiles_x);
  if (fwd) {
    auto kern = fft_lines_kernel<T, NL, W, true>;
    if (int rc = set_smem(kern, smem)) return rc;
    kern<<<blocks, kFftThreads, smem, p->stream>>>(L, g, tw);
  } else {
    auto kern = fft_lines_kernel<T, NL, W, false>;
    if (int rc = set_smem(kern, smem)) return rc;
    kern<<<blocks, kFftThreads, smem, p->stream>>>(L, g, tw);
  }
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

// The fused forward FFT x lambda x backward FFT pass along the last axis.
template <typename T, int NL> int toeplitz_pass_t(nfft_plan* p, int axis, const void* lam, double scale) {
  using C = Cx<T>;
  const C* tw = static_cast<const C*>(p->fft_tw[axis]);
  C* g = static_cast<C*>(p->grid);
  const C* l = static_cast<const C*>(lam);
  int64_t outer_count;
  if constexpr (sizeof(T) == 4 && NL <= 512 && NFFT_FFT_FOURSTEP) {
    const LineGeom L = make_line_geom(p, axis, kW4, &outer_count);
    const unsigned blocks4 = unsigned(outer_count * L.tiles_x);
    const size_t smem4 = fft4_smem_bytes<NL>();
    auto kern = fft4_toeplitz_kernel<NL>;
    if (int rc = set_smem(kern, smem4)) return rc;
    kern<<<blocks4, 256, smem4, p->stream>>>(L, g, l, float(scale), tw);
    NFFT_LAUNCH_CHECK();
    return NFFT_OK;
  }
  constexpr int W = lines_per_cta<T>();
  const size_t smem = fft_smem_bytes<NL, T>();
  const LineGeom L = make_line_geom(p, axis, W, &outer_count);
  const unsigned blocks = unsigned(outer_count * L.tiles_x);
  auto kern = fft_toeplitz_lines_kernel<T, NL, W>;
  if (int rc = set_smem(kern, smem)) return rc;
  kern<<<blocks, kFftThreads, smem, p->stream>>>(L, g, l, T(scale), tw);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

template <typename T> int x_pass(nfft_plan* p, const void* src, void* dst, bool fwd, void* const* slot) {
  switch (p->Nt[0]) {
    case 64: return x_pass_t<T, 64>(p, src, dst, fwd, slot);
    case 128: return x_pass_t<T, 128>(p, src, dst, fwd, slot);
    case 256: return x_pass_t<T, 256>(p, src, dst, fwd, slot);
    case 512: return x_pass_t<T, 512>(p, src, dst, fwd, slot);
    case 1024: return x_pass_t<T, 1024>(p, src, dst, fwd, slot);
  }
  set_error("fused FFT: unsupported length %lld", (long long)p->Nt[0]);
  return NFFT_ERR_UNSUPPORTED;
}

template <typename T> int line_pass(nfft_plan* p, int axis, bool fwd) {
  switch (p->Nt[axis]) {
    case 64: return line_pass_t<T, 64>(p, axis, fwd);
    case 128: return line_pass_t<T, 128>(p, axis, fwd);
    case 256: return line_pass_t<T, 256>(p, axis, fwd);
    case 512: return line_pass_t<T, 512>(p, axis, fwd);
    case 1024: return line_pass_t<T, 1024>(p, axis, fwd);
  }
  set_error("fused FFT: unsupported length %lld", (long long)p->Nt[axis]);
  return NFFT_ERR_UNSUPPORTED;
}

template <typename T> int toeplitz_pass(nfft_plan* p, int axis, const void* lam, double scale) {
  switch (p->Nt[axis]) {
    case 64: return toeplitz_pass_t<T, 64>(p, axis, lam, scale);
    case 128: return toeplitz_pass_t<T, 128>(p, axis, lam, scale);
    case 256: return toeplitz_pass_t<T, 256>(p, axis, lam, scale);
    case 512: return toeplitz_pass_t<T, 512>(p, axis, lam, scale);
    case 1024: return toeplitz_pass_t<T, 1024>(p, axis, lam, scale);
  }
  set_error("fused FFT: unsupported length %lld", (long long)p->Nt[axis]);
  return NFFT_ERR_UNSUPPORTED;
}

template <typename T> int toeplitz_t(nfft_plan* p, const void* lam, double scale, void* y) {
  int rc = x_pass<T>(p, y, p->grid, true, nullptr);
  if (!rc && p->D == 3) rc = line_pass<T>(p, 1, true);
  if (!rc) rc = toeplitz_pass<T>(p, p->D - 1, lam, scale);
  if (!rc && p->D == 3) rc = line_pass<T>(p, 1, false);
  if (!rc) rc = x_pass<T>(p, p->grid, y, false, nullptr);
  return rc;
}

bool pow2_in_range(int64_t n) { return n >= 64 && n <= 1024 && (n & (n - 1)) == 0; }

}  // namespace

// Whether the plan's transforms take the fused pruned path; builds the
// twiddle tables.  NFFT_GB300_FFT=cufft keeps cuFFT (and the separate
// pad / crop kernels) for every plan created afterwards.
int fused_fft_init(nfft_plan* p) {
  p->fused_fft = false;
  if (const char* e = getenv("NFFT_GB300_FFT"))
    if (strcmp(e, "cufft") == 0) return NFFT_OK;
  if (p->D < 2) return NFFT_OK;
  for (int d = 0; d < p->D; ++d)
    if (!pow2_in_range(p->Nt[d])) return NFFT_OK;
  const size_t rs = p->real_size;
  for (int d = 0; d < p->D; ++d) {
    const int64_t n = p->Nt[d];
    std::vector<double> h(2 * n);
    for (int64_t q = 0; q < n; ++q) {
      const double a = -2.0 * 3.14159265358979323846 * double(q) / double(n);
      h[2 * q] = std::cos(a);
      h[2 * q + 1] = std::sin(a);
    }
    std::vector<unsigned char> buf(2 * rs * n);
    for (int64_t q = 0; q < 2 * n; ++q) {
      if (rs == 4) reinterpret_cast<float*>(buf.data())[q] = float(h[q]);
      else reinterpret_cast<double*>(buf.data())[q] = h[q];
    }
    if (cudaMalloc(&p->fft_tw[d], buf.size()) != cudaSuccess) {
      set_error("cudaMalloc of FFT twiddles failed");
      return NFFT_ERR_ALLOC;
    }
    NFFT_CUDA_TRY(cudaMemcpy(p->fft_tw[d], buf.data(), buf.size(), cudaMemcpyHostToDevice));
  }
  p->fused_fft = true;
  return NFFT_OK;
}

// forward: image f -> transformed grid (pad + deconvolve + FFT).  The X
// kernel is stage 1, the Y / Z line passes stage 2 (for the timing ring).
// With f_slot (device memory holding the image pointer) the kernels read the
// pointer at run time, so a captured graph replays with new arrays.
int fused_forward_x(nfft_plan* p, const void* f, void* const* f_slot) {
  return p->precision == 32 ? x_pass<float>(p, f, p->grid, true, f_slot)
                            : x_pass<double>(p, f, p->grid, true, f_slot);
}
int fused_forward_lines(nfft_plan* p) {
  int rc;
  if (p->precision == 32) {
    rc = line_pass<float>(p, 1, true);
    if (!rc && p->D == 3) rc = line_pass<float>(p, 2, true);
  } else {
    rc = line_pass<double>(p, 1, true);
    if (!rc && p->D == 3) rc = line_pass<double>(p, 2, true);
  }
  return rc;
}
// adjoint: grid -> backward FFT lines (Z', Y'), then X' with crop + deconvolution
int fused_adjoint_lines(nfft_plan* p) {
  int rc = NFFT_OK;
  if (p->precision == 32) {
    if (p->D == 3) rc = line_pass<float>(p, 2, false);
    if (!rc) rc = line_pass<float>(p, 1, false);
  } else {
    if (p->D == 3) rc = line_pass<double>(p, 2, false);
    if (!rc) rc = line_pass<double>(p, 1, false);
  }
  return rc;
}
int fused_adjoint_x(nfft_plan* p, void* f, void* const* f_slot) {
  return p->precision == 32 ? x_pass<float>(p, p->grid, f, false, f_slot)
                            : x_pass<double>(p, p->grid, f, false, f_slot);
}

// Toeplitz convolution y <- crop(IFFT(lambda . FFT(pad(y)))) on a
// transform-only plan (N = image, Ntilde = 2N, unit deconvolution factors):
// forward x pass (pad), forward y pass (D = 3), the fused last-axis pass,
// backward y pass (D = 3), backward x pass (crop).  The pruned passes place
// the image centred (wrapped) instead of in the corner of the 2N grid; a
// circular convolution commutes with that circular shift, so the cropped
// result equals the corner-placed one.
int fused_toeplitz(nfft_plan* p, const void* lam, double scale, void* y) {
  return p->precision == 32 ? toeplitz_t<float>(p, lam, scale, y) : toeplitz_t<double>(p, lam, scale, y);
}

}  // namespace nfft
