// Internal declarations of the GB300 NFFT plan: plan object, device helpers,
// window evaluation and kernel launchers.  Only the C ABI in
// include/nfft_gb300.h is public.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>
#include <atomic>
#include <string>

#include "../../include/nfft_gb300.h"

namespace nfft {

constexpr int kMaxDim = 3;
constexpr int kMinM = 2;
constexpr int kMaxM = 8;
constexpr int kMaxL = 2 * kMaxM;
constexpr int kMaxDeg = 2 * kMaxM + 1;
constexpr int kChebNodes = 30;  // ChebyshevInterpolator(κ, 1, N, 30), src/precomputation.jl:351

// Window evaluation modes on the device.
enum WinMode { WIN_POLY = 0, WIN_LINEAR = 1, WIN_EXACT = 2 };

extern std::atomic<int64_t> g_launches;
void set_error(const char* fmt, ...);

#define NFFT_CUDA_TRY(expr)                                                              \
  do {                                                                                   \
    cudaError_t err__ = (expr);                                                          \
    if (err__ != cudaSuccess) {                                                          \
      ::nfft::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #expr,                     \
                        cudaGetErrorString(err__));                                      \
      return NFFT_ERR_CUDA;                                                              \
    }                                                                                    \
  } while (0)

#define NFFT_LAUNCH_CHECK()                                                              \
  do {                                                                                   \
    ::nfft::g_launches.fetch_add(1, std::memory_order_relaxed);                          \
    cudaError_t err__ = cudaGetLastError();                                              \
    if (err__ != cudaSuccess) {                                                          \
      ::nfft::set_error("%s:%d: kernel launch: %s", __FILE__, __LINE__,                 \
                        cudaGetErrorString(err__));                                      \
      return NFFT_ERR_CUDA;                                                              \
    }                                                                                    \
  } while (0)

// Per-launch geometry shared by the convolution kernels (passed by value).
template <typename T> struct Geom {
  int D;
  int m;
  int Nt[kMaxDim];        // oversampled grid, singleton dims = 1
  int bs[kMaxDim];        // tile size, singleton dims = 1
  int ntiles[kMaxDim];
  int64_t plane;          // Nt[0]*Nt[1]
  int64_t M;
  int mode;               // WinMode
  int window;             // NFFT_WINDOW_*
  T sigma;
  T lut_scale;            // LUTSize / m (LINEAR)
  const T* coeffs;        // (2m+1) x 2m, column l contiguous (POLY)
  const T* lut;           // LUTSize+2 (LINEAR)
  bool small_grid;        // some Ntilde < 2m: taps may wrap more than once
  int sh[kMaxDim];        // grid position of index n is (n + sh) mod Ntilde (the centred internal grid; else 0)
};

// Sorted node data produced by nfft_set_nodes.
//   node4[i] = {trunc_x, trunc_y, trunc_z, input index j} of the node at sorted
//              position i (trunc = trunc(k_shift * Ntilde), 0 in singleton dims);
//   frac4[4i + d] = fractional offset e_d in [0,1) (a hair outside for FP32);
//   wtab[i*D*2m + d*2m + l] = window value of tap l in dimension d (the window
//              tensor; stored unless the precompute mode is POLYNOMIAL).
template <typename T> struct Nodes {
  const int4* node4;
  const T* frac4;
  const T* wtab;
  int64_t M;
};

}  // namespace nfft

struct nfft_plan {
  int precision = 32;
  int D = 0;
  int64_t N[3] = {1, 1, 1};
  int64_t Nt[3] = {1, 1, 1};
  int64_t M = 0;
  nfft_params prm{};
  int m = 4;
  double sigma = 2.0;
  int64_t lut_size = 0;
  int64_t bs[3] = {1, 1, 1};
  int64_t ntiles[3] = {1, 1, 1};
  int64_t ntiles_total = 1;
  cudaStream_t stream = nullptr;
  // FFT of the oversampled grid.  D = 1: one plan.  D >= 2 (pruned): the
  // image occupies a head and a tail range along the last dimension, so the
  // transform runs as batched (D-1)-dimensional FFTs over those slices only
  // plus one strided 1-D pass along the last dimension (forward: slices
  // first; backward: the 1-D pass first, then only the slices the crop reads).
  cufftHandle fft = 0;        // D = 1: the transform; D >= 2: slices of the head range
  cufftHandle fft_tail = 0;   // slices of the tail range (when its length differs)
  cufftHandle fft_line = 0;   // strided 1-D pass along the last dimension
  bool fft_ok = false, fft_tail_ok = false, fft_line_ok = false;
  int64_t slice_head = 0, slice_tail = 0, slice_size = 0;
  void* fft_work = nullptr;
  // fused pruned FFT (fft.cu): used instead of pad + cuFFT / cuFFT + crop on
  // the transform path when every Ntilde_d is a power of two in [64, 1024]
  bool fused_fft = false;
  void* fft_tw[3] = {};       // per dimension: exp(-2 pi i q / Ntilde_d), q < Ntilde_d (T complex)
  size_t real_size = 4;

  void* grid = nullptr;       // tmpVec, |Ntilde| complex
  void* inv = nullptr;        // deconvolution factors, N0+N1+N2 reals
  // Centred internal grid: the forward / adjoint transforms keep the
  // oversampled grid shifted by sh = Ntilde/2 in every dimension where that is
  // a whole number of tiles (an fftshift), so the dense centre of k-space (grid
  // index 0) lies inside the grid instead of at its corner.  The shift is the
  // factor (-1)^k on the grid frequencies, folded into inv_c = inv times
  // (-1)^(n - N/2); convolve!/deconvolve! and the batched and directional
  // paths keep the reference layout (cur_center = 0).
  bool center = true;
  int64_t sh[3] = {0, 0, 0};
  void* inv_c = nullptr;
  int cur_center = 0;
  void* coeffs = nullptr;     // poly coefficients (T)
  void* lut = nullptr;        // LINEAR lut (T)
  double coeffs_host[nfft::kMaxDeg * nfft::kMaxL] = {};

  bool has_nodes = false;
  int64_t nodes_version = 0;  // bumped by every successful nfft_set_nodes
  void* k = nullptr;          // D x M nodes (T), user order
  int4* node4 = nullptr;      // M, sorted: trunc per dim + input index
  void* frac4 = nullptr;      // 4M (T), sorted: fractional offsets
  void* wtab = nullptr;       // M * D * 2m (T), sorted window tensor (not for POLYNOMIAL)
  int32_t* tile_start = nullptr;   // ntiles_total + 1: CSR of nodes per home tile
  void* cbuf = nullptr;       // M complex scratch for real-valued convolve calls (lazy)
  void* fsorted = nullptr;    // M complex: fHat in bin-sorted order (spreading input)
  // spreading tasks: (home tile, first node, end node, 0), hot tiles split
  int64_t n_tasks = 0;
  int4* tasks = nullptr;
  int spread_pitch = 0;            // shared-memory row pitch of the padded spreading tile
  int spread_layout = 1;           // D = 3 spreading kernel: 1 = 8 warps owning slices, 2 = 16 warps owning
                                   // (slice group, row parity)
  bool spread_tile3 = true;        // 3-D FP32 m = 4: shape-specialised spreading kernel (spread_tile3.cuh)
  bool spread_tma = true;          // its bulk tensor reduction flush for tiles that do not wrap
  bool gather_tma = true;          // 3-D FP32 m = 4 gather from tiles loaded by bulk tensor copies
  // tensor maps of the grids the tiled kernels moved tiles of (the plan's two
  // grids), with their grid and tile shape; replaced least recently made first
  CUtensorMap tmap[2] = {};
  void* tmap_grid[2] = {nullptr, nullptr};
  int64_t tmap_key[2] = {0, 0};
  int tmap_next = 0;
  // a second grid for the adjoint, zeroed on a side stream beside the next
  // forward transform's gather so that the next adjoint needs no memset
  bool prezero = true;
  bool grid2_dirty = false;        // grid2 holds an adjoint's data
  void* grid2 = nullptr;
  cudaStream_t zero_stream = nullptr;
  cudaEvent_t ev_grid2_used = nullptr, ev_grid2_zeroed = nullptr;
  bool skip_memset = false;
  bool fft_prune = true;           // z-line mask of the forward / inverse z passes (3-D FP32 staged path)
  void* zmask = nullptr;           // tiles_x x Nt1 64-bit masks
  int64_t zmask_key = -1;
  bool spread_zero_copy = true;    // table spreader: clear the tile by a bulk copy of zero_tile
  void* zero_tile = nullptr;       // 128 KB of zeros
  bool fft_staged = true;          // FP32 line FFTs: tile staged by cp.async, in-place four-step
  bool spread_rec = true;          // 3-D FP32 table spreader: one-step staging with per-warp records
  int gather_pf = 4;               // TMA gather: L2 prefetch of the tile gather_pf x (SM count) tasks ahead (0: off)        // set while the spreading target is known to be zero
  int gather_pitch = 0;            // shared-memory row pitch of the staged gather tile
  bool gather_tiled = false;       // gather from shared-memory tiles (else straight from L1/L2)
  // device buffers of nfft_set_nodes, kept across calls (nodes! every step of
  // a node optimisation) and grown on demand; the node tables above point
  // into the first ones
  enum { NB_K, NB_NODE4, NB_FRAC4, NB_WTAB, NB_TSTART, NB_TASKS, NB_FSORTED, NB_TI, NB_TE, NB_KEY, NB_VAL,
         NB_KEY2, NB_VAL2, NB_TCOUNT, NB_SCR, NB_TCNT, NB_TOFF, NB_COUNT };
  void* nbuf[NB_COUNT] = {};
  size_t nbuf_cap[NB_COUNT] = {};
  int* dflag = nullptr;            // device status words: [0] node check, [1] an async copy wait that timed out
  size_t scratch_bytes = 0;

  // TimingStats: every forward/adjoint records 4 events into a ring slot; the
  // slots are harvested (summed per stage) lazily, so timing adds no host
  // synchronisation to the calls themselves.
  bool timing_on = false;
  static constexpr int kRing = 64;
  cudaEvent_t ev[kRing][4] = {};
  int ring_dir[kRing] = {};        // -1 empty, 0 forward, 1 adjoint
  int64_t ring_next = 0;
  double timing[7] = {};           // last call per stage (seconds)
  double timing_sum[7] = {};       // totals since the last reset
  int64_t timing_calls[2] = {0, 0};
};

namespace nfft {

// ------------------------------------------------------------------ launchers
// precompute.cu
int launch_check_nodes(const nfft_plan* p, const void* k, int* flag);
// the same check on n values of the given precision, without a plan
int launch_check_node_values(int precision, const void* k, int64_t n, int* flag, cudaStream_t s);
int launch_reduce_nodes(const nfft_plan* p, const void* k, int32_t* ti_u, void* te_u, uint32_t* key,
                        int32_t* val, int32_t* tile_count);
int launch_build_node_tables(const nfft_plan* p, const int32_t* perm, const int32_t* ti_u, const void* te_u);
int launch_build_weight_table(const nfft_plan* p);
int launch_deconv_factors(nfft_plan* p);
int launch_build_tasks(nfft_plan* p, int chunk);
// autotune.cu
int apply_block_size(nfft_plan* p, const int64_t* bs, const void* k, int ny);
// spread.cu: bank-conflict-free row pitch of a padded spreading tile
int spread_pitch_for(int D, int m, int P0, int elem_bytes, int ny);
// sort.cu
int radix_sort_pairs(uint32_t* keys, int32_t* vals, uint32_t* keys_tmp, int32_t* vals_tmp, int64_t n,
                     int key_bits, void* scratch, size_t scratch_bytes, cudaStream_t s,
                     uint32_t** keys_out, int32_t** vals_out);
size_t radix_sort_scratch_bytes(int64_t n);
int exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, void* scratch, size_t scratch_bytes,
                       cudaStream_t s);
size_t scan_scratch_bytes(int64_t n);
// deconv.cu
int launch_pad_apodize(const nfft_plan* p, const void* f, void* g);
int launch_crop_apodize(const nfft_plan* p, const void* g, void* f);
int launch_real_to_complex(const nfft_plan* p, const void* in, void* out, int64_t n);
int launch_real_part(const nfft_plan* p, const void* in, void* out, int64_t n);
// interp.cu
int launch_interp(const nfft_plan* p, const void* g, int g_real, void* fhat, int fhat_real);
// ncols columns in one launch: grids g + c gcol, node values fhat + c fcol (complex elements)
int launch_interp_cols(const nfft_plan* p, const void* g, void* fhat, int ncols, int64_t gcol, int64_t fcol);
// spread.cu
int launch_spread(nfft_plan* p, const void* fhat, int fhat_real, void* g, int g_real);
// ncols columns in one launch: values fhat + c fcol, contiguous grids g + c gcol (gcol = |Ntilde|),
// bin-sorted values in `sorted` (M x ncols complex)
int launch_spread_cols(nfft_plan* p, const void* fhat, void* g, int ncols, int64_t fcol, int64_t gcol, void* sorted);
// plan.cu: the grid FFT of a plan (pruned for D >= 2)
int exec_fft_plan(nfft_plan* p, int dir);
// fft.cu: fused pruned FFT with the deconvolution
int fused_fft_init(nfft_plan* p);
int fused_forward_x(nfft_plan* p, const void* f, void* const* f_slot = nullptr);
int fused_forward_lines(nfft_plan* p);
int fused_adjoint_lines(nfft_plan* p);
int fused_adjoint_x(nfft_plan* p, void* f, void* const* f_slot = nullptr);
// y <- crop(IFFT(scale * lambda . FFT(pad(y)))) on a transform-only plan (N image, Ntilde = 2N)
int fused_toeplitz(nfft_plan* p, const void* lam, double scale, void* y);
// gradk.cu
int launch_grad_nodes(const nfft_plan* p, const void* g, const void* w, void* dk);
// plain.cu (per-node kernels of the plain path, blocking = 0)
int launch_plain_interp(const nfft_plan* p, const void* g, int g_real, void* fhat, int fhat_real);
int launch_plain_spread(const nfft_plan* p, const void* fhat, int fhat_real, void* g, int g_real);

template <typename T> Geom<T> make_geom(const nfft_plan* p);
// plan.cu: node buffer `which` of at least `bytes` (grown, contents not kept)
void* node_buffer(nfft_plan* p, int which, size_t bytes);
// plan.cu: recompute sh and inv_c after the tiles or the factors changed
int update_center(nfft_plan* p);
// the centred grid during one forward / adjoint / gradient call
struct CenterScope {
  nfft_plan* p;
  explicit CenterScope(nfft_plan* q) : p(q) { p->cur_center = (p->sh[0] | p->sh[1] | p->sh[2]) != 0; }
  ~CenterScope() { p->cur_center = 0; }
};
template <typename T> Nodes<T> make_nodes(const nfft_plan* p);

// ------------------------------------------------------------ device helpers

__host__ __device__ inline int wrap_once(int g, int n) { return g < 0 ? g + n : (g >= n ? g - n : g); }
__host__ __device__ inline int wrap_any(int g, int n) {
  int r = g % n;
  return r < 0 ? r + n : r;
}

template <typename T> struct Cplx;
template <> struct Cplx<float> { using type = float2; };
template <> struct Cplx<double> { using type = double2; };

template <typename T> __device__ inline T dev_sqrt(T x);
template <> __device__ inline float dev_sqrt<float>(float x) { return sqrtf(x); }
template <> __device__ inline double dev_sqrt<double>(double x) { return sqrt(x); }

// Modified Bessel I0 from its power series sum_k (x^2/4)^k / (k!)^2.
template <typename T> __host__ __device__ inline T bessel_i0_series(T x) {
  T q = T(0.25) * x * x, term = T(1), sum = T(1);
  for (int k = 1; k < 200; ++k) {
    term *= q / (T(k) * T(k));
    sum += term;
    if (term <= sum * T(1e-17)) break;
  }
  return sum;
}

// Bessel J0 from its power series sum_k (-x^2/4)^k / (k!)^2 (moderate x only).
template <typename T> __host__ __device__ inline T bessel_j0_series(T x) {
  T q = -T(0.25) * x * x, term = T(1), sum = T(1);
  for (int k = 1; k < 200; ++k) {
    term *= q / (T(k) * T(k));
    sum += term;
    if (term <= sum * T(1e-18) && term >= -sum * T(1e-18) && k > 4) break;
  }
  return sum;
}

// phi-hat of the windows at a real frequency n for a grid of Nt points
// (src/windowFunctions.jl); host and device, FP64.
__host__ __device__ inline double window_hat(int window, double n, double Nt, int m, double sigma) {
  const double PI = 3.14159265358979323846;
  switch (window) {
    case NFFT_WINDOW_KAISER_BESSEL: {  // src/windowFunctions.jl:36-39
      double b = PI * (2.0 - 1.0 / sigma);
      double a = 2.0 * PI * n / Nt;
      return bessel_i0_series<double>(m * sqrt(b * b - a * a));
    }
    case NFFT_WINDOW_GAUSS: {  // :70-73
      double b = m / PI;
      double a = PI * n / Nt;
      return exp(-(a * a) * b);
    }
    case NFFT_WINDOW_SPLINE: {  // :98-100, Julia sinc(x) = sin(pi x)/(pi x)
      double x = n / Nt;
      double s = (x == 0.0) ? 1.0 : sin(PI * x) / (PI * x);
      double r = 1.0;
      for (int i = 0; i < 2 * m; ++i) r *= s;
      return r;
    }
    case NFFT_WINDOW_KAISER_BESSEL_REV: {  // :51-57, real(sinc(sqrt(complex(a2))/pi))
      double b = PI * (2.0 - 1.0 / sigma);
      double u = 2.0 * PI * m * n / Nt;
      double a2 = u * u - (m * b) * (m * b);
      if (a2 > 0.0) {
        double a = sqrt(a2);
        return sin(a) / a;
      } else if (a2 < 0.0) {
        double a = sqrt(-a2);
        return sinh(a) / a;
      }
      return 1.0;
    }
    case NFFT_WINDOW_COSH_TYPE: {  // :118-134
      double beta = PI * m * (2.0 - 1.0 / sigma);
      double gamma = beta / (2.0 * PI);
      double zeta = PI / (cosh(beta) - 1.0) * m;
      double arg = m * n / Nt;
      double aa = fabs(arg);
      double j0 = bessel_j0_series<double>(2.0 * PI * arg);
      if (aa < gamma) {
        double q = 2.0 * PI * arg;
        return zeta * (bessel_i0_series<double>(sqrt(beta * beta - q * q)) - j0);
      } else if (aa > gamma) {
        double q = 2.0 * PI * arg;
        return zeta * (bessel_j0_series<double>(sqrt(q * q - beta * beta)) - j0);
      }
      return zeta * (1.0 - bessel_j0_series<double>(beta));
    }
  }
  return 1.0;
}

// Cardinal B-spline of order n at x (src/windowFunctions.jl:75-87),
// evaluated bottom-up over the shifts it needs.
template <typename T> __host__ __device__ inline T cbspline_eval(int n, T x) {
  T b[2 * kMaxM + 2];
  for (int j = 0; j < n; ++j) b[j] = (x - T(j) >= T(0) && x - T(j) < T(1)) ? T(1) : T(0);
  for (int o = 2; o <= n; ++o) {
    for (int j = 0; j + o <= n; ++j) {
      T xs = x - T(j);
      b[j] = xs / T(o - 1) * b[j] + (T(o) - xs) / T(o - 1) * b[j + 1];
    }
  }
  return b[0];
}

// Window phi at distance x (grid units), i.e. phi(x/Ntilde) of
// src/windowFunctions.jl with the Ntilde factors cancelled.
template <typename T> __host__ __device__ inline T window_exact(int window, T x, int m, T sigma) {
  const T PI = T(3.14159265358979323846);
  T ax = x < T(0) ? -x : x;
  T mm = T(m);
  switch (window) {
    case NFFT_WINDOW_KAISER_BESSEL: {
      T b = PI * (T(2) - T(1) / sigma);
      if (ax < mm) {
        T arg = sqrt(mm * mm - x * x);
        return sinh(b * arg) / (arg * PI);
      } else if (ax > mm) {
        return T(0);
      }
      return b / PI;
    }
    case NFFT_WINDOW_GAUSS: {
      T b = mm / PI;
      if (ax < mm) return T(1) / sqrt(PI * b) * exp(-(x * x) / b);
      return T(0);
    }
    case NFFT_WINDOW_SPLINE:
      if (ax < mm) return cbspline_eval<T>(2 * m, x + mm);
      return T(0);
    case NFFT_WINDOW_KAISER_BESSEL_REV: {
      T b = PI * (T(2) - T(1) / sigma);
      if (ax < mm) {
        T r = x / mm;
        return T(0.5) / mm * bessel_i0_series<T>(mm * b * sqrt(T(1) - r * r));
      }
      return T(0);
    }
    case NFFT_WINDOW_COSH_TYPE: {
      T beta = PI * mm * (T(2) - T(1) / sigma);
      if (ax < mm) {
        T a = x / mm;
        T alpha = sqrt(T(1) - a * a);
        return T(1) / (cosh(beta) - T(1)) * (cosh(beta * alpha) - T(1)) / alpha;
      }
      return T(0);
    }
  }
  return T(0);
}

__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// Reduce node j, dimension d.  The grid index follows NFFT.jl's blocked path
// exactly in the plan's real type T: shiftNodes! (src/utils.jl:32-44), then
// unsafe_trunc(Int, k*Ntilde) (src/precomputation.jl:496,536), so that bin
// ids and grid indices are bit-identical.  The fractional offset is formed in
// FP64: for T = Float64 it is the reference's own kscale - trunc; for
// T = Float32 it is the exact k*Ntilde (+Ntilde for shifted nodes) minus the
// index, which avoids the Float32 rounding of k + 1.
template <typename T>
__device__ __forceinline__ void reduce_coord(T x, int Nt, int32_t& t_out, T& e_out) {
  T xs = x;
  if (xs < T(0)) xs = add_rn(xs, T(1));
  if (xs == T(1)) xs = xs - (sizeof(T) == 4 ? T(1.1920928955078125e-7) : T(2.220446049250313080847e-16));
  T ks = mul_rn(xs, T(Nt));
  int t = int(ks);
  if (t >= Nt) t = Nt - 1;
  if (t < 0) t = 0;
  double e;
  if (sizeof(T) == 4) {
    e = double(x) * double(Nt) + (x < T(0) ? double(Nt) : 0.0) - double(t);
  } else {
    e = double(ks) - double(t);
  }
  t_out = t;
  e_out = T(e);
}

// Window value of tap l (0-based) for a node with fractional offset e:
// the tap sits at trunc - m + 1 + l, the node at trunc + e.
template <typename T>
__device__ __forceinline__ T tap_weight(const Geom<T>& G, const T* __restrict__ coeffs_smem, T e, int l) {
  if (G.mode == WIN_POLY) {
    // evalpoly(e - 1/2, coeffs[:, l]), src/precomputation.jl:205-222
    const int deg = 2 * G.m + 1;
    const T* c = coeffs_smem + l * deg;
    T t = e - T(0.5);
    T r = c[deg - 1];
    for (int i = deg - 2; i >= 0; --i) r = fma(r, t, c[i]);
    return r;
  } else if (G.mode == WIN_LINEAR) {
    // linear LUT interpolation of phi(|x|), src/precomputation.jl:168-190
    T x = e + T(G.m - 1 - l);
    T u = (x < T(0) ? -x : x) * G.lut_scale;
    // the LUT holds LUTSize+2 samples; an offset a hair outside [0,1)
    // (FP32 nodes) must not index past them
    const T umax = T(G.m) * G.lut_scale;
    if (u > umax) u = umax;
    T fi = floor(u);
    int i = int(fi);
    T a = u - fi;
    T v0 = __ldg(G.lut + i), v1 = __ldg(G.lut + i + 1);
    return v0 + a * (v1 - v0);
  }
  return window_exact<T>(G.window, e + T(G.m - 1 - l), G.m, G.sigma);
}

}  // namespace nfft
