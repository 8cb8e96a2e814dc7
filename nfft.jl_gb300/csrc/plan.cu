// C ABI of the GB300 NFFT plan (include/nfft_gb300.h): plan construction,
// node binning, forward/adjoint orchestration, cuFFT, timing, errors.
#include "nfft_internal.cuh"

#include <utility>

#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace nfft {

std::atomic<int64_t> g_launches{0};
static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

template <typename T> Geom<T> make_geom(const nfft_plan* p) {
  Geom<T> G{};
  G.D = p->D;
  G.m = p->m;
  bool small = false;
  for (int d = 0; d < kMaxDim; ++d) {
    G.Nt[d] = int(p->Nt[d]);
    G.bs[d] = int(p->bs[d]);
    G.ntiles[d] = int(p->ntiles[d]);
    if (d < p->D && p->Nt[d] < 2 * p->m) small = true;
  }
  G.plane = p->Nt[0] * p->Nt[1];
  G.M = p->M;
  G.mode = (p->prm.precompute == NFFT_PRECOMPUTE_FULL)     ? WIN_EXACT
           : (p->prm.precompute == NFFT_PRECOMPUTE_LINEAR) ? WIN_LINEAR
                                                           : WIN_POLY;
  G.window = p->prm.window;
  G.sigma = T(p->sigma);
  G.lut_scale = T(p->lut_size / p->m);
  G.coeffs = static_cast<const T*>(p->coeffs);
  G.lut = static_cast<const T*>(p->lut);
  G.small_grid = small;
  for (int d = 0; d < kMaxDim; ++d) G.sh[d] = p->cur_center ? int(p->sh[d]) : 0;
  return G;
}
template Geom<float> make_geom<float>(const nfft_plan*);
template Geom<double> make_geom<double>(const nfft_plan*);

// inv_c[i] = inv[i] * (-1)^(n - N_d/2) for the factors of dimensions with a
// grid shift (n = image index within dimension d's segment), inv[i] elsewhere.
template <typename T>
__global__ void centre_factors_kernel(const T* __restrict__ inv, T* __restrict__ inv_c, int64_t n, int N0, int N1,
                                      int N2, int s0, int s1, int s2) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int d = -1, k = 0, Nd = 1;
  if (i < N0) {
    d = 0; k = int(i); Nd = N0;
  } else if (i < N0 + N1) {
    d = 1; k = int(i - N0); Nd = N1;
  } else if (i < N0 + N1 + N2) {
    d = 2; k = int(i - N0 - N1); Nd = N2;
  }
  const int s = d == 0 ? s0 : d == 1 ? s1 : d == 2 ? s2 : 0;
  const T v = inv[i];
  inv_c[i] = (s && ((k - Nd / 2) & 1)) ? -v : v;
}

void* node_buffer(nfft_plan* p, int which, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (p->nbuf_cap[which] < bytes) {
    cudaFree(p->nbuf[which]);
    p->nbuf[which] = nullptr;
    p->nbuf_cap[which] = 0;
    // 1/8 headroom: node sets that grow a little do not reallocate every time
    const size_t want = bytes + bytes / 8;
    if (cudaMalloc(&p->nbuf[which], want) != cudaSuccess) {
      p->nbuf[which] = nullptr;
      set_error("cudaMalloc of %zu bytes of node buffers failed", want);
      return nullptr;
    }
    p->nbuf_cap[which] = want;
  }
  return p->nbuf[which];
}

int update_center(nfft_plan* p) {
  for (int d = 0; d < 3; ++d) p->sh[d] = 0;
  if (!p->center || !p->prm.blocking) return NFFT_OK;
  bool any = false;
  for (int d = 0; d < p->D; ++d) {
    const int64_t h = p->Nt[d] / 2;
    if (p->Nt[d] % 2 == 0 && h > 0 && h % p->bs[d] == 0) {
      p->sh[d] = h;
      any = true;
    }
  }
  if (!any) return NFFT_OK;
  const int N0 = int(p->N[0]), N1 = p->D > 1 ? int(p->N[1]) : 0, N2 = p->D > 2 ? int(p->N[2]) : 0;
  const int64_t ninv = int64_t(N0) + N1 + N2 + 1;
  if (!p->inv_c && cudaMalloc(&p->inv_c, p->real_size * size_t(ninv)) != cudaSuccess) {
    p->inv_c = nullptr;
    for (int d = 0; d < 3; ++d) p->sh[d] = 0;
    set_error("cudaMalloc of the centred deconvolution factors failed");
    return NFFT_ERR_ALLOC;
  }
  const unsigned nb = unsigned((ninv + 255) / 256);
  if (p->precision == 32)
    centre_factors_kernel<float><<<nb, 256, 0, p->stream>>>(static_cast<const float*>(p->inv),
                                                             static_cast<float*>(p->inv_c), ninv, N0, N1, N2,
                                                             p->sh[0] != 0, p->sh[1] != 0, p->sh[2] != 0);
  else
    centre_factors_kernel<double><<<nb, 256, 0, p->stream>>>(static_cast<const double*>(p->inv),
                                                              static_cast<double*>(p->inv_c), ninv, N0, N1, N2,
                                                              p->sh[0] != 0, p->sh[1] != 0, p->sh[2] != 0);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

template <typename T> Nodes<T> make_nodes(const nfft_plan* p) {
  Nodes<T> n{};
  n.node4 = p->node4;
  n.frac4 = static_cast<const T*>(p->frac4);
  n.wtab = static_cast<const T*>(p->wtab);
  n.M = p->M;
  return n;
}

template Nodes<float> make_nodes<float>(const nfft_plan*);
template Nodes<double> make_nodes<double>(const nfft_plan*);

namespace {

// --------------------------------------------------------------- host math

// Householder least squares min ||A x - b|| for a tall rows x cols matrix
// (column-major), FP64.  Used for the window polynomial fit.
bool lstsq(std::vector<double> A, std::vector<double> b, int rows, int cols, double* x) {
  for (int c = 0; c < cols; ++c) {
    double norm = 0;
    for (int r = c; r < rows; ++r) norm += A[r + rows * c] * A[r + rows * c];
    norm = std::sqrt(norm);
    if (norm == 0) return false;
    double alpha = A[c + rows * c] > 0 ? -norm : norm;
    std::vector<double> v(rows, 0.0);
    for (int r = c; r < rows; ++r) v[r] = A[r + rows * c];
    v[c] -= alpha;
    double vn = 0;
    for (int r = c; r < rows; ++r) vn += v[r] * v[r];
    if (vn == 0) continue;
    for (int cc = c; cc < cols; ++cc) {
      double s = 0;
      for (int r = c; r < rows; ++r) s += v[r] * A[r + rows * cc];
      s = 2 * s / vn;
      for (int r = c; r < rows; ++r) A[r + rows * cc] -= s * v[r];
    }
    double s = 0;
    for (int r = c; r < rows; ++r) s += v[r] * b[r];
    s = 2 * s / vn;
    for (int r = c; r < rows; ++r) b[r] -= s * v[r];
  }
  for (int c = cols - 1; c >= 0; --c) {
    double s = b[c];
    for (int cc = c + 1; cc < cols; ++cc) s -= A[c + rows * cc] * x[cc];
    x[c] = s / A[c + rows * c];
  }
  return true;
}

// precomputePolyInterp, src/precomputation.jl:302-320: for tap column l a
// least-squares fit (V' \ samples) of a degree-2m polynomial in t to
// phi(m - (l - 0.5) + t), sampled at 2(2m+1) equispaced t in [-0.5, 0.5].
bool poly_fit(int window, int m, double sigma, double* out /* deg x 2m, column l contiguous */) {
  const int deg = 2 * m + 1, K = 2 * m, ns = 2 * deg;
  std::vector<double> A(size_t(ns) * deg), t(ns);
  for (int i = 0; i < ns; ++i) t[i] = -0.5 + double(i) / double(ns - 1);
  for (int r = 0; r < deg; ++r)
    for (int i = 0; i < ns; ++i) A[i + ns * r] = std::pow(t[i], double(r));
  for (int l = 1; l <= K; ++l) {
    std::vector<double> b(ns);
    for (int i = 0; i < ns; ++i) b[i] = window_exact<double>(window, (m - (l - 0.5)) + t[i], m, sigma);
    if (!lstsq(A, b, ns, deg, out + size_t(l - 1) * deg)) return false;
  }
  return true;
}

// LUT of src/precomputation.jl:291-300: phi(l * m / K), l = 0..K+1.
template <typename T> __global__ void lut_kernel(int window, int m, double sigma, int64_t K, T* out) {
  int64_t l = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (l >= K + 2) return;
  out[l] = T(window_exact<double>(window, double(l) * double(m) / double(K), m, sigma));
}

int64_t lut_size_for(int m) {
  static const int m2K[] = {1, 3, 7, 9, 14, 17, 20, 23, 24};
  int K = m2K[(m + 1 < 9 ? m + 1 : 9) - 1];
  return (int64_t(1) << K) * m;
}

void default_block(nfft_plan* p) {
  // Default tiles (the autotuner refines them): 16x8x8 (3-D, the fastest
  // shape measured on a 256^3 radial set), 32^2 (2-D, two warps per CTA),
  // 1024 (1-D); the last dimension halved in FP64.  The
  // reference's blockSize keyword overrides them.
  int64_t def[3][3] = {{1024, 1, 1}, {32, 32, 1}, {16, 8, 8}};
  // compensated 1-D rows hold 16- or 32-byte accumulators and one warp each
  if (p->prm.compensated) def[0][0] = 512;
  bool user = false;
  for (int d = 0; d < 3; ++d) {
    int64_t b = def[p->D - 1][d];
    if (p->precision == 64 && d == p->D - 1) b = b > 1 ? b / 2 : 1;
    if (p->prm.block_size[d] > 0 && d < p->D) {
      b = p->prm.block_size[d];
      user = true;
    }
    if (d >= p->D) b = 1;
    if (b > p->Nt[d]) b = p->Nt[d];
    p->bs[d] = b;
  }
  // small grids: halve the largest tile side (down to 8) until there are at
  // least 4 tiles per SM of the plan's GPU, so the spreading tasks fill it
  if (!user) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess || sms < 1)
      sms = 1;
    for (;;) {
      int64_t nt = 1;
      int dmax = 0;
      for (int d = 0; d < p->D; ++d) {
        nt *= (p->Nt[d] + p->bs[d] - 1) / p->bs[d];
        if (p->bs[d] > p->bs[dmax]) dmax = d;
      }
      if (nt >= 4 * int64_t(sms) || p->bs[dmax] <= 8) break;
      p->bs[dmax] /= 2;
    }
  }
}

// The plan forgets its nodes; the node buffers stay allocated for the next
// nfft_set_nodes.
void free_nodes(nfft_plan* p) {
  p->k = p->frac4 = p->wtab = nullptr;
  p->fsorted = nullptr;
  p->node4 = nullptr;
  p->tile_start = nullptr;
  p->tasks = nullptr;
  p->n_tasks = 0;
  p->has_nodes = false;
}

void release_node_buffers(nfft_plan* p) {
  free_nodes(p);
  for (int i = 0; i < nfft_plan::NB_COUNT; ++i) {
    cudaFree(p->nbuf[i]);
    p->nbuf[i] = nullptr;
    p->nbuf_cap[i] = 0;
  }
}

int bits_for(int64_t n) {
  int b = 0;
  while ((int64_t(1) << b) < n) ++b;
  return b;
}

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() { cudaFree(p); }
  bool alloc(size_t n) { return cudaMalloc(&p, n ? n : 16) == cudaSuccess; }
};

#define NFFT_ALLOC(buf, bytes)                                                         \
  do {                                                                                 \
    if (!(buf).alloc(bytes)) {                                                         \
      set_error("cudaMalloc of %zu bytes failed", size_t(bytes));                      \
      return NFFT_ERR_ALLOC;                                                           \
    }                                                                                  \
  } while (0)

int cufft_check(cufftResult r, const char* what) {
  if (r != CUFFT_SUCCESS) {
    set_error("cuFFT %s failed (%d)", what, int(r));
    return NFFT_ERR_CUFFT;
  }
  return NFFT_OK;
}

int exec_one(nfft_plan* p, cufftHandle h, int64_t offset, int dir) {
  if (p->precision == 32) {
    auto* g = static_cast<cufftComplex*>(p->grid) + offset;
    return cufft_check(cufftExecC2C(h, g, g, dir), "exec");
  }
  auto* g = static_cast<cufftDoubleComplex*>(p->grid) + offset;
  return cufft_check(cufftExecZ2Z(h, g, g, dir), "exec");
}

// FFT of the plan's grid, unnormalised, forward sign -1 / backward +1
// (plan_fft! / plan_bfft!, src/implementation.jl:87-88).
int exec_fft(nfft_plan* p, int dir) {
  if (!p->fft_line_ok) return exec_one(p, p->fft, 0, dir);
  const int64_t ntl = p->Nt[p->D - 1];
  auto slices = [&]() -> int {
    int rc = NFFT_OK;
    if (p->slice_head > 0) rc = exec_one(p, p->fft, 0, dir);
    if (!rc && p->slice_tail > 0)
      rc = exec_one(p, p->fft_tail_ok ? p->fft_tail : p->fft, (ntl - p->slice_tail) * p->slice_size, dir);
    return rc;
  };
  int rc;
  if (dir == CUFFT_FORWARD) {
    rc = slices();
    if (!rc) rc = exec_one(p, p->fft_line, 0, dir);
  } else {
    rc = exec_one(p, p->fft_line, 0, dir);
    if (!rc) rc = slices();
  }
  return rc;
}

// cuFFT plans of the grid transform with one shared work area.
int make_fft_plans(nfft_plan* p) {
  const cufftType type = p->precision == 32 ? CUFFT_C2C : CUFFT_Z2Z;
  const int D = p->D;
  size_t ws[3] = {0, 0, 0};
  auto mk = [&](cufftHandle* h, bool* ok, int rank, int* n, int* embed, int stride, int dist, int batch,
                size_t* w) -> int {
    int rc = cufft_check(cufftCreate(h), "create");
    if (rc) return rc;
    *ok = true;
    rc = cufft_check(cufftSetAutoAllocation(*h, 0), "auto allocation");
    if (rc) return rc;
    return cufft_check(cufftMakePlanMany(*h, rank, n, embed, stride, dist, embed, stride, dist, type, batch, w),
                       "plan");
  };
  int rc;
  if (D == 1) {
    int n[1] = {int(p->Nt[0])};
    rc = mk(&p->fft, &p->fft_ok, 1, n, nullptr, 1, 0, 1, &ws[0]);
    if (rc) return rc;
  } else {
    const int64_t nl = p->N[D - 1];
    p->slice_head = nl - nl / 2;  // image rows n >= N/2 land at 0 .. ceil(N/2)-1
    p->slice_tail = nl / 2;       // image rows n < N/2 land at Ntilde - N/2 ..
    p->slice_size = D == 3 ? p->Nt[0] * p->Nt[1] : p->Nt[0];
    int n_in[2];
    const int rank_in = D - 1;
    if (D == 3) {
      n_in[0] = int(p->Nt[1]);
      n_in[1] = int(p->Nt[0]);
    } else {
      n_in[0] = int(p->Nt[0]);
    }
    rc = mk(&p->fft, &p->fft_ok, rank_in, n_in, nullptr, 1, int(p->slice_size), int(p->slice_head), &ws[0]);
    if (rc) return rc;
    if (p->slice_tail > 0 && p->slice_tail != p->slice_head) {
      rc = mk(&p->fft_tail, &p->fft_tail_ok, rank_in, n_in, nullptr, 1, int(p->slice_size), int(p->slice_tail),
              &ws[1]);
      if (rc) return rc;
    }
    int n_l[1] = {int(p->Nt[D - 1])};
    int emb[1] = {int(p->Nt[D - 1])};
    rc = mk(&p->fft_line, &p->fft_line_ok, 1, n_l, emb, int(p->slice_size), 1, int(p->slice_size), &ws[2]);
    if (rc) return rc;
  }
  const size_t wmax = std::max(ws[0], std::max(ws[1], ws[2]));
  if (wmax > 0) {
    if (cudaMalloc(&p->fft_work, wmax) != cudaSuccess) {
      set_error("cudaMalloc of the cuFFT work area (%zu bytes) failed", wmax);
      return NFFT_ERR_ALLOC;
    }
    p->scratch_bytes += wmax;
  }
  cufftHandle hs[3] = {p->fft, p->fft_tail, p->fft_line};
  bool oks[3] = {p->fft_ok, p->fft_tail_ok, p->fft_line_ok};
  for (int i = 0; i < 3; ++i) {
    if (!oks[i]) continue;
    if ((rc = cufft_check(cufftSetWorkArea(hs[i], p->fft_work), "work area"))) return rc;
    if ((rc = cufft_check(cufftSetStream(hs[i], p->stream), "set stream"))) return rc;
  }
  return NFFT_OK;
}

// Harvest one ring slot (waits for its last event).
void harvest(nfft_plan* p, int slot) {
  const int dir = p->ring_dir[slot];
  if (dir < 0) return;
  cudaEventSynchronize(p->ev[slot][3]);
  float a = 0, b = 0, c = 0;
  cudaEventElapsedTime(&a, p->ev[slot][0], p->ev[slot][1]);
  cudaEventElapsedTime(&b, p->ev[slot][1], p->ev[slot][2]);
  cudaEventElapsedTime(&c, p->ev[slot][2], p->ev[slot][3]);
  // forward: deconv, fft, conv; adjoint: conv, fft, deconv
  const int ia = dir == 0 ? 3 : 4, ib = dir == 0 ? 2 : 5, ic = dir == 0 ? 1 : 6;
  p->timing[ia] = a * 1e-3;
  p->timing[ib] = b * 1e-3;
  p->timing[ic] = c * 1e-3;
  p->timing_sum[ia] += a * 1e-3;
  p->timing_sum[ib] += b * 1e-3;
  p->timing_sum[ic] += c * 1e-3;
  p->timing_calls[dir] += 1;
  p->ring_dir[slot] = -1;
}

void harvest_all(nfft_plan* p) {
  if (!p->timing_on) return;
  // oldest first so that timing[] ends with the latest call
  for (int q = 0; q < nfft_plan::kRing; ++q) harvest(p, int((p->ring_next + q) % nfft_plan::kRing));
}

// Slot for the next call; a full ring is harvested first.
int ring_slot(nfft_plan* p) {
  const int slot = int(p->ring_next % nfft_plan::kRing);
  if (p->ring_dir[slot] >= 0) harvest(p, slot);
  return slot;
}

void record(nfft_plan* p, int slot, int i) {
  if (p->timing_on) cudaEventRecord(p->ev[slot][i], p->stream);
}

void finish_record(nfft_plan* p, int slot, int dir) {
  if (!p->timing_on) return;
  p->ring_dir[slot] = dir;
  p->ring_next += 1;
}

}  // namespace

int exec_fft_plan(nfft_plan* p, int dir) { return exec_fft(p, dir); }

}  // namespace nfft

using namespace nfft;

extern "C" {

void nfft_params_default(nfft_params* prm) {
  if (!prm) return;
  std::memset(prm, 0, sizeof(*prm));
  prm->m = 4;
  prm->sigma = 2.0;
  prm->window = NFFT_WINDOW_KAISER_BESSEL;
  prm->precompute = NFFT_PRECOMPUTE_POLYNOMIAL;
  prm->blocking = 1;
}

const char* nfft_status_string(int s) {
  switch (s) {
    case NFFT_OK: return "ok";
    case NFFT_ERR_INVALID_ARG: return "invalid argument";
    case NFFT_ERR_DIM_MISMATCH: return "dimension mismatch";
    case NFFT_ERR_NODE_OUT_OF_RANGE: return "node out of range";
    case NFFT_ERR_ALLOC: return "device allocation failed";
    case NFFT_ERR_CUDA: return "CUDA error";
    case NFFT_ERR_CUFFT: return "cuFFT error";
    case NFFT_ERR_TIMEOUT: return "timeout";
    case NFFT_ERR_UNSUPPORTED: return "unsupported";
    case NFFT_ERR_NO_NODES: return "plan has no nodes";
  }
  return "unknown status";
}

const char* nfft_last_error(void) { return g_err; }

int64_t nfft_kernel_launch_count(void) { return g_launches.load(); }

int nfft_plan_create(nfft_plan** out, int precision, int D, const int64_t* N, int64_t M, const nfft_params* prm_in,
                     void* stream) {
  if (!out || !N) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  *out = nullptr;
  nfft_params prm;
  if (prm_in) prm = *prm_in;
  else nfft_params_default(&prm);
  if (precision != 32 && precision != 64) {
    set_error("precision must be 32 or 64");
    return NFFT_ERR_INVALID_ARG;
  }
  if (D < 1 || D > 3) {
    set_error("D = %d not supported (1..3)", D);
    return NFFT_ERR_UNSUPPORTED;
  }
  if (M < 0 || M > (int64_t(1) << 30)) {
    set_error("M = %lld out of range", (long long)M);
    return NFFT_ERR_INVALID_ARG;
  }
  if (prm.m < kMinM || prm.m > kMaxM) {
    set_error("m = %d not supported (2..8)", prm.m);
    return NFFT_ERR_UNSUPPORTED;
  }
  if (!(prm.sigma >= 1.0) || prm.sigma > 16.0) {
    set_error("sigma = %g out of range [1, 16]", prm.sigma);
    return NFFT_ERR_INVALID_ARG;
  }
  if (prm.window < 0 || prm.window > 4) {
    set_error("Window %d not yet implemented!", prm.window);
    return NFFT_ERR_UNSUPPORTED;
  }
  if (prm.precompute < 1 || prm.precompute > 4) {
    set_error("precompute = %d not supported by NFFT.jl!", prm.precompute);
    return NFFT_ERR_UNSUPPORTED;
  }
  auto* p = new nfft_plan();
  p->precision = precision;
  p->real_size = precision == 32 ? 4 : 8;
  p->D = D;
  p->M = M;
  p->prm = prm;
  p->m = prm.m;
  p->stream = static_cast<cudaStream_t>(stream);
  int64_t total = 1;
  for (int d = 0; d < D; ++d) {
    if (N[d] < 1) {
      delete p;
      set_error("N[%d] = %lld must be positive", d, (long long)N[d]);
      return NFFT_ERR_INVALID_ARG;
    }
    p->N[d] = N[d];
    // Ntilde = (ceil(sigma*N) ÷ 2) * 2, src/precomputation.jl:25-27
    p->Nt[d] = (int64_t(std::ceil(prm.sigma * double(N[d]))) / 2) * 2;
    if (p->Nt[d] < 2) p->Nt[d] = 2;
    if (p->Nt[d] >= (int64_t(1) << 30)) {
      delete p;
      set_error("oversampled size too large");
      return NFFT_ERR_UNSUPPORTED;
    }
    total *= p->Nt[d];
  }
  if (D >= 2 && p->Nt[0] * p->Nt[1] >= (int64_t(1) << 31)) {
    delete p;
    set_error("oversampled planes of 2^31 or more points are not supported");
    return NFFT_ERR_UNSUPPORTED;
  }
  if (total >= (int64_t(1) << 34)) {
    delete p;
    set_error("oversampled grid of %lld points too large", (long long)total);
    return NFFT_ERR_UNSUPPORTED;
  }
  p->sigma = double(p->Nt[0]) / double(p->N[0]);  // sigma = Ntilde/N, :30
  p->lut_size = lut_size_for(p->m);
  default_block(p);
  p->spread_pitch = spread_pitch_for(D, p->m, int(p->bs[0]) + 2 * p->m - 1,
                                     int((prm.compensated ? 4 : 2) * (precision == 32 ? 4 : 8)), 1);
  p->gather_pitch = spread_pitch_for(D == 2 ? 3 : D, p->m, int(p->bs[0]) + 2 * p->m - 1,
                                     int(2 * (precision == 32 ? 4 : 8)), 1);
  if (const char* e = getenv("NFFT_GB300_GATHER_TILED")) p->gather_tiled = e[0] == '1';
  // the shape-specialised 3-D spreader and its bulk-reduction flush (on by default)
  if (const char* e = getenv("NFFT_GB300_SPREAD_TILE3")) p->spread_tile3 = e[0] != '0';
  if (const char* e = getenv("NFFT_GB300_SPREAD_TMA")) p->spread_tma = e[0] != '0';
  if (const char* e = getenv("NFFT_GB300_GATHER_TMA")) p->gather_tma = e[0] != '0';
  // the centred internal grid of the transforms (on by default)
  if (const char* e = getenv("NFFT_GB300_CENTER")) p->center = e[0] != '0';
  // the adjoint's pre-zeroed second grid (on by default)
  if (const char* e = getenv("NFFT_GB300_PREZERO")) p->prezero = e[0] != '0';
  if (const char* e = getenv("NFFT_GB300_FFT_PRUNE")) p->fft_prune = e[0] != '0';
  if (const char* e = getenv("NFFT_GB300_SPREAD_ZERO_COPY")) p->spread_zero_copy = e[0] != '0';
  if (const char* e = getenv("NFFT_GB300_FFT_STAGED")) p->fft_staged = e[0] != '0';
  if (const char* e = getenv("NFFT_GB300_SPREAD_REC")) p->spread_rec = e[0] != '0';
  if (const char* e = getenv("NFFT_GB300_GATHER_PF")) p->gather_pf = std::max(0, std::min(64, atoi(e)));
  p->ntiles_total = 1;
  for (int d = 0; d < 3; ++d) {
    p->ntiles[d] = (p->Nt[d] + p->bs[d] - 1) / p->bs[d];
    p->ntiles_total *= p->ntiles[d];
  }
  if (p->ntiles_total >= (int64_t(1) << 31)) {
    delete p;
    set_error("too many tiles");
    return NFFT_ERR_UNSUPPORTED;
  }
  const size_t rs = p->real_size;
  auto fail = [&](int rc) {
    nfft_plan_destroy(p);
    return rc;
  };
  if (cudaMalloc(&p->grid, 2 * rs * size_t(total)) != cudaSuccess) {
    set_error("cudaMalloc of the oversampled grid (%zu bytes) failed", size_t(2 * rs * total));
    return fail(NFFT_ERR_ALLOC);
  }
  p->scratch_bytes += 2 * rs * size_t(total);
  const int64_t ninv = p->N[0] + (D > 1 ? p->N[1] : 0) + (D > 2 ? p->N[2] : 0) + 1;
  const int deg = 2 * p->m + 1, L = 2 * p->m;
  if (cudaMalloc(&p->inv, rs * ninv) != cudaSuccess || cudaMalloc(&p->coeffs, rs * deg * L) != cudaSuccess ||
      cudaMalloc(&p->dflag, 2 * sizeof(int)) != cudaSuccess || cudaMemset(p->dflag, 0, 2 * sizeof(int)) != cudaSuccess) {
    set_error("cudaMalloc of plan tables failed");
    return fail(NFFT_ERR_ALLOC);
  }
  // window polynomial (FP64 fit on the host, stored in T like Matrix{T})
  if (!poly_fit(prm.window, p->m, p->sigma, p->coeffs_host)) {
    set_error("window polynomial fit failed");
    return fail(NFFT_ERR_INVALID_ARG);
  }
  {
    std::vector<unsigned char> buf(rs * deg * L);
    for (int q = 0; q < deg * L; ++q) {
      if (precision == 32) reinterpret_cast<float*>(buf.data())[q] = float(p->coeffs_host[q]);
      else reinterpret_cast<double*>(buf.data())[q] = p->coeffs_host[q];
    }
    if (cudaMemcpy(p->coeffs, buf.data(), buf.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
      set_error("upload of window coefficients failed");
      return fail(NFFT_ERR_CUDA);
    }
    // trailing "one" factor used for singleton dimensions
    unsigned char one[8];
    if (precision == 32) { float v = 1.0f; std::memcpy(one, &v, 4); }
    else { double v = 1.0; std::memcpy(one, &v, 8); }
    if (cudaMemcpy(static_cast<char*>(p->inv) + rs * (ninv - 1), one, rs, cudaMemcpyHostToDevice) != cudaSuccess) {
      set_error("upload failed");
      return fail(NFFT_ERR_CUDA);
    }
  }
  if (prm.precompute == NFFT_PRECOMPUTE_LINEAR) {
    const int64_t K = p->lut_size;
    if (cudaMalloc(&p->lut, rs * size_t(K + 2)) != cudaSuccess) {
      set_error("cudaMalloc of the window LUT failed");
      return fail(NFFT_ERR_ALLOC);
    }
    p->scratch_bytes += rs * size_t(K + 2);
    const unsigned nb = unsigned((K + 2 + 255) / 256);
    if (precision == 32) lut_kernel<float><<<nb, 256, 0, p->stream>>>(prm.window, p->m, p->sigma, K, static_cast<float*>(p->lut));
    else lut_kernel<double><<<nb, 256, 0, p->stream>>>(prm.window, p->m, p->sigma, K, static_cast<double*>(p->lut));
    g_launches.fetch_add(1);
  }
  int rc = launch_deconv_factors(p);
  if (rc) return fail(rc);
  rc = update_center(p);
  if (rc) return fail(rc);
  // cuFFT plans (Julia's column-major grid is C order with reversed dims)
  rc = make_fft_plans(p);
  if (rc) return fail(rc);
  rc = fused_fft_init(p);
  if (rc) return fail(rc);
  if (prm.timing) {
    p->timing_on = true;
    for (int s = 0; s < nfft_plan::kRing; ++s) {
      p->ring_dir[s] = -1;
      for (int i = 0; i < 4; ++i) cudaEventCreate(&p->ev[s][i]);
    }
  }
  if (cudaStreamSynchronize(p->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    set_error("plan construction failed on the device");
    return fail(NFFT_ERR_CUDA);
  }
  *out = p;
  return NFFT_OK;
}

int nfft_plan_destroy(nfft_plan* p) {
  if (!p) return NFFT_OK;
  release_node_buffers(p);
  if (p->zero_stream) cudaStreamSynchronize(p->zero_stream);
  cudaFree(p->grid2);
  cudaFree(p->zmask);
  cudaFree(p->zero_tile);
  if (p->zero_stream) cudaStreamDestroy(p->zero_stream);
  if (p->ev_grid2_used) cudaEventDestroy(p->ev_grid2_used);
  if (p->ev_grid2_zeroed) cudaEventDestroy(p->ev_grid2_zeroed);
  cudaFree(p->grid);
  cudaFree(p->inv);
  cudaFree(p->inv_c);
  cudaFree(p->coeffs);
  cudaFree(p->lut);
  cudaFree(p->dflag);
  cudaFree(p->cbuf);
  if (p->fft_ok) cufftDestroy(p->fft);
  if (p->fft_tail_ok) cufftDestroy(p->fft_tail);
  if (p->fft_line_ok) cufftDestroy(p->fft_line);
  cudaFree(p->fft_work);
  for (int d = 0; d < 3; ++d) cudaFree(p->fft_tw[d]);
  if (p->timing_on)
    for (int s = 0; s < nfft_plan::kRing; ++s)
      for (int i = 0; i < 4; ++i) cudaEventDestroy(p->ev[s][i]);
  delete p;
  return NFFT_OK;
}

int nfft_set_stream(nfft_plan* p, void* stream) {
  if (!p) return NFFT_ERR_INVALID_ARG;
  p->stream = static_cast<cudaStream_t>(stream);
  int rc = cufft_check(cufftSetStream(p->fft, p->stream), "set stream");
  if (!rc && p->fft_tail_ok) rc = cufft_check(cufftSetStream(p->fft_tail, p->stream), "set stream");
  if (!rc && p->fft_line_ok) rc = cufft_check(cufftSetStream(p->fft_line, p->stream), "set stream");
  return rc;
}

int nfft_set_nodes(nfft_plan* p, const void* k, int k_on_device) {
  if (!p || (!k && p->M > 0)) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  auto t0 = std::chrono::steady_clock::now();
  free_nodes(p);
  const int64_t M = p->M, D = p->D;
  const size_t rs = p->real_size;
  cudaStream_t s = p->stream;
  const int L = 2 * p->m;
  const bool table = p->prm.precompute != NFFT_PRECOMPUTE_POLYNOMIAL;
  using P = nfft_plan;
  p->k = node_buffer(p, P::NB_K, rs * size_t(D * M));
  p->node4 = static_cast<int4*>(node_buffer(p, P::NB_NODE4, sizeof(int4) * size_t(M)));
  p->frac4 = node_buffer(p, P::NB_FRAC4, rs * 4 * size_t(M));
  p->wtab = table ? node_buffer(p, P::NB_WTAB, rs * size_t(M * D * L)) : nullptr;
  p->tile_start = static_cast<int32_t*>(node_buffer(p, P::NB_TSTART, sizeof(int32_t) * size_t(p->ntiles_total + 1)));
  if (!p->k || !p->node4 || !p->frac4 || (table && !p->wtab) || !p->tile_start) {
    free_nodes(p);
    return NFFT_ERR_ALLOC;
  }
  if (M > 0) {
    NFFT_CUDA_TRY(cudaMemcpyAsync(p->k, k, rs * size_t(D * M),
                                  k_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  }
  // checkNodes
  int flag = 0;
  NFFT_CUDA_TRY(cudaMemsetAsync(p->dflag, 0, sizeof(int), s));
  int rc = launch_check_nodes(p, p->k, p->dflag);
  if (rc) return rc;
  NFFT_CUDA_TRY(cudaMemcpyAsync(&flag, p->dflag, sizeof(int), cudaMemcpyDeviceToHost, s));
  NFFT_CUDA_TRY(cudaStreamSynchronize(s));
  if (flag) {
    free_nodes(p);
    set_error("Nodes k need to be within the range [-1/2, 1/2)");
    return NFFT_ERR_NODE_OUT_OF_RANGE;
  }
  const int64_t nt = p->ntiles_total;
  const int kbits = bits_for(nt);
  {
    // reduce + stable radix sort by home tile (scratch kept on the plan)
    const size_t sb = std::max(radix_sort_scratch_bytes(M), scan_scratch_bytes(nt + 1));
    auto* ti_u = static_cast<int32_t*>(node_buffer(p, P::NB_TI, sizeof(int32_t) * size_t(D * M)));
    void* te_u = node_buffer(p, P::NB_TE, rs * size_t(D * M));
    auto* key = static_cast<uint32_t*>(node_buffer(p, P::NB_KEY, sizeof(uint32_t) * size_t(M)));
    auto* val = static_cast<int32_t*>(node_buffer(p, P::NB_VAL, sizeof(int32_t) * size_t(M)));
    auto* key2 = static_cast<uint32_t*>(node_buffer(p, P::NB_KEY2, sizeof(uint32_t) * size_t(M)));
    auto* val2 = static_cast<int32_t*>(node_buffer(p, P::NB_VAL2, sizeof(int32_t) * size_t(M)));
    auto* tcount = static_cast<int32_t*>(node_buffer(p, P::NB_TCOUNT, sizeof(int32_t) * size_t(nt + 1)));
    void* scr = node_buffer(p, P::NB_SCR, sb);
    if (!ti_u || !te_u || !key || !val || !key2 || !val2 || !tcount || !scr) {
      free_nodes(p);
      return NFFT_ERR_ALLOC;
    }
    NFFT_CUDA_TRY(cudaMemsetAsync(tcount, 0, sizeof(int32_t) * size_t(nt + 1), s));
    rc = launch_reduce_nodes(p, p->k, ti_u, te_u, key, val, tcount);
    if (rc) return rc;
    uint32_t* ko = nullptr;
    int32_t* vo = nullptr;
    rc = radix_sort_pairs(key, val, key2, val2, M, kbits, scr, sb, s, &ko, &vo);
    if (rc) return rc;
    rc = exclusive_scan_i32(tcount, p->tile_start, nt + 1, scr, sb, s);
    if (rc) return rc;
    rc = launch_build_node_tables(p, vo, ti_u, te_u);
    if (rc) return rc;
  }
  if (table) {
    rc = launch_build_weight_table(p);
    if (rc) return rc;
  }
  p->scratch_bytes = size_t(2) * rs * size_t(p->Nt[0] * p->Nt[1] * p->Nt[2]) + rs * size_t(D * M) +
                     sizeof(int4) * size_t(M) + rs * 4 * size_t(M) + (table ? rs * size_t(M * D * L) : 0) +
                     sizeof(int32_t) * size_t(nt + 1);
  if (p->prm.blocking) {
    // hot tiles are split into chunks of at most `chunk` nodes (each chunk is
    // one spreading task and flushes its padded tile once);
    // NFFT_GB300_TASK_CHUNK overrides the default 1024
    int chunk = 1024;
    if (const char* e = getenv("NFFT_GB300_TASK_CHUNK")) {
      const int c = atoi(e);
      if (c >= 32 && c <= (1 << 20)) chunk = c;
    }
    rc = launch_build_tasks(p, chunk);
    if (rc) return rc;
    p->fsorted = node_buffer(p, P::NB_FSORTED, 2 * rs * size_t(M));
    if (!p->fsorted) return NFFT_ERR_ALLOC;
    p->scratch_bytes += sizeof(int4) * size_t(p->n_tasks) + 2 * rs * size_t(M);
  }
  NFFT_CUDA_TRY(cudaStreamSynchronize(s));
  NFFT_CUDA_TRY(cudaGetLastError());
  p->has_nodes = true;
  p->nodes_version += 1;
  p->timing[0] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return NFFT_OK;
}

int nfft_plan_copy(const nfft_plan* src, nfft_plan** out) {
  if (!src || !out) return NFFT_ERR_INVALID_ARG;
  int rc = nfft_plan_create(out, src->precision, src->D, src->N, src->M, &src->prm, src->stream);
  if (rc) return rc;
  (*out)->spread_layout = src->spread_layout;  // same tile shape (prm.block_size), same warp layout
  (*out)->spread_pitch = src->spread_pitch;
  if (src->has_nodes) {
    rc = nfft_set_nodes(*out, src->k, 1);
    if (rc) {
      nfft_plan_destroy(*out);
      *out = nullptr;
    }
  }
  return rc;
}

static int require_nodes(const nfft_plan* p) {
  if (!p) {
    set_error("null plan");
    return NFFT_ERR_INVALID_ARG;
  }
  if (!p->has_nodes) {
    set_error("plan has no nodes: call nfft_set_nodes first");
    return NFFT_ERR_NO_NODES;
  }
  return NFFT_OK;
}

static void zero_grid2_beside(nfft_plan* p);

int nfft_forward(nfft_plan* p, const void* f, void* fhat) {
  int rc = require_nodes(p);
  if (rc) return rc;
  CenterScope centred(p);
  const int slot = p->timing_on ? ring_slot(p) : 0;
  record(p, slot, 0);
  rc = p->fused_fft ? fused_forward_x(p, f) : launch_pad_apodize(p, f, p->grid);
  if (rc) return rc;
  record(p, slot, 1);
  rc = p->fused_fft ? fused_forward_lines(p) : exec_fft(p, CUFFT_FORWARD);
  if (rc) return rc;
  record(p, slot, 2);
  zero_grid2_beside(p);
  rc = p->prm.blocking ? launch_interp(p, p->grid, 0, fhat, 0) : launch_plain_interp(p, p->grid, 0, fhat, 0);
  if (rc) return rc;
  record(p, slot, 3);
  finish_record(p, slot, 0);
  return NFFT_OK;
}

// The adjoint's second grid: allocated (and zeroed once, in stream order) on
// first use.  After an adjoint it holds that adjoint's grid; the next forward
// transform zeroes it on the plan's side stream beside its gather (which is
// bound by on-chip traffic, so the memset's HBM writes cost it little), and
// an adjoint that finds it not yet zeroed zeroes it in order.  Not used while
// the plan's stream is being captured into a graph, for small grids (the
// memset is cheap there) or when NFFT_GB300_PREZERO=0.
static size_t grid_bytes(const nfft_plan* p) { return 2 * p->real_size * size_t(p->Nt[0] * p->Nt[1] * p->Nt[2]); }

static bool capturing(const nfft_plan* p) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(p->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone;
}

static void zero_grid2_beside(nfft_plan* p) {
  if (!p->grid2_dirty || capturing(p)) return;
  cudaEventRecord(p->ev_grid2_used, p->stream);
  cudaStreamWaitEvent(p->zero_stream, p->ev_grid2_used, 0);
  cudaMemsetAsync(p->grid2, 0, grid_bytes(p), p->zero_stream);
  cudaEventRecord(p->ev_grid2_zeroed, p->zero_stream);
  p->grid2_dirty = false;
}

static bool use_grid2(nfft_plan* p) {
  const size_t bytes = grid_bytes(p);
  if (!p->prezero || !p->prm.blocking || bytes < (size_t(64) << 20) || capturing(p)) return false;
  if (!p->grid2) {
    if (cudaMalloc(&p->grid2, bytes) != cudaSuccess) {
      p->grid2 = nullptr;
      p->prezero = false;  // not enough memory for the second grid: memset per adjoint
      cudaGetLastError();
      return false;
    }
    if (cudaStreamCreateWithFlags(&p->zero_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&p->ev_grid2_used, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&p->ev_grid2_zeroed, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventRecord(p->ev_grid2_zeroed, p->stream) != cudaSuccess) {
      p->prezero = false;
      cudaGetLastError();
      return false;
    }
    p->grid2_dirty = true;
    p->scratch_bytes += bytes;
  }
  if (p->grid2_dirty) {  // no forward transform since the last adjoint
    if (cudaMemsetAsync(p->grid2, 0, bytes, p->stream) != cudaSuccess) return false;
    p->grid2_dirty = false;
  }
  return true;
}

// Swaps the plan's grid with the zeroed second grid for one adjoint; on exit
// swaps back and marks the second grid as holding data.
struct Grid2Scope {
  nfft_plan* p;
  bool on;
  explicit Grid2Scope(nfft_plan* q) : p(q), on(use_grid2(q)) {
    if (!on) return;
    cudaStreamWaitEvent(p->stream, p->ev_grid2_zeroed, 0);
    std::swap(p->grid, p->grid2);
    p->skip_memset = true;
  }
  ~Grid2Scope() {
    if (!on) return;
    std::swap(p->grid, p->grid2);
    p->skip_memset = false;
    p->grid2_dirty = true;
  }
};

int nfft_adjoint(nfft_plan* p, const void* fhat, void* f) {
  int rc = require_nodes(p);
  if (rc) return rc;
  CenterScope centred(p);
  Grid2Scope zeroed(p);
  const int slot = p->timing_on ? ring_slot(p) : 0;
  record(p, slot, 0);
  rc = p->prm.blocking ? launch_spread(p, fhat, 0, p->grid, 0) : launch_plain_spread(p, fhat, 0, p->grid, 0);
  if (rc) return rc;
  record(p, slot, 1);
  rc = p->fused_fft ? fused_adjoint_lines(p) : exec_fft(p, CUFFT_INVERSE);
  if (rc) return rc;
  record(p, slot, 2);
  rc = p->fused_fft ? fused_adjoint_x(p, f) : launch_crop_apodize(p, p->grid, f);
  if (rc) return rc;
  record(p, slot, 3);
  finish_record(p, slot, 1);
  return NFFT_OK;
}

static int ensure_cbuf(nfft_plan* p) {
  if (p->cbuf) return NFFT_OK;
  if (cudaMalloc(&p->cbuf, 2 * p->real_size * size_t(p->M > 0 ? p->M : 1)) != cudaSuccess) {
    set_error("cudaMalloc of the node scratch failed");
    return NFFT_ERR_ALLOC;
  }
  return NFFT_OK;
}

int nfft_convolve(nfft_plan* p, const void* g, int g_real, void* fhat, int fhat_real) {
  int rc = require_nodes(p);
  if (rc) return rc;
  if (!g_real && fhat_real) {
    set_error("Complex input g requires Complex output fHat");
    return NFFT_ERR_INVALID_ARG;
  }
  const void* src = g;
  void* dst = fhat;
  if (g_real) {  // real grid -> the plan's complex grid
    rc = launch_real_to_complex(p, g, p->grid, p->Nt[0] * p->Nt[1] * p->Nt[2]);
    if (rc) return rc;
    src = p->grid;
  }
  if (fhat_real) {
    if ((rc = ensure_cbuf(p))) return rc;
    dst = p->cbuf;
  }
  rc = p->prm.blocking ? launch_interp(p, src, 0, dst, 0) : launch_plain_interp(p, src, 0, dst, 0);
  if (rc) return rc;
  if (fhat_real) rc = launch_real_part(p, dst, fhat, p->M);
  return rc;
}

int nfft_convolve_transpose(nfft_plan* p, const void* fhat, int fhat_real, void* g, int g_real) {
  int rc = require_nodes(p);
  if (rc) return rc;
  if (!fhat_real && g_real) {
    set_error("Complex input fHat requires Complex output g");
    return NFFT_ERR_INVALID_ARG;
  }
  const void* src = fhat;
  void* dst = g_real ? p->grid : g;
  if (fhat_real) {
    if ((rc = ensure_cbuf(p))) return rc;
    rc = launch_real_to_complex(p, fhat, p->cbuf, p->M);
    if (rc) return rc;
    src = p->cbuf;
  }
  rc = p->prm.blocking ? launch_spread(p, src, 0, dst, 0) : launch_plain_spread(p, src, 0, dst, 0);
  if (rc) return rc;
  if (g_real) rc = launch_real_part(p, dst, g, p->Nt[0] * p->Nt[1] * p->Nt[2]);
  return rc;
}

int nfft_deconvolve(nfft_plan* p, const void* f, void* g) {
  if (!p) return NFFT_ERR_INVALID_ARG;
  return launch_pad_apodize(p, f, g);
}

int nfft_deconvolve_transpose(nfft_plan* p, const void* g, void* f) {
  if (!p) return NFFT_ERR_INVALID_ARG;
  return launch_crop_apodize(p, g, f);
}

int nfft_grad_nodes(nfft_plan* p, const void* v, const void* w, void* dk) {
  int rc = require_nodes(p);
  if (rc) return rc;
  CenterScope centred(p);
  rc = p->fused_fft ? fused_forward_x(p, v) : launch_pad_apodize(p, v, p->grid);
  if (rc) return rc;
  rc = p->fused_fft ? fused_forward_lines(p) : exec_fft(p, CUFFT_FORWARD);
  if (rc) return rc;
  return launch_grad_nodes(p, p->grid, w, dk);
}

int nfft_get_info(const nfft_plan* p, nfft_info* info) {
  if (!p || !info) return NFFT_ERR_INVALID_ARG;
  std::memset(info, 0, sizeof(*info));
  info->precision = p->precision;
  info->D = p->D;
  for (int d = 0; d < 3; ++d) {
    info->N[d] = p->N[d];
    info->Ntilde[d] = p->Nt[d];
    info->block_size[d] = p->bs[d];
  }
  info->M = p->M;
  info->m = p->m;
  info->sigma = p->sigma;
  info->window = p->prm.window;
  info->precompute = p->prm.precompute;
  info->lut_size = p->lut_size;
  info->num_tiles = p->ntiles_total;
  info->num_spread_tasks = p->n_tasks;
  info->num_spread_entries = p->has_nodes ? p->M : 0;
  info->scratch_bytes = int64_t(p->scratch_bytes);
  return NFFT_OK;
}

void* nfft_grid(nfft_plan* p) { return p ? p->grid : nullptr; }

int nfft_get_timing(nfft_plan* p, double out[7]) {
  if (!p || !out) return NFFT_ERR_INVALID_ARG;
  NFFT_CUDA_TRY(cudaStreamSynchronize(p->stream));
  harvest_all(p);
  for (int i = 0; i < 7; ++i) out[i] = p->timing[i];
  return NFFT_OK;
}

int nfft_get_timing_totals(nfft_plan* p, double totals[7], int64_t calls[2]) {
  if (!p) return NFFT_ERR_INVALID_ARG;
  NFFT_CUDA_TRY(cudaStreamSynchronize(p->stream));
  harvest_all(p);
  if (totals)
    for (int i = 0; i < 7; ++i) totals[i] = p->timing_sum[i];
  if (calls) {
    calls[0] = p->timing_calls[0];
    calls[1] = p->timing_calls[1];
  }
  return NFFT_OK;
}

int nfft_timing_reset(nfft_plan* p) {
  if (!p) return NFFT_ERR_INVALID_ARG;
  NFFT_CUDA_TRY(cudaStreamSynchronize(p->stream));
  harvest_all(p);
  for (int i = 1; i < 7; ++i) p->timing_sum[i] = 0.0;
  p->timing_calls[0] = p->timing_calls[1] = 0;
  return NFFT_OK;
}

int nfft_get_binning(nfft_plan* p, int32_t* perm, int32_t* tile_start, int32_t* grid_index) {
  int rc = require_nodes(p);
  if (rc) return rc;
  const int64_t M = p->M, D = p->D;
  NFFT_CUDA_TRY(cudaStreamSynchronize(p->stream));
  std::vector<int4> nodes(M > 0 ? M : 1);
  if (M > 0) NFFT_CUDA_TRY(cudaMemcpy(nodes.data(), p->node4, sizeof(int4) * M, cudaMemcpyDeviceToHost));
  if (perm)
    for (int64_t i = 0; i < M; ++i) perm[i] = nodes[i].w;
  if (tile_start)
    NFFT_CUDA_TRY(cudaMemcpy(tile_start, p->tile_start, sizeof(int32_t) * (p->ntiles_total + 1), cudaMemcpyDeviceToHost));
  if (grid_index) {
    for (int64_t i = 0; i < M; ++i) {
      const int t[3] = {nodes[i].x, nodes[i].y, nodes[i].z};
      for (int d = 0; d < D; ++d)
        grid_index[d + D * int64_t(nodes[i].w)] = int32_t(wrap_any(t[d] - p->m + 1, int(p->Nt[d])));
    }
  }
  return NFFT_OK;
}

int nfft_get_deconv_factors(nfft_plan* p, void* out) {
  if (!p || !out) return NFFT_ERR_INVALID_ARG;
  const int64_t n = p->N[0] + (p->D > 1 ? p->N[1] : 0) + (p->D > 2 ? p->N[2] : 0);
  NFFT_CUDA_TRY(cudaStreamSynchronize(p->stream));
  NFFT_CUDA_TRY(cudaMemcpy(out, p->inv, p->real_size * n, cudaMemcpyDeviceToHost));
  return NFFT_OK;
}

int nfft_sync(nfft_plan* p) {
  if (!p) return NFFT_ERR_INVALID_ARG;
  NFFT_CUDA_TRY(cudaStreamSynchronize(p->stream));
  int st = 0;
  NFFT_CUDA_TRY(cudaMemcpy(&st, p->dflag + 1, sizeof(int), cudaMemcpyDeviceToHost));
  if (st) {
    NFFT_CUDA_TRY(cudaMemset(p->dflag + 1, 0, sizeof(int)));
    set_error("a bulk tensor copy into shared memory did not complete within its wait limit");
    return NFFT_ERR_TIMEOUT;
  }
  return NFFT_OK;
}

}  // extern "C"
