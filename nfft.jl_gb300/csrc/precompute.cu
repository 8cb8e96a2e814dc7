// Device precomputation of the plan: node checks, node reduction to grid
// index + fractional offset, binning keys, deconvolution factors (FP64) and
// the spreading task list.
#include "nfft_internal.cuh"

#include <math.h>

#include <algorithm>

namespace nfft {
namespace {

template <typename T>
__global__ void check_nodes_kernel(const T* __restrict__ k, int64_t n, int* __restrict__ flag) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T x = k[i];
  // checkNodes: !(abs(k) <= 0.5) also rejects NaN (src/utils.jl:46-55)
  if (!(fabs(x) <= T(0.5))) atomicOr(flag, 1);
}

template <typename T>
__global__ void reduce_nodes_kernel(const T* __restrict__ k, int D, int64_t M, int Nt0, int Nt1, int Nt2, int bs0,
                                    int bs1, int bs2, int nt0, int nt1, int32_t* __restrict__ ti,
                                    T* __restrict__ te, uint32_t* __restrict__ key, int32_t* __restrict__ val,
                                    int32_t* __restrict__ tile_count) {
  int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= M) return;
  const int Nt[3] = {Nt0, Nt1, Nt2};
  const int bs[3] = {bs0, bs1, bs2};
  int b[3] = {0, 0, 0};
  for (int d = 0; d < D; ++d) {
    int32_t t;
    T e;
    reduce_coord<T>(k[int64_t(d) + int64_t(D) * j], Nt[d], t, e);
    ti[int64_t(d) * M + j] = t;
    te[int64_t(d) * M + j] = e;
    b[d] = t / bs[d];
  }
  uint32_t kk = uint32_t(b[0] + nt0 * (b[1] + nt1 * b[2]));
  key[j] = kk;
  val[j] = int32_t(j);
  atomicAdd(&tile_count[kk], 1);
}

template <typename T>
__global__ void build_node_tables_kernel(const int32_t* __restrict__ perm, int D, int64_t M,
                                         const int32_t* __restrict__ ti_u, const T* __restrict__ te_u,
                                         int4* __restrict__ node4, T* __restrict__ frac4) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= M) return;
  const int64_t j = perm[i];
  int t[3] = {0, 0, 0};
  T e[4] = {T(0), T(0), T(0), T(0)};
  for (int d = 0; d < D; ++d) {
    t[d] = ti_u[int64_t(d) * M + j];
    e[d] = te_u[int64_t(d) * M + j];
  }
  node4[i] = make_int4(t[0], t[1], t[2], int(j));
  for (int d = 0; d < 4; ++d) frac4[4 * i + d] = e[d];
}

// Window tensor (src/precomputation.jl:556-591 for TENSOR; the window function
// itself for FULL; the LUT for LINEAR): one thread per (node, dimension, tap).
template <typename T>
__global__ void build_weight_table_kernel(Geom<T> G, const T* __restrict__ frac4, int64_t M, T* __restrict__ wtab) {
  const int L = 2 * G.m;
  const int DL = G.D * L;
  const int64_t total = M * DL;
  for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < total; q += int64_t(gridDim.x) * blockDim.x) {
    const int64_t i = q / DL;
    const int r = int(q - i * DL);
    const int d = r / L;
    const int l = r - d * L;
    wtab[q] = tap_weight<T>(G, G.coeffs, frac4[4 * i + d], l);
  }
}

// ---------------------------------------------------------------- phi-hat
// window_hat (nfft_internal.cuh)

// precomputeWindowHatInvLUT (src/precomputation.jl:347-358), FP64: per
// dimension a 30-point first-kind Chebyshev interpolant of
// phi-hat(x + indexOffset(N)) on [1, N], evaluated at x = 1..N, inverted.
// One CTA per dimension.
template <typename T>
__global__ void deconv_factors_kernel(int window, int m, double sigma, int D, int N0, int N1, int N2, int Nt0,
                                      int Nt1, int Nt2, T* __restrict__ out) {
  const int d = blockIdx.x;
  if (d >= D) return;
  const int Ns[3] = {N0, N1, N2};
  const int Nts[3] = {Nt0, Nt1, Nt2};
  const int N = Ns[d];
  const double Nt = double(Nts[d]);
  int offset = 0;
  for (int q = 0; q < d; ++q) offset += Ns[q];
  const double PI = 3.14159265358979323846;
  const int ioff = -1 - N / 2;  // indexOffset, src/precomputation.jl:345
  __shared__ double c[kChebNodes];
  __shared__ double y[kChebNodes];
  const double a = 1.0, b = double(N);
  if (N > 1) {
    for (int i = threadIdx.x; i < kChebNodes; i += blockDim.x) {
      double th = PI * (2.0 * (i + 1) - 1.0) / (2.0 * kChebNodes);
      double x = 0.5 * (b - a) * (cos(th) + 1.0) + a;
      y[i] = window_hat(window, x + ioff, Nt, m, sigma);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kChebNodes; k += blockDim.x) {
      double s = 0.0;
      for (int i = 0; i < kChebNodes; ++i) {
        double th = PI * (2.0 * (i + 1) - 1.0) / (2.0 * kChebNodes);
        s += y[i] * cos(k * th);
      }
      s *= 2.0 / kChebNodes;
      c[k] = (k == 0) ? 0.5 * s : s;
    }
    __syncthreads();
  }
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    double v;
    if (N > 1) {
      double t = (2.0 * (j + 1) - (a + b)) / (b - a);
      double b1 = 0.0, b2 = 0.0;
      for (int k = kChebNodes - 1; k >= 1; --k) {
        double tmp = 2.0 * t * b1 - b2 + c[k];
        b2 = b1;
        b1 = tmp;
      }
      v = t * b1 - b2 + c[0];
    } else {
      v = window_hat(window, double(j + 1 + ioff), Nt, m, sigma);
    }
    out[offset + j] = T(1.0 / v);
  }
}

// ------------------------------------------------------- spreading tasks
// One task per chunk of at most `chunk` nodes of a non-empty home tile.
// Tasks are listed in raster order of the tiles shifted by half the grid in
// every dimension: list position q holds tile ((q_d + nt_d / 2) mod nt_d)_d.
// The tiles at the grid's corners (the centre of k-space, where the nodes are
// dense and the tasks long) then sit in the middle of the launch, and the
// last CTAs of a launch take the short tasks of the grid's middle, so no SM
// is left with a long task while the others idle.
struct TileOrder {
  int n0, n1, n2;
  __device__ __forceinline__ int tile(int64_t q) const {
    const int q0 = int(q % n0), q1 = int((q / n0) % n1), q2 = int(q / (int64_t(n0) * n1));
    const int t0 = (q0 + n0 / 2) % n0, t1 = (q1 + n1 / 2) % n1, t2 = (q2 + n2 / 2) % n2;
    return t0 + n0 * (t1 + n1 * t2);
  }
};

__global__ void task_counts_kernel(const int32_t* __restrict__ tstart, int64_t ntiles, int chunk, TileOrder order,
                                   int32_t* __restrict__ tcnt) {
  int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= ntiles) return;
  const int t = order.tile(q);
  const int n = tstart[t + 1] - tstart[t];
  tcnt[q] = (n + chunk - 1) / chunk;
}

__global__ void fill_tasks_kernel(const int32_t* __restrict__ tstart, const int32_t* __restrict__ toff,
                                  int64_t ntiles, int chunk, TileOrder order, int4* __restrict__ tasks) {
  int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= ntiles) return;
  const int t = order.tile(q);
  const int s = tstart[t], e = tstart[t + 1];
  int pos = toff[q];
  for (int b = s; b < e; b += chunk) tasks[pos++] = make_int4(t, b, min(e, b + chunk), 0);
}

}  // namespace

template <typename T> static int check_nodes_t(const nfft_plan* p, const void* k, int* flag) {
  const int64_t n = p->M * p->D;
  if (n == 0) return NFFT_OK;
  check_nodes_kernel<T><<<unsigned((n + 255) / 256), 256, 0, p->stream>>>(static_cast<const T*>(k), n, flag);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

int launch_check_nodes(const nfft_plan* p, const void* k, int* flag) {
  return p->precision == 32 ? check_nodes_t<float>(p, k, flag) : check_nodes_t<double>(p, k, flag);
}

int launch_check_node_values(int precision, const void* k, int64_t n, int* flag, cudaStream_t s) {
  if (n == 0) return NFFT_OK;
  if (precision == 32)
    check_nodes_kernel<float><<<unsigned((n + 255) / 256), 256, 0, s>>>(static_cast<const float*>(k), n, flag);
  else
    check_nodes_kernel<double><<<unsigned((n + 255) / 256), 256, 0, s>>>(static_cast<const double*>(k), n, flag);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

template <typename T>
static int reduce_t(const nfft_plan* p, const void* k, int32_t* ti_u, void* te_u, uint32_t* key, int32_t* val,
                    int32_t* tile_count) {
  if (p->M == 0) return NFFT_OK;
  reduce_nodes_kernel<T><<<unsigned((p->M + 255) / 256), 256, 0, p->stream>>>(
      static_cast<const T*>(k), p->D, p->M, int(p->Nt[0]), int(p->Nt[1]), int(p->Nt[2]), int(p->bs[0]),
      int(p->bs[1]), int(p->bs[2]), int(p->ntiles[0]), int(p->ntiles[1]), ti_u, static_cast<T*>(te_u), key, val,
      tile_count);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

int launch_reduce_nodes(const nfft_plan* p, const void* k, int32_t* ti_u, void* te_u, uint32_t* key,
                        int32_t* val, int32_t* tile_count) {
  return p->precision == 32 ? reduce_t<float>(p, k, ti_u, te_u, key, val, tile_count)
                            : reduce_t<double>(p, k, ti_u, te_u, key, val, tile_count);
}

template <typename T>
static int node_tables_t(const nfft_plan* p, const int32_t* perm, const int32_t* ti_u, const void* te_u) {
  if (p->M == 0) return NFFT_OK;
  build_node_tables_kernel<T><<<unsigned((p->M + 255) / 256), 256, 0, p->stream>>>(
      perm, p->D, p->M, ti_u, static_cast<const T*>(te_u), p->node4, static_cast<T*>(p->frac4));
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

int launch_build_node_tables(const nfft_plan* p, const int32_t* perm, const int32_t* ti_u, const void* te_u) {
  return p->precision == 32 ? node_tables_t<float>(p, perm, ti_u, te_u) : node_tables_t<double>(p, perm, ti_u, te_u);
}

template <typename T> static int weight_table_t(const nfft_plan* p) {
  const int64_t total = p->M * p->D * 2 * p->m;
  if (total == 0) return NFFT_OK;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 64) blocks = 152 * 64;
  build_weight_table_kernel<T><<<unsigned(blocks), 256, 0, p->stream>>>(
      make_geom<T>(p), static_cast<const T*>(p->frac4), p->M, static_cast<T*>(p->wtab));
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

int launch_build_weight_table(const nfft_plan* p) {
  return p->precision == 32 ? weight_table_t<float>(p) : weight_table_t<double>(p);
}

int launch_deconv_factors(nfft_plan* p) {
  if (p->precision == 32) {
    deconv_factors_kernel<float><<<p->D, 128, 0, p->stream>>>(
        p->prm.window, p->m, p->sigma, p->D, int(p->N[0]), int(p->N[1]), int(p->N[2]), int(p->Nt[0]),
        int(p->Nt[1]), int(p->Nt[2]), static_cast<float*>(p->inv));
  } else {
    deconv_factors_kernel<double><<<p->D, 128, 0, p->stream>>>(
        p->prm.window, p->m, p->sigma, p->D, int(p->N[0]), int(p->N[1]), int(p->N[2]), int(p->Nt[0]),
        int(p->Nt[1]), int(p->Nt[2]), static_cast<double*>(p->inv));
  }
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

// Chunk the non-empty home tiles (CSR p->tile_start) into spreading tasks of
// at most `chunk` nodes.  Allocates p->tasks.
int launch_build_tasks(nfft_plan* p, int chunk) {
  const int64_t nt = p->ntiles_total;
  const size_t sb = scan_scratch_bytes(nt + 1);
  auto* tcnt = static_cast<int32_t*>(node_buffer(p, nfft_plan::NB_TCNT, sizeof(int32_t) * (nt + 1)));
  auto* toff = static_cast<int32_t*>(node_buffer(p, nfft_plan::NB_TOFF, sizeof(int32_t) * (nt + 1)));
  void* scr = node_buffer(p, nfft_plan::NB_SCR, std::max(sb, p->nbuf_cap[nfft_plan::NB_SCR]));
  if (!tcnt || !toff || !scr) return NFFT_ERR_ALLOC;
  const TileOrder order{int(p->ntiles[0]), int(p->ntiles[1]), int(p->ntiles[2])};
  task_counts_kernel<<<unsigned((nt + 255) / 256), 256, 0, p->stream>>>(p->tile_start, nt, chunk, order, tcnt);
  NFFT_LAUNCH_CHECK();
  NFFT_CUDA_TRY(cudaMemsetAsync(tcnt + nt, 0, sizeof(int32_t), p->stream));
  int rc = exclusive_scan_i32(tcnt, toff, nt + 1, scr, p->nbuf_cap[nfft_plan::NB_SCR], p->stream);
  if (rc) return rc;
  int32_t ntasks = 0;
  NFFT_CUDA_TRY(cudaMemcpyAsync(&ntasks, toff + nt, sizeof(int32_t), cudaMemcpyDeviceToHost, p->stream));
  NFFT_CUDA_TRY(cudaStreamSynchronize(p->stream));  // the task count sizes the launches
  p->n_tasks = ntasks;
  p->tasks = static_cast<int4*>(node_buffer(p, nfft_plan::NB_TASKS, sizeof(int4) * size_t(ntasks)));
  if (!p->tasks) return NFFT_ERR_ALLOC;
  if (ntasks > 0) {
    fill_tasks_kernel<<<unsigned((nt + 255) / 256), 256, 0, p->stream>>>(p->tile_start, toff, nt, chunk, order,
                                                                          p->tasks);
    NFFT_LAUNCH_CHECK();
  }
  return NFFT_OK;
}

}  // namespace nfft
