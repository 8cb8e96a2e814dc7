// Batched plans: many NFFT plans of uneven N and M transformed together.
// No reference counterpart (the reference transforms one plan per call).
//
// Every stage runs as ONE launch over all plans (a per-plan descriptor table
// in device memory, plans found by binary search over prefix sums):
//   forward:  pad+apodize (grid-stride over all plans' grid pairs), the
//             plans' FFTs, gather (persistent warps over all plans' nodes);
//   adjoint:  grid zero-fill, value sort, spreading (persistent CTAs taking
//             tasks of all plans from one atomic counter), the plans' FFTs,
//             crop+apodize.
// The plans' FFTs run concurrently on forked streams: the fused pruned FFT
// (with its own pad / crop, reading the image pointer from the per-call
// table) for power-of-two grids, cuFFT for the others.
// The whole sequence of a direction is captured once into a CUDA graph and
// replayed; per call only the table of input/output pointers is copied.
// Plans in a batch share precision, dimension (2 or 3), m, window-evaluation
// mode and spreading variant; their tiles, grids and node sets may differ.
#include "interp_body.cuh"
#include "spread_body.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

struct nfft_batch {
  std::vector<nfft_plan*> plans;
  std::vector<int64_t> versions;  // each plan's node-set version at creation
  int n = 0;
  int precision = 32, D = 3, m = 4;
  bool table = false;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;  // made when the caller passes the legacy default stream
  // the plans' FFTs are independent: inside the captured graph they run on
  // kSide forked streams (plan i on side[i % kSide]) and join before the
  // next stage, so small transforms overlap instead of running back to back
  static constexpr int kSide = 8;
  cudaStream_t side[kSide] = {};
  cudaEvent_t fork_ev = nullptr;
  cudaEvent_t join_ev[kSide] = {};
  void* d_items = nullptr;        // BatchItem<T>[n]
  int64_t* d_base = nullptr;      // 5 prefix arrays of n+1: pairs, nodes, tasks, image, grid
  void** d_ptrs = nullptr;        // per call: input/output pointer of each plan
  int* d_counter = nullptr;       // persistent spreading task counter
  // pinned ring of per-call pointer tables: a slot is refilled only after the
  // copy that last read it has run (its event), so the copy never stalls the host
  static constexpr int kSlots = 8;
  void** h_ring = nullptr;        // kSlots x 2n
  cudaEvent_t ring_ev[kSlots] = {};
  bool ring_used[kSlots] = {};
  int ring_next = 0;
  int64_t total[5] = {};
  size_t spread_smem = 0;
  int spread_ctas = 0, gather_ctas = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  cudaGraph_t graph_def[2] = {nullptr, nullptr};
};

namespace nfft {
namespace {

enum { B_PAIRS = 0, B_NODES = 1, B_TASKS = 2, B_IMAGE = 3, B_GRID = 4 };

template <typename T> struct BatchItem {
  Geom<T> G;
  Nodes<T> Nd;
  const int4* tasks;
  int pitch;
  T* grid;
  typename Cplx<T>::type* fsorted;
  int N[3];
  const T* inv[3];
};

__device__ __forceinline__ int find_plan(const int64_t* __restrict__ base, int n, int64_t x) {
  int lo = 0, hi = n - 1;  // largest p with base[p] <= x
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(base + mid) <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <typename T>
__global__ void __launch_bounds__(256) batch_pad_kernel(const BatchItem<T>* __restrict__ items, const int64_t* base,
                                                        int n, int64_t total, void* const* __restrict__ ptrs) {
  using C = typename Cplx<T>::type;
  for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < total; q += int64_t(gridDim.x) * blockDim.x) {
    const int pi = find_plan(base, n, q);
    const BatchItem<T>& it = items[pi];
    const int64_t lq = q - __ldg(base + pi);
    const int Nt0 = it.G.Nt[0], Nt1 = it.G.Nt[1], Nt2 = it.G.Nt[2];
    const int half = Nt0 >> 1;
    const int64_t row = lq / half;
    const int gx = int(lq - row * half) * 2;
    const int gy = int(row % Nt1), gz = int(row / Nt1);
    const int ny = wrap_once(gy + it.N[1] / 2, Nt1), nz = wrap_once(gz + it.N[2] / 2, Nt2);
    C v0 = {T(0), T(0)}, v1 = {T(0), T(0)};
    if (ny < it.N[1] && nz < it.N[2]) {
      const C* f = static_cast<const C*>(ptrs[2 * pi]);
      const T s = __ldg(it.inv[1] + ny) * __ldg(it.inv[2] + nz);
      const int64_t frow = int64_t(it.N[0]) * (ny + int64_t(it.N[1]) * nz);
      const int nx0 = wrap_once(gx + it.N[0] / 2, Nt0), nx1 = wrap_once(gx + 1 + it.N[0] / 2, Nt0);
      if (nx0 < it.N[0]) {
        const C a = f[frow + nx0];
        const T w = __ldg(it.inv[0] + nx0) * s;
        v0.x = a.x * w;
        v0.y = a.y * w;
      }
      if (nx1 < it.N[0]) {
        const C a = f[frow + nx1];
        const T w = __ldg(it.inv[0] + nx1) * s;
        v1.x = a.x * w;
        v1.y = a.y * w;
      }
    }
    C* out = reinterpret_cast<C*>(it.grid) + row * Nt0 + gx;
    out[0] = v0;
    out[1] = v1;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) batch_crop_kernel(const BatchItem<T>* __restrict__ items, const int64_t* base,
                                                         int n, int64_t total, void* const* __restrict__ ptrs) {
  using C = typename Cplx<T>::type;
  for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < total; q += int64_t(gridDim.x) * blockDim.x) {
    const int pi = find_plan(base, n, q);
    const BatchItem<T>& it = items[pi];
    const int64_t lq = q - __ldg(base + pi);
    const int64_t row = lq / it.N[0];
    const int nx = int(lq - row * it.N[0]);
    const int ny = int(row % it.N[1]), nz = int(row / it.N[1]);
    const int gx = wrap_once(nx - it.N[0] / 2, it.G.Nt[0]);
    const int gy = wrap_once(ny - it.N[1] / 2, it.G.Nt[1]);
    const int gz = wrap_once(nz - it.N[2] / 2, it.G.Nt[2]);
    const C a = reinterpret_cast<const C*>(it.grid)[gx + int64_t(it.G.Nt[0]) * (gy + int64_t(it.G.Nt[1]) * gz)];
    const T w = __ldg(it.inv[0] + nx) * __ldg(it.inv[1] + ny) * __ldg(it.inv[2] + nz);
    C r;
    r.x = a.x * w;
    r.y = a.y * w;
    static_cast<C*>(ptrs[2 * pi + 1])[lq] = r;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) batch_zero_kernel(const BatchItem<T>* __restrict__ items, const int64_t* base,
                                                         int n, int64_t total) {
  using C = typename Cplx<T>::type;
  for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < total; q += int64_t(gridDim.x) * blockDim.x) {
    const int pi = find_plan(base, n, q);
    C z;
    z.x = T(0);
    z.y = T(0);
    reinterpret_cast<C*>(items[pi].grid)[q - __ldg(base + pi)] = z;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) batch_sort_values_kernel(const BatchItem<T>* __restrict__ items,
                                                                const int64_t* base, int n, int64_t total,
                                                                void* const* __restrict__ ptrs) {
  using C = typename Cplx<T>::type;
  for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < total; q += int64_t(gridDim.x) * blockDim.x) {
    const int pi = find_plan(base, n, q);
    const BatchItem<T>& it = items[pi];
    const int64_t i = q - __ldg(base + pi);
    it.fsorted[i] = static_cast<const C*>(ptrs[2 * pi])[__ldg(it.Nd.node4 + i).w];
  }
}

// Gather: each CTA takes a contiguous chunk of the concatenated (bin-sorted)
// node ranges, so the nodes an SM visits close in time share their grid
// neighbourhood in L1 (as in the single-plan gather).
template <int D, int L, typename T, bool TABLE>
__global__ void __launch_bounds__(256) batch_gather_kernel(const BatchItem<T>* __restrict__ items, const int64_t* base,
                                                           int n, int64_t total, void* const* __restrict__ ptrs) {
  using C = typename Cplx<T>::type;
  const int lane = threadIdx.x & 31;
  const int64_t chunk = (total + gridDim.x - 1) / gridDim.x;
  const int64_t lo = int64_t(blockIdx.x) * chunk;
  const int64_t hi = lo + chunk < total ? lo + chunk : total;
  PolyRegs<D, L, T> P;
  // the chunk is contiguous: the plan (and its descriptor) changes only at
  // plan boundaries, so it is looked up once per plan, not per node
  // (D = 2 keeps the descriptor in registers; the 3-D node body needs its
  // registers, so there the fields are read through L1 as needed -- both
  // measured fastest for their dimension)
  int64_t pbeg = 0, pend = -1;
  int pi = 0;
  Geom<T> G2{};
  Nodes<T> N2{};
  for (int64_t q = lo + (threadIdx.x >> 5); q < hi; q += blockDim.x >> 5) {
    if (q >= pend) {
      pi = find_plan(base, n, q);
      pbeg = __ldg(base + pi);
      pend = __ldg(base + pi + 1);
      if constexpr (D == 2) {
        G2 = items[pi].G;
        N2 = items[pi].Nd;
      }
      if constexpr (!TABLE) P.load(items[pi].G.coeffs, lane);
    }
    const BatchItem<T>& it = items[pi];
    const C* grid = reinterpret_cast<const C*>(it.grid);
    C* out = static_cast<C*>(ptrs[2 * pi + 1]);
    if constexpr (D == 2) interp_node<D, L, T, TABLE>(G2, N2, P, q - pbeg, lane, grid, out);
    else interp_node<D, L, T, TABLE>(it.G, it.Nd, P, q - pbeg, lane, grid, out);
  }
}

// Persistent spreading: CTAs take tasks of all plans from one counter.
template <int D, int L, typename T, bool TABLE>
__global__ void __launch_bounds__(OwnedCfg<D, L>::THREADS) batch_spread_kernel(const BatchItem<T>* __restrict__ items,
                                                                               const int64_t* base, int n,
                                                                               int64_t total, int* counter) {
  __shared__ int s_task;
  for (;;) {
    __syncthreads();  // the previous task's flush has read the shared tile
    if (threadIdx.x == 0) s_task = atomicAdd(counter, 1);
    __syncthreads();
    const int64_t q = s_task;
    if (q >= total) break;
    const int pi = find_plan(base, n, q);
    const BatchItem<T>& it = items[pi];
    const Geom<T> G = it.G;
    const Nodes<T> Nd = it.Nd;
    const int4 task = it.tasks[q - __ldg(base + pi)];
    spread_owned_body<D, L, T, TABLE, false>(G, Nd, task, it.fsorted, it.grid, it.pitch);
  }
}

int grid_for_items(int64_t work, int per_block) {
  int64_t b = (work + per_block - 1) / per_block;
  const int64_t cap = 152 * 16;
  if (b > cap) b = cap;
  return int(b < 1 ? 1 : b);
}

// All plans' grid FFTs, forked over the side streams and joined back into
// the batch stream (only ever called while the batch stream is captured).
int forked_ffts(nfft_batch* B, int dir) {
  const int ns = std::min(B->n, nfft_batch::kSide);
  NFFT_CUDA_TRY(cudaEventRecord(B->fork_ev, B->stream));
  for (int s = 0; s < ns; ++s) NFFT_CUDA_TRY(cudaStreamWaitEvent(B->side[s], B->fork_ev, 0));
  int rc = NFFT_OK;
  for (int i = 0; i < B->n && !rc; ++i) {
    nfft_plan* p = B->plans[i];
    rc = nfft_set_stream(p, B->side[i % ns]);
    if (rc) break;
    if (p->fused_fft) {
      // fused pruned FFT with pad (forward) or crop (adjoint) inside; the
      // image pointer is read from the batch's per-call pointer table
      if (dir == CUFFT_FORWARD) {
        rc = fused_forward_x(p, nullptr, B->d_ptrs + 2 * i);
        if (!rc) rc = fused_forward_lines(p);
      } else {
        rc = fused_adjoint_lines(p);
        if (!rc) rc = fused_adjoint_x(p, nullptr, B->d_ptrs + 2 * i + 1);
      }
    } else {
      rc = exec_fft_plan(p, dir);
    }
  }
  for (int s = 0; s < ns; ++s) {
    NFFT_CUDA_TRY(cudaEventRecord(B->join_ev[s], B->side[s]));
    NFFT_CUDA_TRY(cudaStreamWaitEvent(B->stream, B->join_ev[s], 0));
  }
  for (nfft_plan* p : B->plans) {
    const int r2 = nfft_set_stream(p, B->stream);
    if (!rc) rc = r2;
  }
  return rc;
}

template <int D, int L, typename T, bool TABLE> struct Launch {
  static int forward(nfft_batch* B) {
    const auto* items = static_cast<const BatchItem<T>*>(B->d_items);
    const int64_t* base = B->d_base;
    batch_pad_kernel<T><<<grid_for_items(B->total[B_PAIRS], 256), 256, 0, B->stream>>>(
        items, base + B_PAIRS * (B->n + 1), B->n, B->total[B_PAIRS], B->d_ptrs);
    NFFT_LAUNCH_CHECK();
    int rc = forked_ffts(B, CUFFT_FORWARD);
    if (rc) return rc;
    batch_gather_kernel<D, L, T, TABLE><<<B->gather_ctas, 256, 0, B->stream>>>(
        items, base + B_NODES * (B->n + 1), B->n, B->total[B_NODES], B->d_ptrs);
    NFFT_LAUNCH_CHECK();
    return NFFT_OK;
  }
  static int adjoint(nfft_batch* B) {
    const auto* items = static_cast<const BatchItem<T>*>(B->d_items);
    const int64_t* base = B->d_base;
    batch_zero_kernel<T><<<grid_for_items(B->total[B_GRID], 256), 256, 0, B->stream>>>(
        items, base + B_GRID * (B->n + 1), B->n, B->total[B_GRID]);
    NFFT_LAUNCH_CHECK();
    batch_sort_values_kernel<T><<<grid_for_items(B->total[B_NODES], 256), 256, 0, B->stream>>>(
        items, base + B_NODES * (B->n + 1), B->n, B->total[B_NODES], B->d_ptrs);
    NFFT_LAUNCH_CHECK();
    NFFT_CUDA_TRY(cudaMemsetAsync(B->d_counter, 0, sizeof(int), B->stream));
    batch_spread_kernel<D, L, T, TABLE><<<B->spread_ctas, OwnedCfg<D, L>::THREADS, B->spread_smem, B->stream>>>(
        items, base + B_TASKS * (B->n + 1), B->n, B->total[B_TASKS], B->d_counter);
    NFFT_LAUNCH_CHECK();
    int rc = forked_ffts(B, CUFFT_INVERSE);
    if (rc) return rc;
    batch_crop_kernel<T><<<grid_for_items(B->total[B_IMAGE], 256), 256, 0, B->stream>>>(
        items, base + B_IMAGE * (B->n + 1), B->n, B->total[B_IMAGE], B->d_ptrs);
    NFFT_LAUNCH_CHECK();
    return NFFT_OK;
  }
  static int setup(nfft_batch* B) {
    for (nfft_plan* p : B->plans) B->spread_smem = std::max(B->spread_smem, owned_smem<D, L, T>(p, false));
    if (B->spread_smem > 227 * 1024) return NFFT_OK;  // rejected by the caller
    auto kern = batch_spread_kernel<D, L, T, TABLE>;
    NFFT_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(B->spread_smem)));
    int per_sm = 0;
    NFFT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, OwnedCfg<D, L>::THREADS,
                                                                B->spread_smem));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t ctas = int64_t(std::max(per_sm, 1)) * sms;
    B->spread_ctas = int(std::max<int64_t>(1, std::min<int64_t>(ctas, B->total[B_TASKS])));
    // gather: CTAs of 8 warps, one contiguous node chunk each (8 nodes per warp
    // and CTA at least), at most 64 CTAs per SM
    const int64_t want = (B->total[B_NODES] + 63) / 64;
    B->gather_ctas = int(std::max<int64_t>(1, std::min<int64_t>(want, int64_t(sms) * 64)));
    return NFFT_OK;
  }
};

template <typename T, bool TABLE> int dispatch(nfft_batch* B, int what) {
#define NFFT_BATCH_CASE(DD, LL)                                                               \
  if (B->D == DD && 2 * B->m == LL)                                                           \
    return what == 0 ? Launch<DD, LL, T, TABLE>::setup(B)                                     \
                     : (what == 1 ? Launch<DD, LL, T, TABLE>::forward(B) : Launch<DD, LL, T, TABLE>::adjoint(B));
  NFFT_BATCH_CASE(2, 4) NFFT_BATCH_CASE(2, 6) NFFT_BATCH_CASE(2, 8) NFFT_BATCH_CASE(2, 10)
  NFFT_BATCH_CASE(2, 12) NFFT_BATCH_CASE(2, 14) NFFT_BATCH_CASE(2, 16)
  NFFT_BATCH_CASE(3, 4) NFFT_BATCH_CASE(3, 6) NFFT_BATCH_CASE(3, 8) NFFT_BATCH_CASE(3, 10)
  NFFT_BATCH_CASE(3, 12) NFFT_BATCH_CASE(3, 14) NFFT_BATCH_CASE(3, 16)
#undef NFFT_BATCH_CASE
  set_error("batched plans support D = 2 or 3 and m = 2..8");
  return NFFT_ERR_UNSUPPORTED;
}

int run(nfft_batch* B, int what) {
  if (B->precision == 32) return B->table ? dispatch<float, true>(B, what) : dispatch<float, false>(B, what);
  return B->table ? dispatch<double, true>(B, what) : dispatch<double, false>(B, what);
}

template <typename T> int fill_items(nfft_batch* B) {
  std::vector<BatchItem<T>> items(B->n);
  std::vector<int64_t> base(5 * (B->n + 1), 0);
  for (int i = 0; i < B->n; ++i) {
    nfft_plan* p = B->plans[i];
    BatchItem<T>& it = items[i];
    it.G = make_geom<T>(p);
    it.Nd = make_nodes<T>(p);
    it.tasks = p->tasks;
    it.pitch = p->spread_pitch;
    it.grid = static_cast<T*>(p->grid);
    it.fsorted = static_cast<typename Cplx<T>::type*>(p->fsorted);
    const T* inv = static_cast<const T*>(p->inv);
    const int64_t nsum = p->N[0] + (p->D > 1 ? p->N[1] : 0) + (p->D > 2 ? p->N[2] : 0);
    for (int d = 0; d < 3; ++d) it.N[d] = int(p->N[d]);
    it.inv[0] = inv;
    it.inv[1] = p->D > 1 ? inv + p->N[0] : inv + nsum;
    it.inv[2] = p->D > 2 ? inv + p->N[0] + p->N[1] : inv + nsum;
    const int64_t grid = p->Nt[0] * p->Nt[1] * p->Nt[2];
    // plans on the fused pruned FFT pad and crop inside their x-line kernels
    const int64_t sizes[5] = {p->fused_fft ? 0 : grid / 2, p->M, p->n_tasks,
                              p->fused_fft ? 0 : p->N[0] * p->N[1] * p->N[2], grid};
    for (int a = 0; a < 5; ++a) base[a * (B->n + 1) + i + 1] = base[a * (B->n + 1) + i] + sizes[a];
  }
  for (int a = 0; a < 5; ++a) B->total[a] = base[a * (B->n + 1) + B->n];
  NFFT_CUDA_TRY(cudaMalloc(&B->d_items, sizeof(BatchItem<T>) * B->n));
  NFFT_CUDA_TRY(cudaMalloc(&B->d_base, sizeof(int64_t) * base.size()));
  NFFT_CUDA_TRY(cudaMemcpy(B->d_items, items.data(), sizeof(BatchItem<T>) * B->n, cudaMemcpyHostToDevice));
  NFFT_CUDA_TRY(cudaMemcpy(B->d_base, base.data(), sizeof(int64_t) * base.size(), cudaMemcpyHostToDevice));
  return NFFT_OK;
}

}  // namespace
}  // namespace nfft

using namespace nfft;

extern "C" int nfft_batch_destroy(nfft_batch* B) {
  if (!B) return NFFT_OK;
  for (int d = 0; d < 2; ++d) {
    if (B->graph[d]) cudaGraphExecDestroy(B->graph[d]);
    if (B->graph_def[d]) cudaGraphDestroy(B->graph_def[d]);
  }
  cudaFree(B->d_items);
  cudaFree(B->d_base);
  cudaFree(B->d_ptrs);
  cudaFree(B->d_counter);
  for (int i = 0; i < nfft_batch::kSlots; ++i)
    if (B->ring_ev[i]) cudaEventDestroy(B->ring_ev[i]);
  cudaFreeHost(B->h_ring);
  for (int s = 0; s < nfft_batch::kSide; ++s) {
    if (B->side[s]) cudaStreamDestroy(B->side[s]);
    if (B->join_ev[s]) cudaEventDestroy(B->join_ev[s]);
  }
  if (B->fork_ev) cudaEventDestroy(B->fork_ev);
  if (B->own_stream) cudaStreamDestroy(B->own_stream);
  delete B;
  return NFFT_OK;
}

extern "C" int nfft_batch_create(nfft_batch** out, nfft_plan* const* plans, int nplans, void* stream) {
  if (!out || !plans || nplans < 1) {
    set_error("need at least one plan");
    return NFFT_ERR_INVALID_ARG;
  }
  *out = nullptr;
  auto* B = new nfft_batch();
  B->stream = static_cast<cudaStream_t>(stream);
  if (!B->stream) {
    // the legacy default stream cannot be captured into a graph; a blocking
    // stream keeps the implicit ordering with it
    if (cudaStreamCreate(&B->own_stream) != cudaSuccess) {
      delete B;
      set_error("cudaStreamCreate failed");
      return NFFT_ERR_CUDA;
    }
    B->stream = B->own_stream;
  }
  const nfft_plan* p0 = plans[0];
  for (int i = 0; i < nplans; ++i) {
    nfft_plan* p = plans[i];
    if (!p || !p->has_nodes || !p->prm.blocking || p->prm.compensated || p->precision != p0->precision ||
        p->D != p0->D || p->m != p0->m ||
        (p->prm.precompute == NFFT_PRECOMPUTE_POLYNOMIAL) != (p0->prm.precompute == NFFT_PRECOMPUTE_POLYNOMIAL)) {
      nfft_batch_destroy(B);
      set_error("plan %d cannot join the batch: plans need nodes, blocking, no compensation, and the same "
                "precision, D, m and window-evaluation mode", i);
      return NFFT_ERR_INVALID_ARG;
    }
    B->plans.push_back(p);
    B->versions.push_back(p->nodes_version);
  }
  B->n = nplans;
  B->precision = p0->precision;
  B->D = p0->D;
  B->m = p0->m;
  B->table = p0->prm.precompute != NFFT_PRECOMPUTE_POLYNOMIAL;
  if (B->D < 2) {
    nfft_batch_destroy(B);
    set_error("batched plans support D = 2 or 3");
    return NFFT_ERR_UNSUPPORTED;
  }
  int rc = B->precision == 32 ? fill_items<float>(B) : fill_items<double>(B);
  if (!rc && (cudaMalloc(&B->d_ptrs, sizeof(void*) * 2 * nplans) != cudaSuccess ||
              cudaMalloc(&B->d_counter, sizeof(int)) != cudaSuccess ||
              cudaMallocHost(&B->h_ring, sizeof(void*) * 2 * nplans * nfft_batch::kSlots) != cudaSuccess)) {
    set_error("allocation of batch tables failed");
    rc = NFFT_ERR_ALLOC;
  }
  for (int i = 0; !rc && i < nfft_batch::kSlots; ++i)
    if (cudaEventCreateWithFlags(&B->ring_ev[i], cudaEventDisableTiming) != cudaSuccess) {
      set_error("cudaEventCreate failed");
      rc = NFFT_ERR_CUDA;
    }
  if (!rc && cudaEventCreateWithFlags(&B->fork_ev, cudaEventDisableTiming) != cudaSuccess) rc = NFFT_ERR_CUDA;
  for (int s = 0; !rc && s < nfft_batch::kSide; ++s)
    if (cudaStreamCreateWithFlags(&B->side[s], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&B->join_ev[s], cudaEventDisableTiming) != cudaSuccess) {
      set_error("side stream creation failed");
      rc = NFFT_ERR_CUDA;
    }
  if (!rc) rc = run(B, 0);
  if (!rc && B->spread_smem > 227 * 1024) {
    set_error("a plan's padded spreading tile does not fit in shared memory");
    rc = NFFT_ERR_UNSUPPORTED;
  }
  if (!rc) {
    for (nfft_plan* p : B->plans) {
      rc = nfft_set_stream(p, B->stream);
      if (rc) break;
    }
  }
  if (rc) {
    nfft_batch_destroy(B);
    return rc;
  }
  *out = B;
  return NFFT_OK;
}

// dir 0 = forward (in: images f, out: node values fHat), 1 = adjoint.
static int batch_exec(nfft_batch* B, const void* const* in, void* const* out, int dir) {
  if (!B || !in || !out) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  const int slot = B->ring_next;
  if (B->ring_used[slot]) NFFT_CUDA_TRY(cudaEventSynchronize(B->ring_ev[slot]));
  void** h = B->h_ring + size_t(2) * B->n * slot;
  for (int i = 0; i < B->n; ++i) {
    if (!B->plans[i]->has_nodes || B->plans[i]->nodes_version != B->versions[i]) {
      set_error("plan %d of the batch has new nodes since the batch was created; create the batch again", i);
      return NFFT_ERR_INVALID_ARG;
    }
    // node arrays of a plan without nodes may be NULL (never read or written)
    const bool empty = B->plans[i]->M == 0;
    if ((!in[i] && !(empty && dir == 1)) || (!out[i] && !(empty && dir == 0))) {
      set_error("null array for plan %d", i);
      return NFFT_ERR_INVALID_ARG;
    }
    h[2 * i] = const_cast<void*>(in[i]);
    h[2 * i + 1] = out[i];
  }
  NFFT_CUDA_TRY(cudaMemcpyAsync(B->d_ptrs, h, sizeof(void*) * 2 * B->n, cudaMemcpyHostToDevice, B->stream));
  NFFT_CUDA_TRY(cudaEventRecord(B->ring_ev[slot], B->stream));
  B->ring_used[slot] = true;
  B->ring_next = (slot + 1) % nfft_batch::kSlots;
  if (!B->graph[dir]) {
    NFFT_CUDA_TRY(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
    int rc = run(B, dir == 0 ? 1 : 2);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(B->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) {
      set_error("graph capture failed: %s", cudaGetErrorString(e));
      return NFFT_ERR_CUDA;
    }
    B->graph_def[dir] = g;
    NFFT_CUDA_TRY(cudaGraphInstantiate(&B->graph[dir], g, 0));
  }
  NFFT_CUDA_TRY(cudaGraphLaunch(B->graph[dir], B->stream));
  return NFFT_OK;
}

extern "C" int nfft_batch_forward(nfft_batch* B, const void* const* f, void* const* fhat) {
  return batch_exec(B, f, fhat, 0);
}

extern "C" int nfft_batch_adjoint(nfft_batch* B, const void* const* fhat, void* const* f) {
  return batch_exec(B, fhat, f, 1);
}
