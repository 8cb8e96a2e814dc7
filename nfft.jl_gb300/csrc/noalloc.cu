// nfft_bin_nodes_noalloc: the node binning of nfft_set_nodes (node check,
// reduction to grid index, stable radix sort by tile) without any device
// allocation.  Its scratch memory is a file-scope __device__ array that every
// GPU loading this library holds until the process exits.
//
// Why it exists: some callers cannot call cudaMalloc at the point where they
// bin nodes -- for example a host framework whose caching allocator already
// owns the device memory (a foreign cudaMalloc can fail although the pool has
// room), or a latency-critical pipeline that must not take the implicit
// device synchronisation of cudaMalloc/cudaFree.  They pass inputs and
// outputs; this entry point brings nothing else but the static scratch.
#include "nfft_internal.cuh"

#include <algorithm>
#include <map>
#include <mutex>

namespace {

// Limits of the static scratch.
constexpr int64_t kMaxNodes = int64_t(1) << 18;   // 262,144 nodes
constexpr int64_t kMaxTiles = int64_t(1) << 18;   // 262,144 tiles
constexpr size_t kScratchBytes = size_t(16) << 20;  // 16 MiB

static __device__ __align__(256) unsigned char g_bin_scratch[kScratchBytes];

std::mutex g_setup_mutex;
// device address of g_bin_scratch per CUDA context (by the driver's unique
// context id, so a context that was reset and re-created is looked up anew)
std::map<unsigned long long, void*> g_scratch_ptr;

using CtxGetCurrentFn = int (*)(void**);
using CtxGetIdFn = int (*)(void*, unsigned long long*);

// Unique id of the calling thread's current context, 0 if the driver does not
// provide one.  The driver entry points are resolved through the runtime, so
// the library does not link the driver library itself.
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* a = nullptr;
    void* b = nullptr;
    cudaDriverEntryPointQueryResult qa{}, qb{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
        qa == cudaDriverEntryPointSuccess && a &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
        qb == cudaDriverEntryPointSuccess && b) {
      get_current = reinterpret_cast<CtxGetCurrentFn>(a);
      get_id = reinterpret_cast<CtxGetIdFn>(b);
    }
  });
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == 0 && ctx && get_id(ctx, &id) == 0) return id;
  return 0;
}

// Device address of g_bin_scratch in the current device's context.  In host
// code the symbol is only a host-side stand-in, so the address is looked up
// with cudaGetSymbolAddress, with that device current, on the first call made
// in each context (which also loads the module there; this first call should
// come before any stream capture).  Without a context id the lookup is
// repeated on every call.
int scratch_for_current_device(void** out) {
  unsigned long long ctx = current_context_id();  // 0 before the runtime made a context current
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (ctx) {
    auto it = g_scratch_ptr.find(ctx);
    if (it != g_scratch_ptr.end()) {
      *out = it->second;
      return NFFT_OK;
    }
  }
  void* ptr = nullptr;
  cudaError_t err = cudaGetSymbolAddress(&ptr, g_bin_scratch);
  if (err != cudaSuccess || !ptr) {
    nfft::set_error("cudaGetSymbolAddress of the binning scratch failed: %s", cudaGetErrorString(err));
    return NFFT_ERR_CUDA;
  }
  if (!ctx) ctx = current_context_id();  // the lookup initialised the device's primary context
  if (ctx) g_scratch_ptr[ctx] = ptr;
  *out = ptr;
  return NFFT_OK;
}

size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

}  // namespace

extern "C" int nfft_bin_nodes_noalloc(int precision, int D, const int64_t* Ntilde, const int64_t* block_size,
                                      int64_t M, const void* k, int32_t* perm, int32_t* tile_start,
                                      void* stream) {
  using namespace nfft;
  if (!Ntilde || !block_size || (M > 0 && (!k || !perm)) || !tile_start) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  if (precision != 32 && precision != 64) {
    set_error("precision must be 32 or 64");
    return NFFT_ERR_INVALID_ARG;
  }
  if (D < 1 || D > 3) {
    set_error("D = %d not supported (1..3)", D);
    return NFFT_ERR_UNSUPPORTED;
  }
  if (M < 0 || M > kMaxNodes) {
    set_error("nfft_bin_nodes_noalloc handles at most %lld nodes (got %lld)", (long long)kMaxNodes,
              (long long)M);
    return NFFT_ERR_UNSUPPORTED;
  }
  // A plan descriptor on the host stack: only its geometry is used by the
  // launchers below; it owns no device memory.
  nfft_plan g;
  g.precision = precision;
  g.real_size = precision == 32 ? 4 : 8;
  g.D = D;
  g.M = M;
  g.stream = static_cast<cudaStream_t>(stream);
  g.ntiles_total = 1;
  for (int d = 0; d < 3; ++d) {
    const int64_t nt = d < D ? Ntilde[d] : 1;
    const int64_t b = d < D ? block_size[d] : 1;
    if (nt < 1 || nt >= (int64_t(1) << 30) || b < 1 || b > nt) {
      set_error("invalid Ntilde / block size in dimension %d", d);
      return NFFT_ERR_INVALID_ARG;
    }
    g.Nt[d] = nt;
    g.bs[d] = b;
    g.ntiles[d] = (nt + b - 1) / b;
    g.ntiles_total *= g.ntiles[d];
  }
  if (g.ntiles_total > kMaxTiles) {
    set_error("nfft_bin_nodes_noalloc handles at most %lld tiles (got %lld)", (long long)kMaxTiles,
              (long long)g.ntiles_total);
    return NFFT_ERR_UNSUPPORTED;
  }
  const int64_t nt = g.ntiles_total;
  // Scratch layout: flag | ti | te | key | val | key2 | val2 | tile_count | sort/scan scratch
  size_t off = 0;
  const size_t o_flag = off; off += align256(sizeof(int));
  const size_t o_ti = off;   off += align256(sizeof(int32_t) * size_t(D * M));
  const size_t o_te = off;   off += align256(g.real_size * size_t(D * M));
  const size_t o_k1 = off;   off += align256(sizeof(uint32_t) * size_t(M));
  const size_t o_v1 = off;   off += align256(sizeof(int32_t) * size_t(M));
  const size_t o_k2 = off;   off += align256(sizeof(uint32_t) * size_t(M));
  const size_t o_v2 = off;   off += align256(sizeof(int32_t) * size_t(M));
  const size_t o_tc = off;   off += align256(sizeof(int32_t) * size_t(nt + 1));
  const size_t o_scr = off;
  const size_t scr_bytes = std::max(radix_sort_scratch_bytes(M), scan_scratch_bytes(nt + 1));
  off += align256(scr_bytes);
  if (off > kScratchBytes) {
    set_error("binning scratch of %zu bytes exceeds the static %zu bytes", off, kScratchBytes);
    return NFFT_ERR_UNSUPPORTED;
  }
  void* base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc) return rc;
  char* s = static_cast<char*>(base);
  int* flag = reinterpret_cast<int*>(s + o_flag);
  int32_t* ti = reinterpret_cast<int32_t*>(s + o_ti);
  void* te = s + o_te;
  uint32_t* k1 = reinterpret_cast<uint32_t*>(s + o_k1);
  int32_t* v1 = reinterpret_cast<int32_t*>(s + o_v1);
  uint32_t* k2 = reinterpret_cast<uint32_t*>(s + o_k2);
  int32_t* v2 = reinterpret_cast<int32_t*>(s + o_v2);
  int32_t* tcount = reinterpret_cast<int32_t*>(s + o_tc);
  void* scr = s + o_scr;

  // The scratch keeps the previous call's contents: clear what must start at zero.
  NFFT_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), g.stream));
  NFFT_CUDA_TRY(cudaMemsetAsync(tcount, 0, sizeof(int32_t) * size_t(nt + 1), g.stream));
  rc = launch_check_nodes(&g, k, flag);
  if (rc) return rc;
  int hflag = 0;
  NFFT_CUDA_TRY(cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, g.stream));
  NFFT_CUDA_TRY(cudaStreamSynchronize(g.stream));
  if (hflag) {
    set_error("Nodes k need to be within the range [-1/2, 1/2)");
    return NFFT_ERR_NODE_OUT_OF_RANGE;
  }
  rc = launch_reduce_nodes(&g, k, ti, te, k1, v1, tcount);
  if (rc) return rc;
  int bits = 0;
  while ((int64_t(1) << bits) < nt) ++bits;
  uint32_t* ko = nullptr;
  int32_t* vo = nullptr;
  rc = radix_sort_pairs(k1, v1, k2, v2, M, bits, scr, scr_bytes, g.stream, &ko, &vo);
  if (rc) return rc;
  if (M > 0) NFFT_CUDA_TRY(cudaMemcpyAsync(perm, vo, sizeof(int32_t) * size_t(M), cudaMemcpyDeviceToDevice, g.stream));
  rc = exclusive_scan_i32(tcount, tile_start, nt + 1, scr, scr_bytes, g.stream);
  if (rc) return rc;
  return NFFT_OK;
}
