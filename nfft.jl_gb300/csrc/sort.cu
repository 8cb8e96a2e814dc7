// Stable LSD radix sort of (uint32 key, int32 value) pairs and an exclusive
// int32 scan, written for the node binning of nfft_set_nodes.
//
// Stability is what makes the sort permutation bit-exact with NFFT.jl's
// two-pass "count + push" binning (src/precomputation.jl:494-504), where the
// nodes of one block keep their input order.
//
// One pass per 8-bit digit:
//   upsweep   : each CTA counts the digits of its tile of 4096 keys;
//   scan      : exclusive scan of the digit-major (digit, CTA) count table;
//   downsweep : each CTA ranks its keys stably (warp match + per-warp counts,
//               in input order) and scatters them.
#include "nfft_internal.cuh"

namespace nfft {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;  // keys per CTA
constexpr int kRadix = 256;
constexpr int kWarps = kSortThreads / 32;

__global__ void __launch_bounds__(kSortThreads) radix_upsweep(const uint32_t* __restrict__ keys, int64_t n,
                                                               int shift, int nblocks,
                                                               int32_t* __restrict__ hist) {
  __shared__ int32_t cnt[kRadix];
  for (int i = threadIdx.x; i < kRadix; i += blockDim.x) cnt[i] = 0;
  __syncthreads();
  const int64_t base = int64_t(blockIdx.x) * kSortTile;
  for (int it = 0; it < kSortItems; ++it) {
    int64_t i = base + int64_t(it) * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 0xFF], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) hist[int64_t(d) * nblocks + blockIdx.x] = cnt[d];
}

__global__ void __launch_bounds__(kSortThreads) radix_downsweep(const uint32_t* __restrict__ keys_in,
                                                                 const int32_t* __restrict__ vals_in, int64_t n,
                                                                 int shift, int nblocks,
                                                                 const int32_t* __restrict__ offs,
                                                                 uint32_t* __restrict__ keys_out,
                                                                 int32_t* __restrict__ vals_out) {
  __shared__ int32_t running[kRadix];
  __shared__ int32_t wcnt[kWarps][kRadix];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int d = tid; d < kRadix; d += blockDim.x) running[d] = offs[int64_t(d) * nblocks + blockIdx.x];
  const int64_t base = int64_t(blockIdx.x) * kSortTile;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int it = 0; it < kSortItems; ++it) {
    for (int q = tid; q < kWarps * kRadix; q += blockDim.x) (&wcnt[0][0])[q] = 0;
    __syncthreads();
    const int64_t i = base + int64_t(it) * kSortThreads + tid;
    const bool valid = i < n;
    uint32_t key = valid ? keys_in[i] : 0u;
    int digit = valid ? int((key >> shift) & 0xFF) : -1;
    // lanes with the same digit, in lane (= input) order
    unsigned peers = __match_any_sync(0xFFFFFFFFu, digit);
    int rank = __popc(peers & lt_mask);
    if (valid && rank == 0) wcnt[warp][digit] = __popc(peers);
    __syncthreads();
    int pos = 0;
    if (valid) {
      pos = running[digit] + rank;
      for (int w = 0; w < warp; ++w) pos += wcnt[w][digit];
    }
    __syncthreads();
    for (int d = tid; d < kRadix; d += blockDim.x) {
      int s = 0;
      for (int w = 0; w < kWarps; ++w) s += wcnt[w][d];
      running[d] += s;
    }
    if (valid) {
      keys_out[pos] = key;
      vals_out[pos] = vals_in[i];
    }
    __syncthreads();
  }
}

// Block-level exclusive scan of up to 2048 int32 per CTA (4 per thread).
constexpr int kScanThreads = 512;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) scan_tiles(const int32_t* __restrict__ in, int32_t* __restrict__ out,
                                                            int64_t n, int32_t* __restrict__ tile_sums) {
  __shared__ int32_t warp_sums[kScanThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t base = int64_t(blockIdx.x) * kScanTile + int64_t(tid) * kScanItems;
  int32_t v[kScanItems];
  int32_t local = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; ++q) {
    v[q] = (base + q < n) ? in[base + q] : 0;
    local += v[q];
  }
  // inclusive warp scan of thread totals
  int32_t x = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int32_t w = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kScanThreads / 32) warp_sums[lane] = w;
  }
  __syncthreads();
  int32_t prefix = x - local + (warp > 0 ? warp_sums[warp - 1] : 0);
#pragma unroll
  for (int q = 0; q < kScanItems; ++q) {
    if (base + q < n) out[base + q] = prefix;
    prefix += v[q];
  }
  if (tid == kScanThreads - 1 && tile_sums) tile_sums[blockIdx.x] = prefix;
}

__global__ void add_tile_offsets(int32_t* __restrict__ out, int64_t n, const int32_t* __restrict__ offs) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) out[i] += offs[i / kScanTile];
}

int scan_rec(const int32_t* in, int32_t* out, int64_t n, char* scratch, size_t bytes, cudaStream_t s) {
  if (n <= 0) return NFFT_OK;
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 1) {
    scan_tiles<<<1, kScanThreads, 0, s>>>(in, out, n, nullptr);
    NFFT_LAUNCH_CHECK();
    return NFFT_OK;
  }
  const size_t need = size_t(2 * tiles) * sizeof(int32_t);
  if (need > bytes) {
    set_error("scan scratch too small");
    return NFFT_ERR_ALLOC;
  }
  int32_t* sums = reinterpret_cast<int32_t*>(scratch);
  int32_t* sums_scan = sums + tiles;
  scan_tiles<<<unsigned(tiles), kScanThreads, 0, s>>>(in, out, n, sums);
  NFFT_LAUNCH_CHECK();
  int rc = scan_rec(sums, sums_scan, tiles, scratch + need, bytes - need, s);
  if (rc) return rc;
  add_tile_offsets<<<unsigned((n + 255) / 256), 256, 0, s>>>(out, n, sums_scan);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

}  // namespace

size_t scan_scratch_bytes(int64_t n) {
  size_t total = 0;
  int64_t t = n;
  while (t > kScanTile) {
    t = (t + kScanTile - 1) / kScanTile;
    total += size_t(2 * t) * sizeof(int32_t);
  }
  return total + 256;
}

int exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, void* scratch, size_t scratch_bytes,
                       cudaStream_t s) {
  return scan_rec(in, out, n, static_cast<char*>(scratch), scratch_bytes, s);
}

size_t radix_sort_scratch_bytes(int64_t n) {
  const int64_t nb = (n + kSortTile - 1) / kSortTile;
  const int64_t h = int64_t(kRadix) * (nb > 0 ? nb : 1);
  return size_t(2 * h) * sizeof(int32_t) + scan_scratch_bytes(h) + 256;
}

int radix_sort_pairs(uint32_t* keys, int32_t* vals, uint32_t* keys_tmp, int32_t* vals_tmp, int64_t n,
                     int key_bits, void* scratch, size_t scratch_bytes, cudaStream_t s, uint32_t** keys_out,
                     int32_t** vals_out) {
  *keys_out = keys;
  *vals_out = vals;
  if (n <= 1 || key_bits <= 0) return NFFT_OK;
  const int nb = int((n + kSortTile - 1) / kSortTile);
  const int64_t h = int64_t(kRadix) * nb;
  if (radix_sort_scratch_bytes(n) > scratch_bytes) {
    set_error("radix sort scratch too small");
    return NFFT_ERR_ALLOC;
  }
  int32_t* hist = static_cast<int32_t*>(scratch);
  int32_t* offs = hist + h;
  char* scan_scr = reinterpret_cast<char*>(offs + h);
  const size_t scan_bytes = scratch_bytes - size_t(2 * h) * sizeof(int32_t);
  uint32_t* kin = keys;
  int32_t* vin = vals;
  uint32_t* kout = keys_tmp;
  int32_t* vout = vals_tmp;
  for (int shift = 0; shift < key_bits; shift += 8) {
    radix_upsweep<<<nb, kSortThreads, 0, s>>>(kin, n, shift, nb, hist);
    NFFT_LAUNCH_CHECK();
    int rc = exclusive_scan_i32(hist, offs, h, scan_scr, scan_bytes, s);
    if (rc) return rc;
    radix_downsweep<<<nb, kSortThreads, 0, s>>>(kin, vin, n, shift, nb, offs, kout, vout);
    NFFT_LAUNCH_CHECK();
    uint32_t* tk = kin; kin = kout; kout = tk;
    int32_t* tv = vin; vin = vout; vout = tv;
  }
  *keys_out = kin;
  *vals_out = vin;
  return NFFT_OK;
}

}  // namespace nfft
