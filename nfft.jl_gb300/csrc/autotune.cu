// Tile-shape autotuner.  The spreading tile (blockSize) trades shared-memory
// footprint (occupancy) against flush overhead (padded halo / core volume)
// and load balance, and the best shape depends on D, Ntilde, the node count
// and distribution, m and the precision.  nfft_autotune re-bins the plan's
// nodes for each candidate shape, times one gather + one spreading pass with
// CUDA events on the plan's stream (median of three), keeps the fastest and
// records it in a small text cache (file named by NFFT_GB300_TUNE_CACHE, if
// set), keyed by (D, Ntilde, log2 M, m, precision, SM count, mode).
#include "nfft_internal.cuh"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace nfft {
namespace {

std::mutex g_cache_mutex;
std::map<std::string, std::vector<int64_t>> g_cache;
bool g_cache_loaded = false;
std::string g_cache_path;  // the NFFT_GB300_TUNE_CACHE value the cache was read from

std::string cache_key(const nfft_plan* p) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int lm = 0;
  while ((int64_t(1) << (lm + 1)) <= p->M) ++lm;
  char buf[256];
  snprintf(buf, sizeof(buf), "v2_D%d_N%lldx%lldx%lld_M2^%d_m%d_p%d_sm%d_pre%d_c%d", p->D, (long long)p->Nt[0],
           (long long)p->Nt[1], (long long)p->Nt[2], lm, p->m, p->precision, sms, p->prm.precompute,
           p->prm.compensated);
  return buf;
}

// Cache file: one line per entry, "key bs0 bs1 bs2 ny".  Read once per value
// of NFFT_GB300_TUNE_CACHE: pointing the variable at another file (re)loads
// from that file.
void load_cache() {
  const char* path = getenv("NFFT_GB300_TUNE_CACHE");
  const std::string cur = path ? path : "";
  if (g_cache_loaded && cur == g_cache_path) return;
  g_cache_loaded = true;
  g_cache_path = cur;
  g_cache.clear();
  if (!path) return;
  FILE* f = fopen(path, "r");
  if (!f) return;
  char line[512];
  while (fgets(line, sizeof(line), f)) {
    char key[256];
    long long a, b, c, ny;
    if (sscanf(line, "%255s %lld %lld %lld %lld", key, &a, &b, &c, &ny) == 5 && (ny == 1 || ny == 2))
      g_cache[key] = {a, b, c, ny};
  }
  fclose(f);
}

void save_cache() {
  const char* path = getenv("NFFT_GB300_TUNE_CACHE");
  if (!path) return;
  std::string tmp = std::string(path) + ".tmp";
  FILE* f = fopen(tmp.c_str(), "w");
  if (!f) return;
  for (auto& kv : g_cache)
    fprintf(f, "%s %lld %lld %lld %lld\n", kv.first.c_str(), (long long)kv.second[0], (long long)kv.second[1],
            (long long)kv.second[2], (long long)kv.second[3]);
  fclose(f);
  rename(tmp.c_str(), path);
}

// Candidate (tile shape, ny): ny = 2 runs 16-warp 3-D tiles owning
// (slice group, row parity) -- it pays where the tiles are large.
std::vector<std::vector<int64_t>> candidates(const nfft_plan* p) {
  std::vector<std::vector<int64_t>> c;
  if (p->D == 1) {
    for (int64_t b : {256, 512, 1024, 2048, 4096}) c.push_back({b, 1, 1, 1});
  } else if (p->D == 2) {
    // small tiles give small grids enough tasks to fill the GPU
    for (auto s : std::vector<std::vector<int64_t>>{{8, 8, 1}, {16, 8, 1}, {16, 16, 1}, {32, 16, 1}, {32, 32, 1},
                                                     {64, 32, 1}, {64, 64, 1}, {128, 64, 1}, {128, 128, 1}})
      c.push_back({s[0], s[1], s[2], 1});
  } else {
    for (auto s : std::vector<std::vector<int64_t>>{{8, 8, 8}, {16, 16, 8}, {16, 16, 16}, {32, 16, 8}, {32, 32, 8},
                                                     {16, 8, 8}}) {
      c.push_back({s[0], s[1], s[2], 1});
      if (!p->prm.compensated && s[1] >= 16) c.push_back({s[0], s[1], s[2], 2});
    }
  }
  for (auto& s : c)
    for (int d = 0; d < 3; ++d) s[d] = std::min<int64_t>(s[d], p->Nt[d]);
  std::sort(c.begin(), c.end());
  c.erase(std::unique(c.begin(), c.end()), c.end());
  return c;
}

}  // namespace

// Apply a tile shape (and 3-D warp layout ny) to the plan and re-bin its
// nodes (from `k`, device).
int apply_block_size(nfft_plan* p, const int64_t* bs, const void* k, int ny) {
  int64_t nt = 1;
  int64_t nb[3], tiles[3];
  for (int d = 0; d < 3; ++d) {
    nb[d] = d < p->D ? std::max<int64_t>(1, std::min<int64_t>(bs[d], p->Nt[d])) : 1;
    tiles[d] = (p->Nt[d] + nb[d] - 1) / nb[d];
    nt *= tiles[d];
  }
  if (nt >= (int64_t(1) << 31)) {
    set_error("too many tiles");
    return NFFT_ERR_UNSUPPORTED;
  }
  const int layout = (p->D == 3 && !p->prm.compensated && ny == 2) ? 2 : 1;
  for (int d = 0; d < 3; ++d) {
    p->bs[d] = nb[d];
    p->ntiles[d] = tiles[d];
    p->prm.block_size[d] = d < p->D ? nb[d] : 0;
  }
  p->ntiles_total = nt;
  p->spread_layout = layout;
  int rc = update_center(p);  // the grid shift is a whole number of tiles
  if (rc) return rc;
  p->spread_pitch = spread_pitch_for(p->D, p->m, int(p->bs[0]) + 2 * p->m - 1,
                                     int((p->prm.compensated ? 4 : 2) * p->real_size), p->spread_layout == 2 ? 2 : 1);
  p->gather_pitch = spread_pitch_for(p->D == 2 ? 3 : p->D, p->m, int(p->bs[0]) + 2 * p->m - 1,
                                     int(2 * p->real_size), 1);
  return nfft_set_nodes(p, k, 1);
}

}  // namespace nfft

using namespace nfft;

extern "C" int nfft_autotune(nfft_plan* p, int use_cache) {
  if (!p || !p->has_nodes) {
    set_error("nfft_autotune needs a plan with nodes");
    return p ? NFFT_ERR_NO_NODES : NFFT_ERR_INVALID_ARG;
  }
  if (!p->prm.blocking) return NFFT_OK;  // the plain path has no tiles
  const std::string key = cache_key(p);
  const size_t kbytes = p->real_size * size_t(p->D * p->M);
  void* k = nullptr;
  if (p->M > 0 && cudaMalloc(&k, kbytes) != cudaSuccess) {
    set_error("cudaMalloc of the autotuner's node copy failed");
    return NFFT_ERR_ALLOC;
  }
  struct Free {
    void* q;
    ~Free() { cudaFree(q); }
  } free_k{k};
  if (p->M > 0) NFFT_CUDA_TRY(cudaMemcpyAsync(k, p->k, kbytes, cudaMemcpyDeviceToDevice, p->stream));
  NFFT_CUDA_TRY(cudaStreamSynchronize(p->stream));
  if (use_cache) {
    std::lock_guard<std::mutex> lock(g_cache_mutex);
    load_cache();
    auto it = g_cache.find(key);
    if (it != g_cache.end()) return apply_block_size(p, it->second.data(), k, int(it->second[3]));
  }
  // timing buffers: node values (ones) and the plan's grid
  void* fhat = nullptr;
  if (cudaMalloc(&fhat, 2 * p->real_size * size_t(std::max<int64_t>(p->M, 1))) != cudaSuccess) {
    set_error("cudaMalloc of the autotuner's node values failed");
    return NFFT_ERR_ALLOC;
  }
  Free free_f{fhat};
  NFFT_CUDA_TRY(cudaMemsetAsync(fhat, 0, 2 * p->real_size * size_t(std::max<int64_t>(p->M, 1)), p->stream));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 1e30;
  std::vector<int64_t> best_bs = {p->bs[0], p->bs[1], p->bs[2], p->spread_layout};
  for (const auto& c : candidates(p)) {
    if (apply_block_size(p, c.data(), k, int(c[3])) != NFFT_OK) continue;
    CenterScope centred(p);  // time the grid layout the transforms use
    float times[3];
    bool ok = true;
    for (int r = 0; r < 3 && ok; ++r) {
      cudaEventRecord(e0, p->stream);
      ok = launch_spread(p, fhat, 0, p->grid, 0) == NFFT_OK && launch_interp(p, p->grid, 0, fhat, 0) == NFFT_OK;
      cudaEventRecord(e1, p->stream);
      cudaEventSynchronize(e1);
      cudaEventElapsedTime(&times[r], e0, e1);
    }
    if (!ok) continue;  // e.g. the tile does not fit in shared memory
    std::sort(times, times + 3);
    if (times[1] < best) {
      best = times[1];
      best_bs = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaGetLastError();  // clear a rejected candidate's error state
  int rc = apply_block_size(p, best_bs.data(), k, int(best_bs[3]));
  if (!rc) {
    std::lock_guard<std::mutex> lock(g_cache_mutex);
    load_cache();
    g_cache[key] = best_bs;
    save_cache();
  }
  return rc;
}

extern "C" int nfft_set_tiling(nfft_plan* p, const int64_t* block_size, int row_parity_warps);

extern "C" int nfft_set_block_size(nfft_plan* p, const int64_t* block_size) {
  return nfft_set_tiling(p, block_size, p ? p->spread_layout : 1);
}

extern "C" int nfft_set_tiling(nfft_plan* p, const int64_t* block_size, int row_parity_warps) {
  if (!p || !block_size) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  for (int d = 0; d < p->D; ++d)
    if (block_size[d] < 1) {
      set_error("block size must be positive");
      return NFFT_ERR_INVALID_ARG;
    }
  if (row_parity_warps < 1 || row_parity_warps > 2) {
    set_error("row_parity_warps must be 1 or 2");
    return NFFT_ERR_INVALID_ARG;
  }
  if (!p->has_nodes) {
    for (int d = 0; d < 3; ++d) p->prm.block_size[d] = d < p->D ? block_size[d] : 0;
    set_error("plan has no nodes: the block size applies at the next nfft_set_nodes");
    return NFFT_ERR_NO_NODES;
  }
  const size_t kbytes = p->real_size * size_t(p->D * p->M);
  void* k = nullptr;
  if (p->M > 0 && cudaMalloc(&k, kbytes) != cudaSuccess) {
    set_error("cudaMalloc of the node copy failed");
    return NFFT_ERR_ALLOC;
  }
  int rc = NFFT_OK;
  if (p->M > 0 && cudaMemcpyAsync(k, p->k, kbytes, cudaMemcpyDeviceToDevice, p->stream) != cudaSuccess) {
    set_error("node copy failed");
    rc = NFFT_ERR_CUDA;
  }
  if (!rc) rc = apply_block_size(p, block_size, k, row_parity_warps);
  cudaFree(k);
  return rc;
}
