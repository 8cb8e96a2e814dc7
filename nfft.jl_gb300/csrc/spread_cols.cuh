// Column-owned register spreading for 3-D FP32 plans (spreading layout 3).
//
// The CTA spreads the nodes of one task (home tile or chunk of a hot tile)
// into the tile padded by 2m-1 points, as the slice-owned kernel does, but the
// padded tile lives in registers instead of shared memory:
//   * lane (x, y) of the CTA owns one column of the padded tile and holds its
//     PZ = BZ + 2m - 1 points along z as float2 registers.  Warp w owns an
//     8 (x) x 4 (y) block of columns;
//   * nodes are staged in shared memory in batches of 64 (footprint origin,
//     the x and y window values, and the complex value times each z window
//     value), then every warp selects with a ballot the nodes whose footprint
//     touches its block and visits only those;
//   * per node a lane forms its column weight w = phi_x * phi_y (zero outside
//     the footprint) and adds w * (c phi_z[i]) to its registers z0 + i, where
//     the footprint's z origin z0 is the same for the whole warp: a switch on
//     z0 turns the dynamic register index into BZ unrolled static ones.
// A tap then costs two FFMAs and no shared-memory traffic; the accumulation
// never leaves the registers until the flush, which adds each column to the
// grid with 16-byte vector atomics over point pairs (grid-aligned: the
// columns start at an even grid x) and skips zeros, as the other spreading
// kernels do.  Nodes are visited in bin-sorted order, so the floating-point
// sums are those of the slice-owned kernel up to the order of additions.
#pragma once

#include "spread_body.cuh"

namespace nfft {
namespace {

constexpr int kColBatch = 64;        // nodes per staged batch
constexpr int kColMaxThreads = 768;  // up to 24 warps of 8 x 4 columns

template <int L> struct ColCfg {
  static_assert(L % 2 == 0, "2m taps per dimension");
  static constexpr int LH = L / 2;
};

// acc[P + i] += w * cz[i], i < L (cz as pairs of complex values).
template <int P, int L, int PZ>
__device__ __forceinline__ void col_add(float2 (&acc)[PZ], float w, const float4 (&cz)[L / 2]) {
#pragma unroll
  for (int i = 0; i < L / 2; ++i) {
    acc[P + 2 * i].x = fmaf(w, cz[i].x, acc[P + 2 * i].x);
    acc[P + 2 * i].y = fmaf(w, cz[i].y, acc[P + 2 * i].y);
    acc[P + 2 * i + 1].x = fmaf(w, cz[i].z, acc[P + 2 * i + 1].x);
    acc[P + 2 * i + 1].y = fmaf(w, cz[i].w, acc[P + 2 * i + 1].y);
  }
}

#define NFFT_COL_CASE(P)                                       \
  case P:                                                      \
    if constexpr (P < BZ) col_add<P, L, BZ + L - 1>(acc, w, cz); \
    break;

template <int L, int BZ>
__device__ __forceinline__ void col_add_at(int pz, float2 (&acc)[BZ + L - 1], float w, const float4 (&cz)[L / 2]) {
  static_assert(BZ <= 16, "at most 16 z offsets");
  switch (pz) {
    NFFT_COL_CASE(0) NFFT_COL_CASE(1) NFFT_COL_CASE(2) NFFT_COL_CASE(3) NFFT_COL_CASE(4) NFFT_COL_CASE(5)
    NFFT_COL_CASE(6) NFFT_COL_CASE(7) NFFT_COL_CASE(8) NFFT_COL_CASE(9) NFFT_COL_CASE(10) NFFT_COL_CASE(11)
    NFFT_COL_CASE(12) NFFT_COL_CASE(13) NFFT_COL_CASE(14) NFFT_COL_CASE(15)
    default:
      break;
  }
}
#undef NFFT_COL_CASE

// Column blocks of a tile: nxb x nyb warps (x blocks of 8 columns starting
// at the even grid x below the padded tile, y blocks of 4 rows).
__host__ __device__ inline int col_xblocks(int bx, int L) { return (bx + L + 7) / 8; }
__host__ __device__ inline int col_yblocks(int by, int L) { return (by + L - 1 + 3) / 4; }

template <int L, int BZ, bool TABLE>
__global__ void __launch_bounds__(kColMaxThreads) spread_cols_kernel(Geom<float> G, Nodes<float> Nd,
                                                                      const int4* __restrict__ tasks,
                                                                      const float2* __restrict__ fsorted,
                                                                      float* __restrict__ g, int nxb, int pair,
                                                                      int64_t fcol = 0, int64_t gcol = 0) {
  constexpr int PZ = BZ + L - 1;
  constexpr int NB = kColBatch;
  constexpr int LH = L / 2;
  constexpr int DEG = L + 1;
  __shared__ int4 s_meta[NB];              // footprint origin (column x, row y, z) in the padded tile
  __shared__ float s_wx[NB][L], s_wy[NB][L];
  __shared__ float4 s_cz[NB][LH];          // value times z window values, two taps per float4
  fsorted += blockIdx.y * fcol;            // column of a multi-column launch
  g += blockIdx.y * gcol;
  const int4 task = tasks[blockIdx.x];
  const int tile = task.x;
  const int tc0 = tile % G.ntiles[0];
  const int tc1 = (tile / G.ntiles[0]) % G.ntiles[1];
  const int tc2 = tile / (G.ntiles[0] * G.ntiles[1]);
  const int m1 = G.m - 1;
  const int o0 = tc0 * G.bs[0], o1 = tc1 * G.bs[1], o2 = tc2 * G.bs[2];
  const int x0 = (o0 - m1) & ~1;  // even grid x of column 0 (pairs never straddle the wrap)
  const int y0 = o1 - m1, z0 = o2 - m1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int bx0 = (warp % nxb) * 8, by0 = (warp / nxb) * 4;
  const int cx = bx0 + (lane & 7), cy = by0 + (lane >> 3);
  float2 acc[PZ];
#pragma unroll
  for (int i = 0; i < PZ; ++i) acc[i] = make_float2(0.f, 0.f);

  for (int b = task.y; b < task.z; b += NB) {
    const int n = min(NB, task.z - b);
    __syncthreads();  // the previous batch has been consumed
    // ---- stage the batch: footprint origins, x/y window values, c * phi_z
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
      const int4 nd = __ldg(Nd.node4 + b + q);
      s_meta[q] = make_int4(nd.x - m1 - x0, nd.y - o1, nd.z - o2, 0);
    }
    for (int q = threadIdx.x; q < n * 2 * L; q += blockDim.x) {
      const int s = q / (2 * L), r = q - s * (2 * L);
      float w;
      if constexpr (TABLE) {
        w = __ldg(Nd.wtab + int64_t(b + s) * (3 * L) + r);
      } else {
        const int d = r / L, l = r - d * L;
        const float t = __ldg(Nd.frac4 + 4 * int64_t(b + s) + d) - 0.5f;
        const float* c = G.coeffs + l * DEG;
        w = __ldg(c + DEG - 1);
#pragma unroll
        for (int i = DEG - 2; i >= 0; --i) w = fmaf(w, t, __ldg(c + i));
      }
      if (r < L) s_wx[s][r] = w;
      else s_wy[s][r - L] = w;
    }
    for (int q = threadIdx.x; q < n * LH; q += blockDim.x) {
      const int s = q / LH, i = q - s * LH;
      const float2 c = __ldg(fsorted + b + s);
      float wa, wb;
      if constexpr (TABLE) {
        const float* wz = Nd.wtab + int64_t(b + s) * (3 * L) + 2 * L + 2 * i;
        wa = __ldg(wz);
        wb = __ldg(wz + 1);
      } else {
        const float t = __ldg(Nd.frac4 + 4 * int64_t(b + s) + 2) - 0.5f;
        const float* ca = G.coeffs + (2 * i) * DEG;
        const float* cb = ca + DEG;
        wa = __ldg(ca + DEG - 1);
        wb = __ldg(cb + DEG - 1);
#pragma unroll
        for (int k = DEG - 2; k >= 0; --k) {
          wa = fmaf(wa, t, __ldg(ca + k));
          wb = fmaf(wb, t, __ldg(cb + k));
        }
      }
      s_cz[s][i] = make_float4(c.x * wa, c.y * wa, c.x * wb, c.y * wb);
    }
    __syncthreads();
    // ---- the nodes whose footprint touches this warp's 8 x 4 column block
    unsigned mask[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int s = lane + 32 * h;
      bool hit = false;
      if (s < n) {
        const int4 mt = s_meta[s];
        hit = mt.x < bx0 + 8 && mt.x + L > bx0 && mt.y < by0 + 4 && mt.y + L > by0;
      }
      mask[h] = __ballot_sync(0xFFFFFFFFu, hit);
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      unsigned mk = mask[h];
      while (mk) {
        const int s = 32 * h + __ffs(mk) - 1;
        mk &= mk - 1;
        const int4 mt = s_meta[s];
        const int dx = cx - mt.x, dy = cy - mt.y;
        float w = 0.f;
        if (unsigned(dx) < unsigned(L) && unsigned(dy) < unsigned(L)) w = s_wx[s][dx] * s_wy[s][dy];
        float4 cz[LH];
#pragma unroll
        for (int i = 0; i < LH; ++i) cz[i] = s_cz[s][i];
        col_add_at<L, BZ>(mt.z, acc, w, cz);
      }
    }
  }

  // ---- flush: columns into the grid (periodic wrap), pairs of points along x
  const bool small = G.small_grid;
  const int Nt0 = G.Nt[0];
  const int gx = small ? wrap_any(x0 + cx, Nt0) : wrap_once(x0 + cx, Nt0);
  const int gy = small ? wrap_any(y0 + cy, G.Nt[1]) : wrap_once(y0 + cy, G.Nt[1]);
  int gz = small ? wrap_any(z0, G.Nt[2]) : wrap_once(z0, G.Nt[2]);
  float* col = g + 2 * (int64_t(gy) * Nt0 + gx);
  const bool even = (lane & 1) == 0;
#pragma unroll
  for (int i = 0; i < PZ; ++i) {
    const float2 v = acc[i];
    float* p = col + 2 * int64_t(gz) * G.plane;
    if (pair) {
      const float ox = __shfl_down_sync(0xFFFFFFFFu, v.x, 1);
      const float oy = __shfl_down_sync(0xFFFFFFFFu, v.y, 1);
      if (even && (v.x != 0.f || v.y != 0.f || ox != 0.f || oy != 0.f))
        atomicAdd(reinterpret_cast<float4*>(p), make_float4(v.x, v.y, ox, oy));
    } else if (v.x != 0.f || v.y != 0.f) {
      atomicAdd(reinterpret_cast<float2*>(p), v);
    }
    if (++gz == G.Nt[2]) gz = 0;
  }
}

}  // namespace
}  // namespace nfft
