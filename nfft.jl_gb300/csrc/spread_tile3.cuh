// Shape-specialised slice-owned spreading for 3-D FP32 plans with m = 4
// (2m = 8 taps per dimension) and tile shapes fixed at compile time.
//
// The algorithm is the slice-owned kernel of spread_body.cuh (warp w owns the
// z slices w mod 8 of the tile padded by 2m - 1 points, atomic-free
// read-modify-writes in shared memory), specialised so that the tap loop is
// almost only its memory operations and FFMAs:
//   * the padded tile's row pitch is a constant, so a lane's two taps of a
//     node (rows iy and iy + 4) are one base address plus immediate offsets,
//     and every lane is active in both steps (8 x 4 lanes, 8 rows);
//   * with 8 owner warps and 8 taps along z every warp owns exactly one slice
//     of every node: no ownership or activity tests;
//   * staging computes the 64 x-y weight products of a node one window row
//     per thread;
//   * the padded tile starts at the even grid x o0 - m (one leading column
//     that stays zero), so it is laid out as a TMA box: a tile that does not
//     wrap around the grid is added to it by one bulk tensor reduction
//     (cp.reduce.async.bulk.tensor ... .add) issued by one thread, instead of
//     ~2700 vector atomics spread over the CTA; tiles that wrap (and grids
//     without a tensor map) use the per-point flush of spread_body.cuh.
#pragma once

#include "spread_body.cuh"
#include "tile3.cuh"

namespace nfft {
namespace {

template <int BX, int BY, int BZ, bool TABLE>
__global__ void __launch_bounds__(256) spread_tile3_kernel(const __grid_constant__ CUtensorMap tmap, int use_tma,
                                                            Geom<float> G, Nodes<float> Nd,
                                                            const int4* __restrict__ tasks,
                                                            const float2* __restrict__ fsorted,
                                                            float* __restrict__ g, int64_t fcol, int64_t gcol) {
  using TC = Tile3<BX, BY, BZ>;
  constexpr int L = TC::L, NB = TC::NB, DL = 3 * L, DEG = L + 1;
  constexpr int PITCH = TC::PITCH, PLANE = TC::PLANE;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  fsorted += blockIdx.y * fcol;  // column of a multi-column launch
  g += blockIdx.y * gcol;
  float2* acc = reinterpret_cast<float2*>(smem_raw);
  int4* s_meta = reinterpret_cast<int4*>(smem_raw + TC::ACC_BYTES);  // [NB] {tap offset, z plane}
  float2* s_c = reinterpret_cast<float2*>(s_meta + NB);                // [NB]
  float2* s_cz = s_c + NB;                                             // [NB][L]: value x z window value
  float* s_w = reinterpret_cast<float*>(s_cz + NB * L);                // [NB][3L]
  float* s_xy = s_w + NB * DL;                                         // [NB][L * L]
  const int4 task = tasks[blockIdx.x];
  const int tile = task.x;
  const int tc0 = tile % G.ntiles[0];
  const int tc1 = (tile / G.ntiles[0]) % G.ntiles[1];
  const int tc2 = tile / (G.ntiles[0] * G.ntiles[1]);
  const int o0 = tc0 * BX, o1 = tc1 * BY, o2 = tc2 * BZ;
  {
    float4* a4 = reinterpret_cast<float4*>(acc);
    for (int q = threadIdx.x; q < TC::NACC / 2; q += TC::THREADS) a4[q] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int lofs = (lane >> 3) * PITCH + (lane & 7);  // this lane's tap (x = lane mod 8, row = lane / 8)

  // register prefetch of one batch: node, value, window values (or fractional offsets)
  constexpr int WPT = NB * DL / TC::THREADS;  // 3
  int4 r_nd = make_int4(0, 0, 0, 0);
  float2 r_c = make_float2(0.f, 0.f);
  float r_w[WPT];
  auto prefetch = [&](int b) {
    const int n = min(NB, task.z - b);
    if (threadIdx.x < n) {
      r_nd = __ldg(Nd.node4 + b + threadIdx.x);
      r_c = __ldg(fsorted + b + threadIdx.x);
    }
#pragma unroll
    for (int u = 0; u < WPT; ++u) {
      const int q = threadIdx.x + u * TC::THREADS;
      if (q < n * DL) {
        if constexpr (TABLE) r_w[u] = __ldg(Nd.wtab + int64_t(b) * DL + q);
        else r_w[u] = __ldg(Nd.frac4 + 4 * int64_t(b + q / DL) + (q % DL) / L);
      }
    }
  };
  if (task.y < task.z) prefetch(task.y);
  __syncthreads();

  for (int b = task.y; b < task.z; b += NB) {
    const int n = min(NB, task.z - b);
    // stage 1: registers -> shared (window values evaluated here for POLYNOMIAL)
    if (threadIdx.x < n) {
      // {offset of the window's first tap in the padded tile, its z plane}
      const int z0 = r_nd.z - o2;
      s_meta[threadIdx.x] = make_int4(z0 * PLANE + (r_nd.y - o1) * PITCH + (r_nd.x - o0 + 1), z0, 0, 0);
      s_c[threadIdx.x] = r_c;
    }
#pragma unroll
    for (int u = 0; u < WPT; ++u) {
      const int q = threadIdx.x + u * TC::THREADS;
      if (q < n * DL) {
        float w = r_w[u];
        if constexpr (!TABLE) {
          const int l = (q % DL) % L;
          const float t = w - 0.5f;
          const float* c = G.coeffs + l * DEG;
          w = __ldg(c + DEG - 1);
#pragma unroll
          for (int i = DEG - 2; i >= 0; --i) w = fmaf(w, t, __ldg(c + i));
        }
        s_w[q] = w;
      }
    }
    __syncthreads();
    // stage 2: thread (node s, row iy): the row of x-y products, and for
    // warp iy the value times the z window value of the slice it owns,
    // c * wz[(iy - z0) mod 8]
    {
      const int s = threadIdx.x >> 3, iy = threadIdx.x & 7;
      if (s < n) {
        const float* ws = s_w + s * DL;
        const float wyv = ws[L + iy];
        const float4 x0 = *reinterpret_cast<const float4*>(ws);
        const float4 x1 = *reinterpret_cast<const float4*>(ws + 4);
        float4* out = reinterpret_cast<float4*>(s_xy + s * L * L + iy * L);
        out[0] = make_float4(x0.x * wyv, x0.y * wyv, x0.z * wyv, x0.w * wyv);
        out[1] = make_float4(x1.x * wyv, x1.y * wyv, x1.z * wyv, x1.w * wyv);
        const float wz = ws[2 * L + ((iy - s_meta[s].y) & 7)];
        const float2 c = s_c[s];
        s_cz[s * L + iy] = make_float2(c.x * wz, c.y * wz);
      }
    }
    __syncthreads();
    if (b + NB < task.z) prefetch(b + NB);
    // taps: warp w updates its slice of every node, rows iy and iy + 4 of the
    // lane's column; the next node's record is loaded during this node's taps
    int4 mt = s_meta[0];
    float2* const accl = acc + lofs;
    for (int s = 0; s < n; ++s) {
      const int4 mn = s_meta[s + 1];  // (past the last node: a value in s_c, unused)
      float2* p = accl + mt.x + ((warp - mt.y) & 7) * PLANE;
      const float* xy = s_xy + s * L * L + lane;
      const float2 cz = s_cz[s * L + warp];
      float2 a0 = p[0], a1 = p[4 * PITCH];
      const float w0 = xy[0], w1 = xy[32];
      a0.x = fmaf(cz.x, w0, a0.x);
      a0.y = fmaf(cz.y, w0, a0.y);
      a1.x = fmaf(cz.x, w1, a1.x);
      a1.y = fmaf(cz.y, w1, a1.y);
      p[0] = a0;
      p[4 * PITCH] = a1;
      mt = mn;
    }
    __syncthreads();
  }
  // the tile's shared-memory writes, made visible to the bulk (async) copy
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();

  // (the bulk copy's shared-memory source must be 128-byte aligned)
  // the tile's origin in the (possibly centred) grid; a whole number of tiles
  const int q0 = wrap_once(o0 + G.sh[0], G.Nt[0]), q1 = wrap_once(o1 + G.sh[1], G.Nt[1]);
  const int q2 = wrap_once(o2 + G.sh[2], G.Nt[2]);
  if (use_tma && tile3_interior<BX, BY, BZ>(G, q0, q1, q2) &&
      (static_cast<unsigned>(__cvta_generic_to_shared(acc)) & 127u) == 0) {
    if (threadIdx.x == 0) {
      const int x = 2 * (q0 - 4), y = q1 - 3, z = q2 - 3;  // x in floats: a multiple of 4 (16 bytes)
      const unsigned src = static_cast<unsigned>(__cvta_generic_to_shared(acc));
      asm volatile(
          "cp.reduce.async.bulk.tensor.3d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2, %3}], [%4];"
          ::"l"(reinterpret_cast<uint64_t>(&tmap)), "r"(x), "r"(y), "r"(z), "r"(src)
          : "memory");
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // the tile has been read before exit
    }
    return;
  }
  // wrapping tiles: per-point flush from padded column 1 (grid x o0 - m + 1)
  flush_tile<3, float, false, 8>(G, acc + 1, g, o0, o1, o2, TC::P0 - 1, TC::P1, TC::P2, PITCH);
}

// Variant with one staging step: thread (node s, row iy) of a batch loads
// the node's record, value (from the caller's order through the node's input
// index: no separate value sort) and window values (from the table, or its
// fractional offsets for Horner evaluation) itself, a batch ahead in
// registers, and writes row iy of the x-y products and the 16-byte record of
// the warp that owns window slice iy, warp (z0 + iy) mod 8: {offset of the
// warp's first tap in the padded tile, value x z window value iy}.  The
// tap loop then reads one broadcast record per node instead of a node record
// and a slice value, and the staging needs neither a window-value area nor a
// second CTA barrier: ~11 instead of ~15 shared-memory wavefronts per node
// and warp outside the taps' read-modify-writes.
template <int BX, int BY, int BZ> struct Tile3Rec {
  using TC = Tile3<BX, BY, BZ>;
  static constexpr int NB = 32;
  static constexpr size_t REC_BYTES = size_t(NB) * 8 * 16;  // float4 [NB][8 warps]
  static constexpr size_t XY_OFF = TC::ACC_BYTES + REC_BYTES;
  static constexpr size_t BAR_OFF = XY_OFF + size_t(NB) * 64 * 4;  // mbarrier of the tile's zero fill
  static constexpr size_t SMEM = BAR_OFF + 16;
};

// The polynomial window's coefficients, column l at c[9 l .. 9 l + 8]
// (degree 2m = 8 at m = 4), passed by value so that uniform reads hit the
// constant cache.
struct WinCoeffs8 {
  float c[8 * 9];
};

__device__ __forceinline__ float horner9(const float* c, float t) {
  float v = c[8];
#pragma unroll
  for (int i = 7; i >= 0; --i) v = fmaf(v, t, c[i]);
  return v;
}

template <int BX, int BY, int BZ, bool TABLE>
__global__ void __launch_bounds__(256, 4) spread_tile3_rec_kernel(const __grid_constant__ CUtensorMap tmap, int use_tma,
                                                                Geom<float> G, Nodes<float> Nd,
                                                                const int4* __restrict__ tasks,
                                                                const float2* __restrict__ fhat,
                                                                float* __restrict__ g, int64_t fcol, int64_t gcol,
                                                                const float4* __restrict__ zeros, int* status,
                                                                const __grid_constant__ WinCoeffs8 wc) {
  using TC = Tile3<BX, BY, BZ>;
  using TR = Tile3Rec<BX, BY, BZ>;
  constexpr int NB = TR::NB, PITCH = TC::PITCH, PLANE = TC::PLANE;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  fhat += blockIdx.y * fcol;  // column of a multi-column launch
  g += blockIdx.y * gcol;
  float2* acc = reinterpret_cast<float2*>(smem_raw);
  float4* s_rec = reinterpret_cast<float4*>(smem_raw + TC::ACC_BYTES);        // [NB][8]
  float* s_xy = reinterpret_cast<float*>(smem_raw + TR::XY_OFF);  // [NB][64]
  const unsigned acc_s = static_cast<unsigned>(__cvta_generic_to_shared(acc));
  const unsigned bar_s = static_cast<unsigned>(__cvta_generic_to_shared(smem_raw + TR::BAR_OFF));
  const int4 task = tasks[blockIdx.x];
  const int tile = task.x;
  const int tc0 = tile % G.ntiles[0];
  const int tc1 = (tile / G.ntiles[0]) % G.ntiles[1];
  const int tc2 = tile / (G.ntiles[0] * G.ntiles[1]);
  const int o0 = tc0 * BX, o1 = tc1 * BY, o2 = tc2 * BZ;
  // zero fill of the tile: one bulk copy from a zeroed global buffer (the
  // copy engine writes shared memory; the load/store pipe stays free for the
  // staging), or plain stores without that buffer
  if (zeros) {
    if (threadIdx.x == 0) {
      mbar_init(bar_s, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      mbar_expect_tx(bar_s, unsigned(TC::NACC) * 8u);
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       acc_s),
                   "l"(zeros), "r"(unsigned(TC::NACC) * 8u), "r"(bar_s)
                   : "memory");
    }
  } else {
    float4* a4 = reinterpret_cast<float4*>(acc);
    for (int q = threadIdx.x; q < TC::NACC / 2; q += TC::THREADS) a4[q] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int s = threadIdx.x >> 3, iy = threadIdx.x & 7, hsel = (iy >> 2) & 1;
  bool zeroed = zeros == nullptr;  // the zero fill has landed

  // register prefetch of this thread's node of one batch: record, value,
  // and the x window values with y / z window value iy (table) or the
  // fractional offsets (Horner)
  int4 r_nd = make_int4(0, 0, 0, 0);
  float2 r_c = make_float2(0.f, 0.f);
  float4 r_x0 = make_float4(0.f, 0.f, 0.f, 0.f), r_x1 = r_x0, r_f = r_x0;
  float r_y = 0.f, r_z = 0.f;
  float cy[9];  // Horner: the coefficients of window column iy
  if constexpr (!TABLE) {
#pragma unroll
    for (int i = 0; i < 9; ++i) cy[i] = wc.c[iy * 9 + i];
  }
  auto prefetch = [&](int b) {
    const int j = b + s;
    if (j < task.z) {
      r_nd = __ldg(Nd.node4 + j);
      r_c = __ldg(fhat + r_nd.w);
      if constexpr (TABLE) {
        const float* wt = Nd.wtab + int64_t(j) * 24;
        r_x0 = __ldg(reinterpret_cast<const float4*>(wt));
        r_x1 = __ldg(reinterpret_cast<const float4*>(wt + 4));
        r_y = __ldg(wt + 8 + iy);
        r_z = __ldg(wt + 16 + iy);
      } else {
        r_f = __ldg(reinterpret_cast<const float4*>(Nd.frac4) + j);
      }
    }
  };
  if (task.y < task.z) prefetch(task.y);
  __syncthreads();

  float2* const accl = acc + (lane >> 3) * PITCH + (lane & 7);  // this lane's tap (x = lane mod 8, row = lane / 8)
  for (int b = task.y; b < task.z; b += NB) {
    const int n = min(NB, task.z - b);
    if (s < n) {
      float wy = r_y, wz = r_z;
      if constexpr (!TABLE) {  // evalpoly(frac - 1/2, coefficients of column l)
        const float tx = r_f.x - 0.5f;
        r_x0 = make_float4(horner9(wc.c + 0, tx), horner9(wc.c + 9, tx), horner9(wc.c + 18, tx),
                           horner9(wc.c + 27, tx));
        r_x1 = make_float4(horner9(wc.c + 36, tx), horner9(wc.c + 45, tx), horner9(wc.c + 54, tx),
                           horner9(wc.c + 63, tx));
        wy = horner9(cy, r_f.y - 0.5f);
        wz = horner9(cy, r_f.z - 0.5f);
      }
      // the record of the warp that owns window slice iy (tile plane z0 + iy)
      const int z0 = r_nd.z - o2;
      const int off = (z0 + iy) * PLANE + (r_nd.y - o1) * PITCH + (r_nd.x - o0 + 1);
      s_rec[s * 8 + ((z0 + iy) & 7)] = make_float4(__int_as_float(off), 0.f, r_c.x * wz, r_c.y * wz);
      // row iy of the x-y products; the two halves in an order that keeps
      // the eight lanes of each 128-bit store phase on distinct banks
      float4* out = reinterpret_cast<float4*>(s_xy + s * 64 + iy * 8);
      const float4 xa = hsel ? r_x1 : r_x0, xb = hsel ? r_x0 : r_x1;
      out[hsel] = make_float4(xa.x * wy, xa.y * wy, xa.z * wy, xa.w * wy);
      out[hsel ^ 1] = make_float4(xb.x * wy, xb.y * wy, xb.z * wy, xb.w * wy);
    }
    __syncthreads();
    if (b + NB < task.z) prefetch(b + NB);
    if (!zeroed) {  // (bounded: on timeout the CTA raises its status bit and adds nothing)
      zeroed = __syncthreads_and(mbar_wait_bounded(bar_s, 0));  // the whole CTA agrees
      if (!zeroed) break;
    }
    // taps: warp w updates its slice of every node, rows iy and iy + 4 of the
    // lane's column; the next node's record is loaded during this node's taps
    float4 rt = s_rec[warp];
    for (int q = 0; q < n; ++q) {
      const float4 rn = s_rec[(q + 1) * 8 + warp];  // (past the last node: in-bounds, unused)
      float2* p = accl + __float_as_int(rt.x);
      const float* xy = s_xy + q * 64 + lane;
      float2 a0 = p[0], a1 = p[4 * PITCH];
      const float w0 = xy[0], w1 = xy[32];
      a0.x = fmaf(rt.z, w0, a0.x);
      a0.y = fmaf(rt.w, w0, a0.y);
      a1.x = fmaf(rt.z, w1, a1.x);
      a1.y = fmaf(rt.w, w1, a1.y);
      p[0] = a0;
      p[4 * PITCH] = a1;
      rt = rn;
    }
    __syncthreads();
  }
  // a task without nodes (or a timed-out wait) still waits for its zero
  // fill, so that no copy into shared memory outlives the CTA
  if (!zeroed) zeroed = mbar_wait_bounded(bar_s, 0);
  // the tile's shared-memory writes, made visible to the bulk (async) copy
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (!__syncthreads_and(zeroed)) {
    if (threadIdx.x == 0) atomicOr(status, 1);
    return;
  }
  const int q0 = wrap_once(o0 + G.sh[0], G.Nt[0]), q1 = wrap_once(o1 + G.sh[1], G.Nt[1]);
  const int q2 = wrap_once(o2 + G.sh[2], G.Nt[2]);
  if (use_tma && tile3_interior<BX, BY, BZ>(G, q0, q1, q2) && (acc_s & 127u) == 0) {
    if (threadIdx.x == 0) {
      const int x = 2 * (q0 - 4), y = q1 - 3, z = q2 - 3;  // x in floats: a multiple of 4 (16 bytes)
      asm volatile(
          "cp.reduce.async.bulk.tensor.3d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2, %3}], [%4];"
          ::"l"(reinterpret_cast<uint64_t>(&tmap)), "r"(x), "r"(y), "r"(z), "r"(acc_s)
          : "memory");
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // the tile has been read before exit
    }
    return;
  }
  flush_tile<3, float, false, 8>(G, acc + 1, g, o0, o1, o2, TC::P0 - 1, TC::P1, TC::P2, PITCH);
}

}  // namespace
}  // namespace nfft
