// Gather interpolation (convolve!): fHat[j] = sum over the (2m)^D window taps
// of prod_d phi_d * g[tap], src/convolution.jl:229-344 (blocked) and :56-99.
//
// Warp per node (D >= 2) or 32/G nodes per warp (D = 1), nodes visited in
// bin-sorted order; for D >= 2 each CTA takes a contiguous chunk of the
// sorted nodes, so the nodes an SM visits close in time read overlapping grid
// neighbourhoods through L1, and a warp issues all of a node's grid loads
// before its sums (memory-level parallelism).  Window values come from the stored window
// tensor (TENSOR / FULL / LINEAR) or from the fitted polynomial evaluated with
// its coefficients held in registers (POLYNOMIAL).  Grid offsets within a
// plane are 32-bit; the plane offset is 64-bit.
#include "interp_body.cuh"
#include "tile3.cuh"

namespace nfft {
namespace {

constexpr int kInterpThreads = 256;

// 8- or 16-byte asynchronous global -> shared copy (cp.async, sm_80+).
template <typename C> __device__ __forceinline__ void cp_async_elem(C* smem, const C* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  if constexpr (sizeof(C) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <int D, int L, typename T, bool TABLE, bool COLS = false>
__global__ void __launch_bounds__(kInterpThreads) interp_kernel(Geom<T> G, Nodes<T> Nd,
                                                                 const typename Cplx<T>::type* __restrict__ g,
                                                                 typename Cplx<T>::type* __restrict__ fhat,
                                                                 int64_t gcol = 0, int64_t fcol = 0) {
  using C = typename Cplx<T>::type;
  using LN = Lanes<D, L>;
  if constexpr (COLS) {  // column of a multi-column launch
    g += blockIdx.y * gcol;
    fhat += blockIdx.y * fcol;
  }
  const int lane = threadIdx.x & 31;
  const int64_t warp_global = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int64_t warps_total = int64_t(gridDim.x) * (blockDim.x >> 5);
  const int m = G.m;
  const bool small = G.small_grid;

  if constexpr (D == 1) {
    // 32/G1 nodes per warp, lane -> (node slot, tap ix)
    const int slot = lane / LN::G1, ix = lane % LN::G1;
    const bool act = ix < L;
    T c[LN::DEG];
    if constexpr (!TABLE) {
#pragma unroll
      for (int q = 0; q < LN::DEG; ++q) c[q] = act ? __ldg(G.coeffs + ix * LN::DEG + q) : T(0);
    }
    for (int64_t base = warp_global * LN::NPW; base < Nd.M; base += warps_total * LN::NPW) {
      const int64_t i = base + slot;
      T ar = T(0), ai = T(0);
      int4 nd = make_int4(0, 0, 0, 0);
      if (i < Nd.M) nd = __ldg(Nd.node4 + i);
      if (i < Nd.M && act) {
        T w;
        if constexpr (TABLE) {
          w = __ldg(Nd.wtab + i * L + ix);
        } else {
          const T t = __ldg(Nd.frac4 + 4 * i) - T(0.5);
          w = c[LN::DEG - 1];
#pragma unroll
          for (int q = LN::DEG - 2; q >= 0; --q) w = fma(w, t, c[q]);
        }
        const int gx = small ? wrap_any(nd.x + G.sh[0] - m + 1 + ix, G.Nt[0])
                             : wrap_once(nd.x + G.sh[0] - m + 1 + ix, G.Nt[0]);
        const C v = __ldg(g + gx);
        ar = w * v.x;
        ai = w * v.y;
      }
#pragma unroll
      for (int o = LN::G1 / 2; o > 0; o >>= 1) {
        ar += __shfl_xor_sync(0xFFFFFFFFu, ar, o);
        ai += __shfl_xor_sync(0xFFFFFFFFu, ai, o);
      }
      if (ix == 0 && i < Nd.M) {
        C r;
        r.x = ar;
        r.y = ai;
        fhat[nd.w] = r;
      }
    }
  } else {
    PolyRegs<D, L, T> P;
    if constexpr (!TABLE) P.load(G.coeffs, lane);
    // each CTA takes a contiguous chunk of the bin-sorted nodes: nodes a CTA
    // visits close in time share their grid neighbourhood in L1
    const int64_t chunk = (Nd.M + gridDim.x - 1) / gridDim.x;
    const int64_t lo = int64_t(blockIdx.x) * chunk;
    const int64_t hi = lo + chunk < Nd.M ? lo + chunk : Nd.M;
    for (int64_t i = lo + (threadIdx.x >> 5); i < hi; i += blockDim.x >> 5)
      interp_node<D, L, T, TABLE>(G, Nd, P, i, lane, g, fhat);
  }
}

// Tile-staged gather: one CTA per spreading task (home tile or chunk of a hot
// tile).  The CTA copies the tile's padded neighbourhood of the grid (with
// periodic wrap) into shared memory with coalesced row loads, then each warp
// interpolates one node at a time from shared memory: no wrap logic and no
// global addressing in the tap loop.
template <int D, int L, typename T, bool TABLE>
__global__ void __launch_bounds__(kInterpThreads) interp_tile_kernel(Geom<T> G, Nodes<T> Nd,
                                                                      const int4* __restrict__ tasks,
                                                                      const typename Cplx<T>::type* __restrict__ g,
                                                                      typename Cplx<T>::type* __restrict__ fhat,
                                                                      int pitch) {
  using C = typename Cplx<T>::type;
  using LN = Lanes<D, L>;
  extern __shared__ __align__(32) unsigned char smem_raw[];
  C* tile = reinterpret_cast<C*>(smem_raw);
  const int4 task = tasks[blockIdx.x];
  const int t = task.x;
  const int tc0 = t % G.ntiles[0];
  const int tc1 = (t / G.ntiles[0]) % G.ntiles[1];
  const int tc2 = t / (G.ntiles[0] * G.ntiles[1]);
  const int P0 = G.bs[0] + L - 1;
  const int P1 = D >= 2 ? G.bs[1] + L - 1 : 1;
  const int P2 = D == 3 ? G.bs[2] + L - 1 : 1;
  const int o0 = tc0 * G.bs[0], o1 = D >= 2 ? tc1 * G.bs[1] : 0, o2 = D == 3 ? tc2 * G.bs[2] : 0;
  const int plane = pitch * P1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int m1 = G.m - 1;
  const bool small = G.small_grid;
  // stage the padded tile with asynchronous copies (cp.async): every row
  // copy is issued before the single wait, so a warp keeps all of its rows'
  // loads in flight instead of one load-store round trip per row
  {
    const int rows = P1 * P2;
    int r = warp, y = r % P1, z = r / P1;
    for (; r < rows; r += nwarps) {
      const int gy = D >= 2 ? wrap_any(o1 + G.sh[1] - m1 + y, G.Nt[1]) : 0;
      const int gz = D == 3 ? wrap_any(o2 + G.sh[2] - m1 + z, G.Nt[2]) : 0;
      const C* grow = g + int64_t(gz) * G.plane + int64_t(gy) * G.Nt[0];
      C* srow = tile + z * plane + y * pitch;
      for (int x = lane; x < P0; x += 32) {
        const int gx = wrap_any(o0 + G.sh[0] - m1 + x, G.Nt[0]);
        cp_async_elem(srow + x, grow + gx);
      }
      y += nwarps;
      while (y >= P1) {
        y -= P1;
        ++z;
      }
    }
    cp_async_wait_all();
  }
  __syncthreads();
  if constexpr (D == 1) {
    const int slot = lane / LN::G1, ix = lane % LN::G1;
    const bool act = ix < L;
    T c[LN::DEG];
    if constexpr (!TABLE) {
#pragma unroll
      for (int q = 0; q < LN::DEG; ++q) c[q] = act ? __ldg(G.coeffs + ix * LN::DEG + q) : T(0);
    }
    for (int b = task.y + warp * LN::NPW; b < task.z; b += nwarps * LN::NPW) {
      const int i = b + slot;
      T ar = T(0), ai = T(0);
      int4 nd = make_int4(0, 0, 0, 0);
      if (i < task.z) nd = __ldg(Nd.node4 + i);
      if (i < task.z && act) {
        T w;
        if constexpr (TABLE) {
          w = __ldg(Nd.wtab + int64_t(i) * L + ix);
        } else {
          const T tt = __ldg(Nd.frac4 + 4 * int64_t(i)) - T(0.5);
          w = c[LN::DEG - 1];
#pragma unroll
          for (int q = LN::DEG - 2; q >= 0; --q) w = fma(w, tt, c[q]);
        }
        const C v = tile[nd.x - o0 + ix];
        ar = w * v.x;
        ai = w * v.y;
      }
#pragma unroll
      for (int o = LN::G1 / 2; o > 0; o >>= 1) {
        ar += __shfl_xor_sync(0xFFFFFFFFu, ar, o);
        ai += __shfl_xor_sync(0xFFFFFFFFu, ai, o);
      }
      if (ix == 0 && i < task.z) {
        C r;
        r.x = ar;
        r.y = ai;
        fhat[nd.w] = r;
      }
    }
  } else {
    PolyRegs<D, L, T> P;
    if constexpr (!TABLE) P.load(G.coeffs, lane);
    const int ix = lane % L, ry = lane / L;
    const bool xact = ry < LN::RY;
    for (int i = task.y + warp; i < task.z; i += nwarps) {
      const int4 nd = __ldg(Nd.node4 + i);
      T W[LN::NW];
      node_weights<D, L, T, TABLE>(Nd, P, i, lane, W);
      const T wx = wsel<D, L>(W, ix);
      const int px = nd.x - o0 + ix, py = nd.y - o1;
      int row[LN::NSTEP];
      T wxy[LN::NSTEP];
#pragma unroll
      for (int s = 0; s < LN::NSTEP; ++s) {
        const int iy = s * LN::RY + ry;
        const bool ok = xact && iy < L;
        const int iyc = ok ? iy : 0;
        const T wy = wsel<D, L>(W, L + iyc);  // every lane shuffles
        row[s] = (py + iyc) * pitch + px;
        wxy[s] = ok ? wx * wy : T(0);
      }
      T ar = T(0), ai = T(0);
      if constexpr (D == 2) {
#pragma unroll
        for (int s = 0; s < LN::NSTEP; ++s) {
          const C v = tile[row[s]];
          ar = fma(wxy[s], v.x, ar);
          ai = fma(wxy[s], v.y, ai);
        }
      } else {
        const C* pl = tile + (nd.z - o2) * plane;
#pragma unroll
        for (int iz = 0; iz < L; ++iz) {
          const T wz = wsel<D, L>(W, 2 * L + iz);
#pragma unroll
          for (int s = 0; s < LN::NSTEP; ++s) {
            const C v = pl[iz * plane + row[s]];
            const T w = wxy[s] * wz;
            ar = fma(w, v.x, ar);
            ai = fma(w, v.y, ai);
          }
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        ar += __shfl_xor_sync(0xFFFFFFFFu, ar, o);
        ai += __shfl_xor_sync(0xFFFFFFFFu, ai, o);
      }
      if (lane == 0) {
        C r;
        r.x = ar;
        r.y = ai;
        fhat[nd.w] = r;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Shape-specialised 3-D FP32 gather (m = 4, the tiles of tile3.cuh).  One CTA
// per spreading task; a tile whose padded box lies inside the grid is brought
// into shared memory by one bulk tensor copy (TMA, completion on an
// mbarrier), and each warp then interpolates one node at a time from shared
// memory: lane (x = lane mod 8, row = lane / 8) reads its 8 z values of rows
// iy and iy + 4 at constant offsets (16 loads, 2 wavefronts each), sums over
// z and weights by phi_x phi_y; the warp adds the 32 partial sums of four
// nodes at once.  Window values come straight from the table (broadcast
// loads): shuffles share the shared-memory pipe with the tile reads.  Tiles
// whose box wraps around the grid gather their nodes straight from L1/L2 as
// interp_kernel does.  The wait for the copy is bounded: on timeout the CTA
// raises status word 1 (reported by nfft_sync) and skips its nodes.


// Per-warp staging of the TMA gather: NK nodes per group, WCH 16-byte chunks
// of window data per node (24 table values, or the 4 fractional offsets),
// one slot = NK records + NK window blocks; two slots per warp.
template <bool TABLE> struct Tile3Gather {
  static constexpr int NK = 4;
  static constexpr int WCH = TABLE ? 6 : 1;
  // records, window values (copied from the table, or evaluated by Horner
  // from the fractional offsets staged behind them)
  static constexpr int SLOT = NK * (16 + 96 + (TABLE ? 0 : 16));
  static constexpr int NS = 2;  // (3 slots measured the same, 4 cost a CTA per SM)
  static constexpr size_t STAGE_BYTES = size_t(kInterpThreads / 32) * NS * SLOT;
};

template <int BX, int BY, int BZ, bool TABLE>
__global__ void __launch_bounds__(kInterpThreads, 4) interp_tile3_kernel(const __grid_constant__ CUtensorMap tmap,
                                                                       Geom<float> G, Nodes<float> Nd,
                                                                       const int4* __restrict__ tasks,
                                                                       const float2* __restrict__ g,
                                                                       float2* __restrict__ fhat, int* status,
                                                                       int pf_dist) {
  using TC = Tile3<BX, BY, BZ>;
  using LN = Lanes<3, 8>;
  constexpr int PITCH = TC::PITCH, PLANE = TC::PLANE;
  constexpr unsigned BOX_BYTES = unsigned(2 * PITCH) * 4u * TC::P1 * TC::P2;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  float2* tile = reinterpret_cast<float2*>(smem_raw);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw + TC::ACC_BYTES);
  const int4 task = tasks[blockIdx.x];
  const int t = task.x;
  const int tc0 = t % G.ntiles[0];
  const int tc1 = (t / G.ntiles[0]) % G.ntiles[1];
  const int tc2 = t / (G.ntiles[0] * G.ntiles[1]);
  const int o0 = tc0 * BX, o1 = tc1 * BY, o2 = tc2 * BZ;
  // the tile's origin in the (possibly centred) grid; a whole number of tiles
  const int q0 = wrap_once(o0 + G.sh[0], G.Nt[0]), q1 = wrap_once(o1 + G.sh[1], G.Nt[1]);
  const int q2 = wrap_once(o2 + G.sh[2], G.Nt[2]);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NWARPS = kInterpThreads / 32;
  PolyRegs<3, 8, float> P;
  if constexpr (!TABLE) P.load(G.coeffs, lane);
  const unsigned tile_s = static_cast<unsigned>(__cvta_generic_to_shared(tile));
  const unsigned mbar_s = static_cast<unsigned>(__cvta_generic_to_shared(mbar));
  // the bulk copy's shared-memory destination must be 128-byte aligned
  if (!tile3_interior<BX, BY, BZ>(G, q0, q1, q2) || (tile_s & 127u) != 0) {
    for (int64_t i = task.y + warp; i < task.z; i += NWARPS) interp_node<3, 8, float, TABLE>(G, Nd, P, i, lane, g, fhat);
    return;
  }
  // Warp w takes the nodes task.y + NK w + NK NWARPS j + k, k < NK: the NK
  // nodes' partial sums are reduced together (transposed butterfly: 3
  // shuffles per node and component instead of 5).  The node records and
  // window data (table values, or fractional offsets for Horner) of the next
  // group are copied into the warp's other stage slot by cp.async while this
  // group is summed; the first group's while the tile arrives.
  constexpr int NK = Tile3Gather<TABLE>::NK, WCH = Tile3Gather<TABLE>::WCH, SLOT = Tile3Gather<TABLE>::SLOT;
  constexpr int NS = Tile3Gather<TABLE>::NS;
  const int ix = lane & 7, ry = lane >> 3;
  unsigned char* stage_base = smem_raw + TC::ACC_BYTES + 16 + warp * NS * SLOT;
  // this lane's copy in a stage: window chunk c of node k (lanes < NK WCH)
  // or the record of node lane - 24 (lanes 24 .. 24 + NK - 1); node indices
  // within a task fit in 32 bits
  const bool win_lane = lane < NK * WCH, rec_lane = lane >= 24 && lane < 24 + NK;
  const int cp_k = win_lane ? lane / WCH : lane - 24, cp_c = win_lane ? lane % WCH : 0;
  const int cp_dst = win_lane ? (TABLE ? NK * 16 + cp_k * 96 + 16 * cp_c : NK * (16 + 96) + 16 * cp_k) : 16 * cp_k;
  auto stage = [&](int buf, int gbase) {
    const int id = gbase + cp_k;
    if ((win_lane || rec_lane) && id < task.z) {
      const float4* src = win_lane ? reinterpret_cast<const float4*>(TABLE ? Nd.wtab + int64_t(id) * 24 + 4 * cp_c
                                                                              : Nd.frac4 + 4 * int64_t(id))
                                   : reinterpret_cast<const float4*>(Nd.node4 + id);
      cp_async_elem(reinterpret_cast<float4*>(stage_base + buf * SLOT + cp_dst), src);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
#pragma unroll
  for (int b = 0; b + 1 < NS; ++b) stage(b, task.y + NK * warp + b * NK * NWARPS);
  if (threadIdx.x == 0) {
    mbar_init(mbar_s, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(mbar_s, BOX_BYTES);
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(tile_s),
        "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(2 * (q0 - 4)), "r"(q1 - 3), "r"(q2 - 3), "r"(mbar_s)
        : "memory");
  } else if (threadIdx.x == 32 && pf_dist > 0 && blockIdx.x + unsigned(pf_dist) < gridDim.x) {
    // the tile of the task about one wave of resident CTAs ahead, fetched
    // into L2 now so that its CTA's bulk copy need not wait on DRAM
    const int tn = tasks[blockIdx.x + pf_dist].x;
    if (tn != t) {
      const int p0 = wrap_once((tn % G.ntiles[0]) * BX + G.sh[0], G.Nt[0]);
      const int p1 = wrap_once(((tn / G.ntiles[0]) % G.ntiles[1]) * BY + G.sh[1], G.Nt[1]);
      const int p2 = wrap_once((tn / (G.ntiles[0] * G.ntiles[1])) * BZ + G.sh[2], G.Nt[2]);
      if (tile3_interior<BX, BY, BZ>(G, p0, p1, p2))
        asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];" ::"l"(
                         reinterpret_cast<uint64_t>(&tmap)),
                     "r"(2 * (p0 - 4)), "r"(p1 - 3), "r"(p2 - 3)
                     : "memory");
    }
  }
  bool done = false;
  for (int it = 0; it < (1 << 22) && !done; ++it) done = mbar_try_wait(mbar_s, 0);
  if (!done) {
    asm volatile("cp.async.wait_all;" ::: "memory");  // no copy into shared memory outlives the CTA
    if (threadIdx.x == 0) atomicOr(status, 1);
    return;
  }
  int buf = 0;
  // the lane's tap offset in the tile relative to a node's grid index
  const int lane_off = ry * PITCH + ix + 1 - o0 - o1 * PITCH - o2 * PLANE;
  for (int base = task.y + NK * warp; base < task.z; base += NK * NWARPS) {
    stage(buf == 0 ? NS - 1 : buf - 1, base + (NS - 1) * NK * NWARPS);
    asm volatile("cp.async.wait_group %0;" ::"n"(NS - 1) : "memory");  // this group's slot has landed
    __syncwarp();
    unsigned char* st = stage_base + buf * SLOT;
    if constexpr (!TABLE) {
      // the group's 4 x 24 window values, three per lane: value q = lane + 32 r
      // is column q mod 8 = lane mod 8 (the lane's coefficients) of dimension
      // (q mod 24) / 8 of node q / 24, evalpoly(frac - 1/2, coefficients)
      const float* fr = reinterpret_cast<const float*>(st + NK * (16 + 96));
      float* wv = reinterpret_cast<float*>(st + NK * 16);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const int q = lane + 32 * r, k = q / 24, d = (q % 24) / 8;
        if (base + k < task.z) wv[q] = P.eval(0, fr[4 * k + d]);
      }
      __syncwarp();
    }
    const int4* rec = reinterpret_cast<const int4*>(st);
    const float* win = reinterpret_cast<const float*>(st + NK * 16);
    float ar[NK], ai[NK];
    // node k's partial sums (tail groups: nodes past the task end add zero)
    auto node = [&](int k, bool valid) {
      const int4 nd = rec[k];
      // window values: x at the lane's column, y at its two rows, all 8 z
      float wx, wy0, wy1, wz[8];
      {  // broadcast reads of the staged window values
        const float* wt = win + k * 24;
        wx = wt[ix];
        wy0 = wt[8 + ry];
        wy1 = wt[12 + ry];
        const float4 z0 = *reinterpret_cast<const float4*>(wt + 16);
        const float4 z1 = *reinterpret_cast<const float4*>(wt + 20);
        wz[0] = z0.x, wz[1] = z0.y, wz[2] = z0.z, wz[3] = z0.w;
        wz[4] = z1.x, wz[5] = z1.y, wz[6] = z1.z, wz[7] = z1.w;
      }
      // (a node past the task end reads tap 0 of the tile and is dropped)
      const float2* bp = tile + (valid ? nd.z * PLANE + nd.y * PITCH + nd.x + lane_off : 0);
      float2 v0[8], v1[8];
#pragma unroll
      for (int iz = 0; iz < 8; ++iz) {
        v0[iz] = bp[iz * PLANE];
        v1[iz] = bp[iz * PLANE + 4 * PITCH];
      }
      float s0r = 0.f, s0i = 0.f, s1r = 0.f, s1i = 0.f;
#pragma unroll
      for (int iz = 0; iz < 8; ++iz) {
        s0r = fmaf(wz[iz], v0[iz].x, s0r);
        s0i = fmaf(wz[iz], v0[iz].y, s0i);
        s1r = fmaf(wz[iz], v1[iz].x, s1r);
        s1i = fmaf(wz[iz], v1[iz].y, s1i);
      }
      ar[k] = valid ? wx * fmaf(wy0, s0r, wy1 * s1r) : 0.f;
      ai[k] = valid ? wx * fmaf(wy0, s0i, wy1 * s1i) : 0.f;
    };
    if (base + NK <= task.z) {
#pragma unroll
      for (int k = 0; k < NK; ++k) node(k, true);
    } else {
#pragma unroll
      for (int k = 0; k < NK; ++k) node(k, base + k < task.z);
    }
    // transposed reduction: after the xor-16 and xor-8 steps lane l holds
    // node l / 8 summed over 4 lanes' worth of partials; three more steps
    // finish it on the lanes l = 8 k
    const bool h = (lane & 16) != 0, q = (lane & 8) != 0;
    float a0 = (h ? ar[2] : ar[0]) + __shfl_xor_sync(0xFFFFFFFFu, h ? ar[0] : ar[2], 16);
    float a1 = (h ? ar[3] : ar[1]) + __shfl_xor_sync(0xFFFFFFFFu, h ? ar[1] : ar[3], 16);
    float b0 = (h ? ai[2] : ai[0]) + __shfl_xor_sync(0xFFFFFFFFu, h ? ai[0] : ai[2], 16);
    float b1 = (h ? ai[3] : ai[1]) + __shfl_xor_sync(0xFFFFFFFFu, h ? ai[1] : ai[3], 16);
    float sr = (q ? a1 : a0) + __shfl_xor_sync(0xFFFFFFFFu, q ? a0 : a1, 8);
    float si = (q ? b1 : b0) + __shfl_xor_sync(0xFFFFFFFFu, q ? b0 : b1, 8);
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
      sr += __shfl_xor_sync(0xFFFFFFFFu, sr, o);
      si += __shfl_xor_sync(0xFFFFFFFFu, si, o);
    }
    const int kk = lane >> 3;
    if ((lane & 7) == 0 && base + kk < task.z) fhat[rec[kk].w] = make_float2(sr, si);
    __syncwarp();  // the slot is read before it is staged again
    buf = buf + 1 == NS ? 0 : buf + 1;
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
}

template <int BX, int BY, int BZ>
int interp_tile3_launch(const nfft_plan* p, const CUtensorMap* map, const Geom<float>& G, const Nodes<float>& Nd,
                        const float2* g, float2* fhat) {
  using TC = Tile3<BX, BY, BZ>;
  const size_t smem =
      TC::ACC_BYTES + 16 + (p->wtab ? Tile3Gather<true>::STAGE_BYTES : Tile3Gather<false>::STAGE_BYTES);
  auto kern = p->wtab ? interp_tile3_kernel<BX, BY, BZ, true> : interp_tile3_kernel<BX, BY, BZ, false>;
  NFFT_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    sms = 0;
  kern<<<unsigned(p->n_tasks), kInterpThreads, smem, p->stream>>>(*map, G, Nd, p->tasks, g, fhat, p->dflag + 1,
                                                                   p->gather_pf * sms);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

// The TMA-tiled 3-D gather when the plan has one of the fixed tile shapes and
// the grid's tensor map can be made; -1 = not applicable.
int interp_tile3(const nfft_plan* cp, const Geom<float>& G, const Nodes<float>& Nd, const float2* g, float2* fhat) {
  nfft_plan* p = const_cast<nfft_plan*>(cp);  // the tensor-map cache only
  if (!p->gather_tma || !p->tasks || p->n_tasks == 0 || !tile3_shape(p)) return -1;
  void* gv = const_cast<float2*>(g);
  const int64_t bx = p->bs[0], by = p->bs[1];
  const CUtensorMap* map = nullptr;
  if (bx == 16 && by == 8) return (map = tile3_map<16, 8, 8>(p, gv)) ? interp_tile3_launch<16, 8, 8>(p, map, G, Nd, g, fhat) : -1;
  if (bx == 16 && by == 16)
    return (map = tile3_map<16, 16, 8>(p, gv)) ? interp_tile3_launch<16, 16, 8>(p, map, G, Nd, g, fhat) : -1;
  if (bx == 32 && by == 8) return (map = tile3_map<32, 8, 8>(p, gv)) ? interp_tile3_launch<32, 8, 8>(p, map, G, Nd, g, fhat) : -1;
  if (bx == 8 && by == 8) return (map = tile3_map<8, 8, 8>(p, gv)) ? interp_tile3_launch<8, 8, 8>(p, map, G, Nd, g, fhat) : -1;
  return -1;
}

// ncols columns in one launch (blockIdx.y): grids g + c gcol, values fhat + c fcol.
template <int D, int L, typename T>
int interp_launch(const nfft_plan* p, const void* g, void* fhat, int ncols, int64_t gcol, int64_t fcol) {
  Geom<T> G = make_geom<T>(p);
  Nodes<T> Nd = make_nodes<T>(p);
  if (Nd.M == 0) return NFFT_OK;
  using C = typename Cplx<T>::type;
  const int64_t per_block = (kInterpThreads / 32) * (D == 1 ? Lanes<D, L>::NPW : 1);
  int64_t blocks = (Nd.M + per_block - 1) / per_block;
  int dev = 0, sms = 1;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                cudaSuccess || sms < 1)
    sms = 1;
  const int64_t cap = (int64_t(sms) * 64 + ncols - 1) / ncols;
  if (blocks > cap) blocks = cap;
  const C* gp = static_cast<const C*>(g);
  C* fp = static_cast<C*>(fhat);
  if (ncols > 1) {
    const dim3 grid{unsigned(blocks), unsigned(ncols), 1u};
    if (p->wtab)
      interp_kernel<D, L, T, true, true><<<grid, kInterpThreads, 0, p->stream>>>(G, Nd, gp, fp, gcol, fcol);
    else
      interp_kernel<D, L, T, false, true><<<grid, kInterpThreads, 0, p->stream>>>(G, Nd, gp, fp, gcol, fcol);
    NFFT_LAUNCH_CHECK();
    return NFFT_OK;
  }
  if constexpr (D == 3 && L == 8 && sizeof(T) == 4) {
    const int rc = interp_tile3(p, G, Nd, gp, fp);
    if (rc != -1) return rc;
  }
  if (p->tasks && p->gather_tiled) {
    const int P1 = D >= 2 ? int(p->bs[1]) + L - 1 : 1;
    const int P2 = D == 3 ? int(p->bs[2]) + L - 1 : 1;
    const size_t smem = sizeof(C) * size_t(p->gather_pitch) * P1 * P2;
    if (smem <= 227 * 1024 && p->n_tasks > 0) {
      auto kern = p->wtab ? interp_tile_kernel<D, L, T, true> : interp_tile_kernel<D, L, T, false>;
      NFFT_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
      kern<<<unsigned(p->n_tasks), kInterpThreads, smem, p->stream>>>(G, Nd, p->tasks, gp, fp, p->gather_pitch);
      NFFT_LAUNCH_CHECK();
      return NFFT_OK;
    }
  }
  if (p->wtab)
    interp_kernel<D, L, T, true><<<unsigned(blocks), kInterpThreads, 0, p->stream>>>(G, Nd, gp, fp);
  else
    interp_kernel<D, L, T, false><<<unsigned(blocks), kInterpThreads, 0, p->stream>>>(G, Nd, gp, fp);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

#define NFFT_INTERP_ARGS p, g, fhat, ncols, gcol, fcol
template <int D, typename T>
int interp_dispatch_l(const nfft_plan* p, const void* g, void* fhat, int ncols, int64_t gcol, int64_t fcol) {
  switch (p->m) {
    case 2: return interp_launch<D, 4, T>(NFFT_INTERP_ARGS);
    case 3: return interp_launch<D, 6, T>(NFFT_INTERP_ARGS);
    case 4: return interp_launch<D, 8, T>(NFFT_INTERP_ARGS);
    case 5: return interp_launch<D, 10, T>(NFFT_INTERP_ARGS);
    case 6: return interp_launch<D, 12, T>(NFFT_INTERP_ARGS);
    case 7: return interp_launch<D, 14, T>(NFFT_INTERP_ARGS);
    case 8: return interp_launch<D, 16, T>(NFFT_INTERP_ARGS);
  }
  set_error("m = %d not supported (2..8)", p->m);
  return NFFT_ERR_UNSUPPORTED;
}

template <typename T>
int interp_dispatch(const nfft_plan* p, const void* g, void* fhat, int ncols, int64_t gcol, int64_t fcol) {
  switch (p->D) {
    case 1: return interp_dispatch_l<1, T>(NFFT_INTERP_ARGS);
    case 2: return interp_dispatch_l<2, T>(NFFT_INTERP_ARGS);
    case 3: return interp_dispatch_l<3, T>(NFFT_INTERP_ARGS);
  }
  return NFFT_ERR_UNSUPPORTED;
}
#undef NFFT_INTERP_ARGS

}  // namespace

int launch_interp(const nfft_plan* p, const void* g, int, void* fhat, int) {
  return p->precision == 32 ? interp_dispatch<float>(p, g, fhat, 1, 0, 0) : interp_dispatch<double>(p, g, fhat, 1, 0, 0);
}

int launch_interp_cols(const nfft_plan* p, const void* g, void* fhat, int ncols, int64_t gcol, int64_t fcol) {
  return p->precision == 32 ? interp_dispatch<float>(p, g, fhat, ncols, gcol, fcol)
                            : interp_dispatch<double>(p, g, fhat, ncols, gcol, fcol);
}

}  // namespace nfft
