// Spreading kernels (device bodies and single-plan kernels), shared by the
// single-plan launchers (spread.cu) and the batched launches (batch.cu).
// See spread.cu for the design.
#pragma once

#include "warpnode.cuh"


namespace nfft {
namespace {

constexpr int kSpreadThreads = 256;
constexpr int kSpreadWarps = kSpreadThreads / 32;
constexpr int kStageNodes = 32;

template <typename T> __device__ __forceinline__ void red_add2(T* g, T x, T y);
template <> __device__ __forceinline__ void red_add2<float>(float* g, float x, float y) {
  atomicAdd(reinterpret_cast<float2*>(g), make_float2(x, y));
}
template <> __device__ __forceinline__ void red_add2<double>(double* g, double x, double y) {
  atomicAdd(g, x);
  atomicAdd(g + 1, y);
}

// Accumulator element: (re, im) or, compensated, (re, im, comp re, comp im).
template <typename T, bool KAHAN> struct Acc;
template <> struct Acc<float, false> { using type = float2; };
template <> struct Acc<double, false> { using type = double2; };
template <> struct Acc<float, true> { using type = float4; };
template <> struct Acc<double, true> { struct __align__(32) type { double x, y, z, w; }; };

// (re, im) of an accumulator element (compensated: sum minus compensation).
template <typename T, typename A, bool KAHAN>
__device__ __forceinline__ void acc_value(const A& a, T& vr, T& vi) {
  vr = a.x;
  vi = a.y;
  if constexpr (KAHAN) {
    vr -= a.z;
    vi -= a.w;
  }
}

// Add the padded tile to the grid: padded point (x, y, z) -> grid point
// ((o - m + 1 + x) mod Ntilde, ...); all-zero units are skipped.  FP32 on a
// 16-byte aligned grid adds two neighbouring points per vector atomic
// (red.global.add.v4.f32): units are grid-aligned pairs (even grid x,
// Ntilde[0] even, so a pair never straddles the periodic wrap), and the
// padded columns outside [0, P0) read as zero.  Otherwise (FP64, or a
// caller's grid that is only 8-byte aligned) a unit is one point.  Lanes
// cover (row, unit) jointly so short rows do not leave most of a warp idle.
template <int D, typename T, bool KAHAN, int NWARPS>
__device__ __forceinline__ void flush_tile(const Geom<T>& G, const typename Acc<T, KAHAN>::type* __restrict__ acc,
                                           T* __restrict__ g, int o0, int o1, int o2, int P0, int P1, int P2,
                                           int pitch) {
  const bool pair = sizeof(T) == 4 && (reinterpret_cast<uintptr_t>(g) & 15) == 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int m1 = G.m - 1;
  const bool small = G.small_grid;
  const int Nt0 = G.Nt[0];
  const int x0 = o0 + G.sh[0] - m1;                        // grid x of padded column 0
  const int lead = pair ? (x0 & 1) : 0;                    // column 0 is the odd half of a pair
  const int nunit = pair ? (P0 + lead + 1) >> 1 : P0;      // units per row
  const int lpr = nunit < 32 ? nunit : 32;                 // lanes per row
  const int rpi = 32 / lpr;                                // rows per warp and iteration
  const int rr = lane / lpr, j0 = lane - rr * lpr;
  const int rows = P1 * P2;
  const int plane = pitch * P1;
  const int step = NWARPS * rpi;
  int r = rr < rpi ? warp * rpi + rr : rows;
  int y = r % P1, z = r / P1;
  for (; r < rows; r += step) {
    const int gy = D >= 2 ? (small ? wrap_any(o1 + G.sh[1] - m1 + y, G.Nt[1]) : wrap_once(o1 + G.sh[1] - m1 + y, G.Nt[1]))
                          : 0;
    const int gz = D == 3 ? (small ? wrap_any(o2 + G.sh[2] - m1 + z, G.Nt[2]) : wrap_once(o2 + G.sh[2] - m1 + z, G.Nt[2]))
                          : 0;
    T* grow = g + 2 * (int64_t(gz) * G.plane + int64_t(gy) * Nt0);
    const auto* srow = acc + z * plane + y * pitch;
    for (int j = j0; j < nunit; j += lpr) {
      if constexpr (sizeof(T) == 4) {
        if (pair) {
          const int xa = 2 * j - lead;
          T ar = T(0), ai = T(0), br = T(0), bi = T(0);
          if (xa >= 0) acc_value<T, typename Acc<T, KAHAN>::type, KAHAN>(srow[xa], ar, ai);
          if (xa + 1 < P0) acc_value<T, typename Acc<T, KAHAN>::type, KAHAN>(srow[xa + 1], br, bi);
          if (ar != T(0) || ai != T(0) || br != T(0) || bi != T(0)) {
            const int gx = small ? wrap_any(x0 + xa, Nt0) : wrap_once(x0 + xa, Nt0);
            atomicAdd(reinterpret_cast<float4*>(grow + 2 * gx), make_float4(ar, ai, br, bi));
          }
          continue;
        }
      }
      T vr, vi;
      acc_value<T, typename Acc<T, KAHAN>::type, KAHAN>(srow[j], vr, vi);
      if (vr != T(0) || vi != T(0)) {
        const int gx = small ? wrap_any(x0 + j, Nt0) : wrap_once(x0 + j, Nt0);
        red_add2<T>(grow + 2 * gx, vr, vi);
      }
    }
    y += step;
    while (y >= P1) {
      y -= P1;
      ++z;
    }
  }
}

template <typename A, typename T> __device__ __forceinline__ void acc_add(A& a, T vr, T vi);
template <> __device__ __forceinline__ void acc_add<float2, float>(float2& a, float vr, float vi) {
  a.x += vr;
  a.y += vi;
}
template <> __device__ __forceinline__ void acc_add<double2, double>(double2& a, double vr, double vi) {
  a.x += vr;
  a.y += vi;
}
template <typename A, typename T> __device__ __forceinline__ void kahan_add(A& a, T vr, T vi) {
  // Kahan: y = v - c; t = s + y; c = (t - s) - y; s = t
  const T yr = vr - a.z, yi = vi - a.w;
  const T tr = a.x + yr, ti = a.y + yi;
  a.z = (tr - a.x) - yr;
  a.w = (ti - a.y) - yi;
  a.x = tr;
  a.y = ti;
}

// --------------------------------------------------------------------------
// D >= 2: slice-owned, atomic-free.
//
// OwnedCfg: NZ warp groups own the slices along the last dimension with
// index = group mod NZ.  D = 3: NZ = 8, a slice is an x-y plane of L x L taps,
// lanes = (tap x, row slot), NSTEP steps over the rows; with NY = 2 the CTA
// has 16 warps and warp (group, parity) also owns only the padded rows of one
// parity, so every tile point still has exactly one writer and a warp does
// half the rows of a node (for L = 8 one 32-tap step).  D = 2: NZ = 2, a
// warp's taps of one node are ceil(L/2) rows x L columns, flattened over the
// lanes.  Staging precomputes per node, once per CTA, the complex value times
// the last-dimension window value of every slice (cz) and the products of the
// other window values (wxy), so a warp's per-node work is a few shared loads
// and its read-modify-writes.
template <int D, int L, int NY = 1> struct OwnedCfg {
  static_assert(NY == 1 || (D == 3 && L % 2 == 0), "row-parity ownership needs D = 3");
  static constexpr int NZ = D == 3 ? 8 : 2;
  static constexpr int NW = NZ * NY;
  static constexpr int THREADS = NW * 32;
  static constexpr int KS = (L + NZ - 1) / NZ;              // owned slices per node (max)
  static constexpr int XY = D == 3 ? L * L : L;              // staged products per node
  static constexpr int RY = D == 3 ? 32 / L : 1;             // D = 3 row slots per step
  static constexpr int NSTEP = D == 3 ? (L / NY + RY - 1) / RY : (KS * L + 31) / 32;
};

template <int D, int L, typename T, bool TABLE, bool KAHAN, int NY = 1>
__device__ __forceinline__ void spread_owned_body(const Geom<T>& G, const Nodes<T>& Nd, const int4 task,
                                                  const typename Cplx<T>::type* __restrict__ fsorted,
                                                  T* __restrict__ g, int pitch) {
  static_assert(D >= 2, "slice ownership needs D >= 2");
  using C = typename Cplx<T>::type;
  using A = typename Acc<T, KAHAN>::type;
  using CF = OwnedCfg<D, L, NY>;
  constexpr int DL = D * L;
  constexpr int DEG = L + 1;
  constexpr int NB = kStageNodes;
  constexpr int WPT = (NB * DL + CF::THREADS - 1) / CF::THREADS;  // staged window values per thread
  extern __shared__ __align__(32) unsigned char smem_raw[];
  const int tile = task.x;
  const int tc0 = tile % G.ntiles[0];
  const int tc1 = (tile / G.ntiles[0]) % G.ntiles[1];
  const int tc2 = tile / (G.ntiles[0] * G.ntiles[1]);
  const int P0 = G.bs[0] + L - 1;
  const int P1 = G.bs[1] + L - 1;
  const int P2 = D == 3 ? G.bs[2] + L - 1 : 1;
  const int o0 = tc0 * G.bs[0], o1 = tc1 * G.bs[1], o2 = D == 3 ? tc2 * G.bs[2] : 0;
  const int plane = pitch * P1;
  const int nacc = plane * P2;
  const int slice_stride = D == 3 ? plane : pitch;
  A* acc = reinterpret_cast<A*>(smem_raw);
  int2* s_meta = reinterpret_cast<int2*>(smem_raw + ((size_t(nacc) * sizeof(A) + 31) & ~size_t(31)));
  C* s_cz = reinterpret_cast<C*>(s_meta + NB);   // [NB][L]: value x last-dimension window value
  C* s_c = s_cz + NB * L;                        // [NB]
  T* s_w = reinterpret_cast<T*>(s_c + NB);       // [NB][DL]
  T* s_xy = s_w + NB * DL;                       // [NB][XY]
  {
    A zero;
    memset(&zero, 0, sizeof(A));
    for (int q = threadIdx.x; q < nacc; q += blockDim.x) acc[q] = zero;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wz = warp % CF::NZ, wy = warp / CF::NZ;  // slice group, row parity (NY = 2)
  // static per-lane tap pattern: product index and shared offset of each step
  // (rows NY apart; the node's row parity adds one row for NY = 2)
  int xy_idx[CF::NSTEP], lofs[CF::NSTEP], kslice[CF::NSTEP];
  bool act[CF::NSTEP];
#pragma unroll
  for (int st = 0; st < CF::NSTEP; ++st) {
    if constexpr (D == 3) {
      const int ix = lane % L, rr = st * CF::RY + lane / L;
      act[st] = (lane / L) < CF::RY && rr < L / NY;
      const int iyc = act[st] ? NY * rr : 0;
      xy_idx[st] = iyc * L + ix;
      lofs[st] = iyc * pitch + ix;
      kslice[st] = 0;
    } else {
      const int item = lane + 32 * st;
      const int k = item / L, ix = item % L;
      act[st] = k < CF::KS;
      xy_idx[st] = ix;
      lofs[st] = ix;
      kslice[st] = act[st] ? k : 0;
    }
  }

  // register prefetch of one batch: node, value (bin-sorted order), window
  // values (or fractional offsets for the polynomial)
  int4 r_nd = make_int4(0, 0, 0, 0);
  C r_c;
  T r_w[WPT];
  auto prefetch = [&](int b) {
    const int n = min(NB, task.z - b);
    if (threadIdx.x < n) {
      r_nd = __ldg(Nd.node4 + b + threadIdx.x);
      r_c = __ldg(fsorted + b + threadIdx.x);
    }
#pragma unroll
    for (int u = 0; u < WPT; ++u) {
      const int q = threadIdx.x + u * CF::THREADS;
      if (q < n * DL) {
        const int s = q / DL, r = q - s * DL;
        if constexpr (TABLE) r_w[u] = __ldg(Nd.wtab + int64_t(b + s) * DL + r);
        else r_w[u] = __ldg(Nd.frac4 + 4 * int64_t(b + s) + r / L);
      }
    }
  };
  if (task.y < task.z) prefetch(task.y);
  __syncthreads();

  for (int b = task.y; b < task.z; b += NB) {
    const int n = min(NB, task.z - b);
    // stage 1: registers -> shared (window values evaluated here for POLYNOMIAL)
    if (threadIdx.x < n) {
      const int px = r_nd.x - o0, py = r_nd.y - o1;
      s_meta[threadIdx.x] = D == 3 ? make_int2((r_nd.z - o2) | ((py & 1) << 8), py * pitch + px) : make_int2(py, px);
      s_c[threadIdx.x] = r_c;
    }
#pragma unroll
    for (int u = 0; u < WPT; ++u) {
      const int q = threadIdx.x + u * CF::THREADS;
      if (q < n * DL) {
        T w = r_w[u];
        if constexpr (!TABLE) {
          const int l = (q % DL) % L;
          const T t = w - T(0.5);
          const T* c = G.coeffs + l * DEG;
          w = __ldg(c + DEG - 1);
#pragma unroll
          for (int i = DEG - 2; i >= 0; --i) w = fma(w, t, __ldg(c + i));
        }
        s_w[q] = w;
      }
    }
    __syncthreads();
    // stage 2: per-slice values, then tap products (two uniform loops over
    // contiguous items: no divergence between the two kinds of item)
    for (int q = threadIdx.x; q < n * L; q += blockDim.x) {
      const int s = q / L, r = q - s * L;
      const T wl = s_w[s * DL + (D - 1) * L + r];
      const C c = s_c[s];
      C v;
      v.x = c.x * wl;
      v.y = c.y * wl;
      s_cz[q] = v;
    }
    for (int q = threadIdx.x; q < n * CF::XY; q += blockDim.x) {
      const int s = q / CF::XY, u = q - s * CF::XY;
      if constexpr (D == 3) {
        const int iy = u / L, jx = u - iy * L;
        s_xy[q] = s_w[s * DL + jx] * s_w[s * DL + L + iy];
      } else {
        s_xy[q] = s_w[s * DL + u];
      }
    }
    __syncthreads();
    // the next batch's global loads overlap the spreading of this one
    if (b + NB < task.z) prefetch(b + NB);
    // Node s+1's slice offset and values are loaded while node s's taps run
    // (software pipeline), and all of a node's accumulator loads are issued
    // before its stores: one node's taps hit distinct points of the slices.
    const T* xy = s_xy;
    if constexpr (D == 3) {
      int so_c, xo_c;
      C cz_c[CF::KS];
      bool ok_c[CF::KS];
      // slice offset, row-parity offset of the products, and slice values of node s
      auto load_node = [&](int s, int& so, int& xo, C(&cz)[CF::KS], bool(&ok)[CF::KS]) {
        const int2 meta = s_meta[s];
        const int pz = meta.x & 0xFF;
        const int is0 = (wz - pz) & (CF::NZ - 1);
        const int par = NY == 2 ? ((wy - (meta.x >> 8)) & 1) : 0;  // first owned row of the window
        so = (pz + is0) * slice_stride + meta.y + par * pitch;
        xo = par * L;
#pragma unroll
        for (int k = 0; k < CF::KS; ++k) {
          const int is = is0 + k * CF::NZ;
          ok[k] = is < L;
          cz[k] = s_cz[s * L + (ok[k] ? is : 0)];
        }
      };
      load_node(0, so_c, xo_c, cz_c, ok_c);
      for (int s = 0; s < n; ++s, xy += CF::XY) {
        int so_n, xo_n;
        C cz_n[CF::KS];
        bool ok_n[CF::KS];
        load_node(s + 1 < n ? s + 1 : s, so_n, xo_n, cz_n, ok_n);
#pragma unroll
        for (int k = 0; k < CF::KS; ++k) {
          if (ok_c[k]) {
            const int so = so_c + k * CF::NZ * slice_stride;
            A a[CF::NSTEP];
            T w[CF::NSTEP];
#pragma unroll
            for (int st = 0; st < CF::NSTEP; ++st) {
              if (act[st]) {
                a[st] = acc[so + lofs[st]];
                w[st] = xy[xo_c + xy_idx[st]];
              }
            }
#pragma unroll
            for (int st = 0; st < CF::NSTEP; ++st) {
              if (act[st]) {
                if constexpr (KAHAN) kahan_add<A, T>(a[st], cz_c[k].x * w[st], cz_c[k].y * w[st]);
                else acc_add<A, T>(a[st], cz_c[k].x * w[st], cz_c[k].y * w[st]);
                acc[so + lofs[st]] = a[st];
              }
            }
          }
        }
        so_c = so_n;
        xo_c = xo_n;
#pragma unroll
        for (int k = 0; k < CF::KS; ++k) {
          cz_c[k] = cz_n[k];
          ok_c[k] = ok_n[k];
        }
      }
    } else {
      int2 meta_c = s_meta[0];
      for (int s = 0; s < n; ++s, xy += CF::XY) {
        const int2 meta_n = s_meta[s + 1 < n ? s + 1 : s];
        const int is0 = (wz - meta_c.x) & (CF::NZ - 1);
        A a[CF::NSTEP];
        T w[CF::NSTEP];
        C cz[CF::NSTEP];
        int off[CF::NSTEP];
        bool ok[CF::NSTEP];
#pragma unroll
        for (int st = 0; st < CF::NSTEP; ++st) {
          const int is = is0 + kslice[st] * CF::NZ;
          ok[st] = act[st] && is < L;
          if (ok[st]) {
            off[st] = (meta_c.x + is) * slice_stride + meta_c.y + lofs[st];
            a[st] = acc[off[st]];
            w[st] = xy[xy_idx[st]];
            cz[st] = s_cz[s * L + is];
          }
        }
#pragma unroll
        for (int st = 0; st < CF::NSTEP; ++st) {
          if (ok[st]) {
            if constexpr (KAHAN) kahan_add<A, T>(a[st], cz[st].x * w[st], cz[st].y * w[st]);
            else acc_add<A, T>(a[st], cz[st].x * w[st], cz[st].y * w[st]);
            acc[off[st]] = a[st];
          }
        }
        meta_c = meta_n;
      }
    }
    __syncthreads();
  }

  // (the batch loop ends with a barrier: the tile is complete)
  flush_tile<D, T, KAHAN, CF::NW>(G, acc, g, o0, o1, o2, P0, P1, P2, pitch);
}

template <int D, int L, typename T, bool TABLE, bool KAHAN, int NY = 1>
__global__ void __launch_bounds__(OwnedCfg<D, L, NY>::THREADS) spread_owned_kernel(Geom<T> G, Nodes<T> Nd,
                                                                               const int4* __restrict__ tasks,
                                                                               const typename Cplx<T>::type* __restrict__ fsorted,
                                                                               T* __restrict__ g, int pitch,
                                                                               int64_t fcol = 0, int64_t gcol = 0) {
  // blockIdx.y: column of a multi-column launch (values fsorted + y fcol, grid g + y gcol)
  spread_owned_body<D, L, T, TABLE, KAHAN, NY>(G, Nd, tasks[blockIdx.x], fsorted + blockIdx.y * fcol,
                                               g + blockIdx.y * gcol, pitch);
}

// --------------------------------------------------------------------------
// D = 1: 32/G nodes per warp, shared-memory atomics into the padded row.
template <int L, typename T, bool TABLE>
__global__ void __launch_bounds__(kSpreadThreads) spread_pad1_kernel(Geom<T> G, Nodes<T> Nd,
                                                                      const int4* __restrict__ tasks,
                                                                      const typename Cplx<T>::type* __restrict__ fhat,
                                                                      T* __restrict__ g, int64_t fcol = 0,
                                                                      int64_t gcol = 0) {
  using C = typename Cplx<T>::type;
  using LN = Lanes<1, L>;
  extern __shared__ __align__(32) unsigned char smem_raw[];
  fhat += blockIdx.y * fcol;  // column of a multi-column launch
  g += blockIdx.y * gcol;
  const int4 task = tasks[blockIdx.x];
  const int o0 = task.x * G.bs[0];
  const int P0 = G.bs[0] + L - 1;
  T* sre = reinterpret_cast<T*>(smem_raw);
  T* sim = sre + P0;
  for (int q = threadIdx.x; q < P0; q += blockDim.x) {
    sre[q] = T(0);
    sim[q] = T(0);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slot = lane / LN::G1, ix = lane % LN::G1;
  const bool act = ix < L;
  T c[LN::DEG];
  if constexpr (!TABLE) {
#pragma unroll
    for (int q = 0; q < LN::DEG; ++q) c[q] = act ? __ldg(G.coeffs + ix * LN::DEG + q) : T(0);
  }
  __syncthreads();
  for (int b = task.y + warp * LN::NPW; b < task.z; b += kSpreadWarps * LN::NPW) {
    const int i = b + slot;
    if (i < task.z && act) {
      const int4 nd = __ldg(Nd.node4 + i);
      T w;
      if constexpr (TABLE) {
        w = __ldg(Nd.wtab + int64_t(i) * L + ix);
      } else {
        const T t = __ldg(Nd.frac4 + 4 * int64_t(i)) - T(0.5);
        w = c[LN::DEG - 1];
#pragma unroll
        for (int q = LN::DEG - 2; q >= 0; --q) w = fma(w, t, c[q]);
      }
      const C v = __ldg(fhat + nd.w);
      const int px = nd.x - o0 + ix;
      atomicAdd(sre + px, w * v.x);
      atomicAdd(sim + px, w * v.y);
    }
  }
  __syncthreads();
  const int m1 = G.m - 1;
  const bool small = G.small_grid;
  for (int x = threadIdx.x; x < P0; x += blockDim.x) {
    const T a = sre[x], bb = sim[x];
    if (a != T(0) || bb != T(0)) {
      const int gx = small ? wrap_any(o0 + G.sh[0] - m1 + x, G.Nt[0]) : wrap_once(o0 + G.sh[0] - m1 + x, G.Nt[0]);
      red_add2<T>(g + 2 * int64_t(gx), a, bb);
    }
  }
}

// D = 1, compensated (compensated = 1): one warp per task; lane l owns the
// padded positions x = l mod 32, so each of a node's L <= 16 taps has exactly
// one owner lane and the Kahan read-modify-write needs no atomics.  Nodes are
// visited in bin-sorted order (input order within a tile) in batches of 32:
// lane l loads node b + l's position and value (broadcast by shuffles) and
// the batch's window values go to shared memory, the next batch being
// loaded while the current one is added.
template <int L, typename T, bool TABLE>
__global__ void __launch_bounds__(32) spread_line_kahan_kernel(Geom<T> G, Nodes<T> Nd, const int4* __restrict__ tasks,
                                                                const typename Cplx<T>::type* __restrict__ fhat,
                                                                T* __restrict__ g) {
  using C = typename Cplx<T>::type;
  using A = typename Acc<T, true>::type;
  constexpr int DEG = L + 1;
  static_assert(L <= 32, "one owner lane per tap");
  extern __shared__ __align__(32) unsigned char smem_raw[];
  A* acc = reinterpret_cast<A*>(smem_raw);
  const int4 task = tasks[blockIdx.x];
  const int o0 = task.x * G.bs[0];
  const int P0 = G.bs[0] + L - 1;
  // window values of two batches (double buffer) and, POLYNOMIAL, the coefficients
  T* s_w = reinterpret_cast<T*>(smem_raw + ((size_t(P0) * sizeof(A) + 31) & ~size_t(31)));
  T* s_coef = s_w + 2 * 32 * L;
  const int lane = threadIdx.x;
  {
    A zero;
    memset(&zero, 0, sizeof(A));
    for (int q = lane; q < P0; q += 32) acc[q] = zero;
    if constexpr (!TABLE)
      for (int q = lane; q < L * DEG; q += 32) s_coef[q] = __ldg(G.coeffs + q);
  }
  __syncwarp();
  // batch loads: lane l holds node b + l's padded position and value; the
  // window values of the batch land in s_w[buf]
  auto load = [&](int b, int buf, int& x0, C& v) {
    const int n = min(32, task.z - b);
    x0 = 0;
    v.x = T(0);
    v.y = T(0);
    T fr = T(0);
    if (lane < n) {
      const int4 nd = __ldg(Nd.node4 + b + lane);
      x0 = nd.x - o0;
      v = __ldg(fhat + nd.w);
      if constexpr (!TABLE) fr = __ldg(Nd.frac4 + 4 * int64_t(b + lane));
    }
    T* w = s_w + buf * 32 * L;
    if constexpr (TABLE) {
      for (int q = lane; q < n * L; q += 32) w[q] = __ldg(Nd.wtab + int64_t(b) * L + q);
    } else {
      // lane l evaluates the L window values of node b + l
      const T t = fr - T(0.5);
      if (lane < n) {
#pragma unroll
        for (int l = 0; l < L; ++l) {
          const T* c = s_coef + l * DEG;
          T r = c[DEG - 1];
#pragma unroll
          for (int q = DEG - 2; q >= 0; --q) r = fma(r, t, c[q]);
          w[lane * L + l] = r;
        }
      }
    }
  };
  if (task.y < task.z) {
    int x0c, x0n = 0;
    C vc, vn;
    load(task.y, 0, x0c, vc);
    int buf = 0;
    for (int b = task.y; b < task.z; b += 32, buf ^= 1) {
      const int n = min(32, task.z - b);
      if (b + 32 < task.z) load(b + 32, buf ^ 1, x0n, vn);
      __syncwarp();
      const T* w = s_w + buf * 32 * L;
      for (int s = 0; s < n; ++s) {
        const int x0 = __shfl_sync(0xFFFFFFFFu, x0c, s);
        const T vr = __shfl_sync(0xFFFFFFFFu, vc.x, s), vi = __shfl_sync(0xFFFFFFFFu, vc.y, s);
        const int t = (lane - x0) & 31;
        if (t < L) {
          const T wt = w[s * L + t];
          kahan_add<A, T>(acc[x0 + t], wt * vr, wt * vi);
        }
      }
      __syncwarp();
      x0c = x0n;
      vc = vn;
    }
  }
  __syncwarp();
  flush_tile<1, T, true, 1>(G, acc, g, o0, 0, 0, P0, 1, 1, P0);
}

template <int D, int L, typename T>
size_t owned_smem(const nfft_plan* p, bool kahan) {
  const int P1 = int(p->bs[1]) + L - 1;
  const int P2 = D == 3 ? int(p->bs[2]) + L - 1 : 1;
  const size_t acc = ((kahan ? 4 : 2) * sizeof(T) * size_t(p->spread_pitch) * P1 * P2 + 31) & ~size_t(31);
  const size_t stage = kStageNodes * (sizeof(int2) + 2 * sizeof(T) * (L + 1) +
                                      sizeof(T) * (D * L + OwnedCfg<D, L>::XY));
  return acc + stage;
}

}  // namespace
}  // namespace nfft
