// Spreading (convolve_transpose!): g[tap] += prod_d phi_d * fHat[j] over the
// (2m)^D window taps of every node, src/convolution.jl:349-520.
//
// The GB300 form of NFFT.jl's blocked adjoint (private padded block per
// block, then a locked wrap-add into g, :356-443):
//   * nodes are bin-sorted by home tile (bs[0] x bs[1] x bs[2] grid points);
//     one CTA per task = one home tile or a chunk of a hot tile;
//   * the CTA accumulates into the tile padded by 2m-1 points in shared
//     memory (re and im planes, row pitch chosen so that the lanes of one
//     warp step hit distinct banks), so every tap of every node lands inside
//     it: no per-tap bounds tests and no wrap-around in the hot loop;
//   * a warp spreads one node at a time (32/G nodes for D = 1) with shared-
//     memory atomics, window values shuffled between lanes;
//   * the padded tile is added to the zeroed grid with vector global atomics
//     (red.global.add.v2), wrapping periodically; all-zero points are skipped.
// The lock of the reference becomes the L2 atomics of the flush.
#include "warpnode.cuh"

namespace nfft {
namespace {

constexpr int kSpreadThreads = 256;

template <typename T> __device__ __forceinline__ void red_add2(T* g, T x, T y);
template <> __device__ __forceinline__ void red_add2<float>(float* g, float x, float y) {
  atomicAdd(reinterpret_cast<float2*>(g), make_float2(x, y));
}
template <> __device__ __forceinline__ void red_add2<double>(double* g, double x, double y) {
  atomicAdd(g, x);
  atomicAdd(g + 1, y);
}

template <int D, int L, typename T, bool TABLE>
__global__ void __launch_bounds__(kSpreadThreads) spread_pad_kernel(Geom<T> G, Nodes<T> Nd,
                                                                     const int4* __restrict__ tasks,
                                                                     const typename Cplx<T>::type* __restrict__ fhat,
                                                                     T* __restrict__ g, int pitch) {
  using C = typename Cplx<T>::type;
  using LN = Lanes<D, L>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int4 task = tasks[blockIdx.x];
  const int tile = task.x;
  const int tc0 = tile % G.ntiles[0];
  const int tc1 = (tile / G.ntiles[0]) % G.ntiles[1];
  const int tc2 = tile / (G.ntiles[0] * G.ntiles[1]);
  // padded extents and origin (grid coordinate of padded index 0)
  const int P0 = G.bs[0] + L - 1;
  const int P1 = D >= 2 ? G.bs[1] + L - 1 : 1;
  const int P2 = D >= 3 ? G.bs[2] + L - 1 : 1;
  const int o0 = tc0 * G.bs[0], o1 = tc1 * G.bs[1], o2 = tc2 * G.bs[2];
  const int plane = pitch * P1;
  const int nwords = plane * P2;
  T* sre = reinterpret_cast<T*>(smem_raw);
  T* sim = sre + nwords;
  for (int q = threadIdx.x; q < nwords; q += blockDim.x) {
    sre[q] = T(0);
    sim[q] = T(0);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
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
        const int px = nd.x - o0 + ix;  // padded index of this tap
        atomicAdd(sre + px, w * v.x);
        atomicAdd(sim + px, w * v.y);
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
      const C v = __ldg(fhat + nd.w);
      const T wx = wsel<D, L>(W, ix);
      const T cr = v.x * wx, ci = v.y * wx;
      const int px = nd.x - o0 + ix;
      const int py0 = nd.y - o1;
      int base[LN::NSTEP];
      T vr[LN::NSTEP], vi[LN::NSTEP];
      bool ok[LN::NSTEP];
#pragma unroll
      for (int s = 0; s < LN::NSTEP; ++s) {
        const int iy = s * LN::RY + ry;
        ok[s] = xact && iy < L;
        const int iyc = ok[s] ? iy : 0;
        const T wy = wsel<D, L>(W, L + iyc);  // every lane shuffles
        base[s] = px + pitch * (py0 + iyc);
        vr[s] = cr * wy;
        vi[s] = ci * wy;
      }
      if constexpr (D == 2) {
#pragma unroll
        for (int s = 0; s < LN::NSTEP; ++s) {
          if (ok[s]) {
            atomicAdd(sre + base[s], vr[s]);
            atomicAdd(sim + base[s], vi[s]);
          }
        }
      } else {
        const int pz0 = (nd.z - o2) * plane;
#pragma unroll
        for (int iz = 0; iz < L; ++iz) {
          const T wz = wsel<D, L>(W, 2 * L + iz);
          const int pz = pz0 + iz * plane;
#pragma unroll
          for (int s = 0; s < LN::NSTEP; ++s) {
            if (ok[s]) {
              atomicAdd(sre + pz + base[s], vr[s] * wz);
              atomicAdd(sim + pz + base[s], vi[s] * wz);
            }
          }
        }
      }
    }
  }
  __syncthreads();

  // flush: padded point (x, y, z) -> grid ((o - m + 1 + x) mod Ntilde, ...)
  const int m1 = G.m - 1;
  const bool small = G.small_grid;
  const int rows = P1 * P2;
  for (int r = warp; r < rows; r += nwarps) {
    const int y = r % P1, z = r / P1;
    const int gy = D >= 2 ? (small ? wrap_any(o1 - m1 + y, G.Nt[1]) : wrap_once(o1 - m1 + y, G.Nt[1])) : 0;
    const int gz = D >= 3 ? (small ? wrap_any(o2 - m1 + z, G.Nt[2]) : wrap_once(o2 - m1 + z, G.Nt[2])) : 0;
    T* grow = g + 2 * (int64_t(gz) * G.plane + int64_t(gy) * G.Nt[0]);
    const int srow = z * plane + y * pitch;
    for (int x = lane; x < P0; x += 32) {
      const T a = sre[srow + x], b = sim[srow + x];
      if (a != T(0) || b != T(0)) {
        const int gx = small ? wrap_any(o0 - m1 + x, G.Nt[0]) : wrap_once(o0 - m1 + x, G.Nt[0]);
        red_add2<T>(grow + 2 * gx, a, b);
      }
    }
  }
}

// Compensated variant: warp w owns the slices of the padded tile along the
// last dimension whose index is w mod (number of warps); a slice is an x-y
// plane (D = 3), an x row (D = 2) or a point (D = 1).  Every point then has
// one writer, which adds the node contributions in node order with Kahan
// compensation (sum and compensation kept in shared memory).
template <int D, int L, typename T, bool TABLE>
__global__ void __launch_bounds__(kSpreadThreads) spread_kahan_kernel(Geom<T> G, Nodes<T> Nd,
                                                                       const int4* __restrict__ tasks,
                                                                       const typename Cplx<T>::type* __restrict__ fhat,
                                                                       T* __restrict__ g, int pitch) {
  using C = typename Cplx<T>::type;
  using LN = Lanes<D, L>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int4 task = tasks[blockIdx.x];
  const int tile = task.x;
  const int tc0 = tile % G.ntiles[0];
  const int tc1 = (tile / G.ntiles[0]) % G.ntiles[1];
  const int tc2 = tile / (G.ntiles[0] * G.ntiles[1]);
  const int P0 = G.bs[0] + L - 1;
  const int P1 = D >= 2 ? G.bs[1] + L - 1 : 1;
  const int P2 = D >= 3 ? G.bs[2] + L - 1 : 1;
  const int o0 = tc0 * G.bs[0], o1 = tc1 * G.bs[1], o2 = tc2 * G.bs[2];
  const int plane = pitch * P1;
  const int nwords = plane * P2;
  T* sre = reinterpret_cast<T*>(smem_raw);
  T* sim = sre + nwords;
  T* cre = sim + nwords;
  T* cim = cre + nwords;
  for (int q = threadIdx.x; q < 4 * nwords; q += blockDim.x) sre[q] = T(0);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  __syncthreads();
  PolyRegs<D, L, T> P;
  if constexpr (!TABLE) P.load(G.coeffs, lane);
  // lane layout inside a slice
  const int ix = D == 1 ? 0 : lane % L;
  const int ry = D == 3 ? lane / L : 0;
  const bool xact = D == 1 ? lane == 0 : (D == 2 ? lane < L : ry < LN::RY);
  constexpr int NST = D == 3 ? LN::NSTEP : 1;
  auto kahan = [](T* s, T* c, int idx, T v) {
    const T y = v - c[idx];
    const T t = s[idx] + y;
    c[idx] = (t - s[idx]) - y;
    s[idx] = t;
  };
  for (int i = task.y; i < task.z; ++i) {
    const int4 nd = __ldg(Nd.node4 + i);
    const int tlast = D == 3 ? nd.z - o2 : (D == 2 ? nd.y - o1 : nd.x - o0);
    // first of this node's slices owned by this warp
    int is = (warp - tlast) % nwarps;
    if (is < 0) is += nwarps;
    if (is >= L) continue;  // uniform per warp: no slice of this node is owned
    T W[LN::NW];
    node_weights<D, L, T, TABLE>(Nd, P, i, lane, W);
    const C v = __ldg(fhat + nd.w);
    for (; is < L; is += nwarps) {
      const T wl = wsel<D, L>(W, (D - 1) * L + is);
      const T br = v.x * wl, bi = v.y * wl;
      if constexpr (D == 1) {
        if (lane == 0) kahan(sre, cre, tlast + is, br), kahan(sim, cim, tlast + is, bi);
      } else if constexpr (D == 2) {
        const T wx = wsel<D, L>(W, ix);
        const int idx = (nd.y - o1 + is) * pitch + (nd.x - o0 + ix);
        if (xact) kahan(sre, cre, idx, br * wx), kahan(sim, cim, idx, bi * wx);
      } else {
        const T wx = wsel<D, L>(W, ix);
        const int pz = (nd.z - o2 + is) * plane;
#pragma unroll
        for (int s = 0; s < NST; ++s) {
          const int iy = s * LN::RY + ry;
          const bool ok = xact && iy < L;
          const int iyc = ok ? iy : 0;
          const T wy = wsel<D, L>(W, L + iyc);
          const int idx = pz + (nd.y - o1 + iyc) * pitch + (nd.x - o0 + ix);
          if (ok) kahan(sre, cre, idx, br * wx * wy), kahan(sim, cim, idx, bi * wx * wy);
        }
      }
    }
  }
  __syncthreads();
  const int m1 = G.m - 1;
  const bool small = G.small_grid;
  const int rows = P1 * P2;
  for (int r = warp; r < rows; r += nwarps) {
    const int y = r % P1, z = r / P1;
    const int gy = D >= 2 ? (small ? wrap_any(o1 - m1 + y, G.Nt[1]) : wrap_once(o1 - m1 + y, G.Nt[1])) : 0;
    const int gz = D >= 3 ? (small ? wrap_any(o2 - m1 + z, G.Nt[2]) : wrap_once(o2 - m1 + z, G.Nt[2])) : 0;
    T* grow = g + 2 * (int64_t(gz) * G.plane + int64_t(gy) * G.Nt[0]);
    const int srow = z * plane + y * pitch;
    for (int x = lane; x < P0; x += 32) {
      const T a = sre[srow + x] - cre[srow + x], b = sim[srow + x] - cim[srow + x];
      if (a != T(0) || b != T(0)) {
        const int gx = small ? wrap_any(o0 - m1 + x, G.Nt[0]) : wrap_once(o0 - m1 + x, G.Nt[0]);
        red_add2<T>(grow + 2 * gx, a, b);
      }
    }
  }
}

template <int D, int L, typename T>
int spread_launch(nfft_plan* p, const void* fhat, void* g) {
  Geom<T> G = make_geom<T>(p);
  Nodes<T> Nd = make_nodes<T>(p);
  const size_t gbytes = size_t(p->Nt[0] * p->Nt[1] * p->Nt[2]) * sizeof(T) * 2;
  NFFT_CUDA_TRY(cudaMemsetAsync(g, 0, gbytes, p->stream));
  if (p->n_tasks == 0) return NFFT_OK;
  const int P1 = D >= 2 ? int(p->bs[1]) + L - 1 : 1;
  const int P2 = D >= 3 ? int(p->bs[2]) + L - 1 : 1;
  const bool comp = p->prm.compensated != 0;
  const size_t smem = size_t(comp ? 4 : 2) * sizeof(T) * size_t(p->spread_pitch) * P1 * P2;
  if (smem > 227 * 1024) {
    set_error("padded spreading tile (%zu bytes) does not fit in shared memory; use a smaller blockSize", smem);
    return NFFT_ERR_UNSUPPORTED;
  }
  auto kern = comp ? (p->wtab ? spread_kahan_kernel<D, L, T, true> : spread_kahan_kernel<D, L, T, false>)
                   : (p->wtab ? spread_pad_kernel<D, L, T, true> : spread_pad_kernel<D, L, T, false>);
  NFFT_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  kern<<<unsigned(p->n_tasks), kSpreadThreads, smem, p->stream>>>(
      G, Nd, p->tasks, static_cast<const typename Cplx<T>::type*>(fhat), static_cast<T*>(g), p->spread_pitch);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

template <int D, typename T> int spread_dispatch_l(nfft_plan* p, const void* fhat, void* g) {
  switch (p->m) {
    case 2: return spread_launch<D, 4, T>(p, fhat, g);
    case 3: return spread_launch<D, 6, T>(p, fhat, g);
    case 4: return spread_launch<D, 8, T>(p, fhat, g);
    case 5: return spread_launch<D, 10, T>(p, fhat, g);
    case 6: return spread_launch<D, 12, T>(p, fhat, g);
    case 7: return spread_launch<D, 14, T>(p, fhat, g);
    case 8: return spread_launch<D, 16, T>(p, fhat, g);
  }
  set_error("m = %d not supported (2..8)", p->m);
  return NFFT_ERR_UNSUPPORTED;
}

template <typename T> int spread_dispatch(nfft_plan* p, const void* fhat, void* g) {
  switch (p->D) {
    case 1: return spread_dispatch_l<1, T>(p, fhat, g);
    case 2: return spread_dispatch_l<2, T>(p, fhat, g);
    case 3: return spread_dispatch_l<3, T>(p, fhat, g);
  }
  return NFFT_ERR_UNSUPPORTED;
}

}  // namespace

// Row pitch (in elements) of the padded tile: the smallest pitch >= the
// padded row length for which the lanes of one warp step (L taps along x
// times RY rows) touch distinct shared-memory banks.
int spread_pitch_for(int D, int m, int P0, int elem_bytes) {
  const int L = 2 * m;
  const int RY = D == 1 ? 1 : 32 / L;
  const int words = elem_bytes / 4;
  for (int pitch = P0; pitch < P0 + 64; ++pitch) {
    int used[32] = {};
    int worst = 0;
    for (int ry = 0; ry < RY; ++ry)
      for (int ix = 0; ix < L; ++ix) {
        const int bank = ((ix + pitch * ry) * words) % 32;
        worst = ++used[bank] > worst ? used[bank] : worst;
      }
    if (worst <= words) return pitch;
  }
  return P0;
}

int launch_spread(nfft_plan* p, const void* fhat, int, void* g, int) {
  return p->precision == 32 ? spread_dispatch<float>(p, fhat, g) : spread_dispatch<double>(p, fhat, g);
}

}  // namespace nfft
