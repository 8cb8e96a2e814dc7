// Spreading (convolve_transpose!): g[tap] += prod_d phi_d * fHat[j] over the
// (2m)^D window taps of every node, src/convolution.jl:349-520.
//
// Owner-computes tiles.  The grid is cut into tiles of bs[0] x bs[1] x bs[2]
// points; nfft_set_nodes lists, for every tile, the (bin-sorted) nodes whose
// window touches it and splits long lists into tasks.  One CTA per task:
//   1. zero the tile accumulator in shared memory;
//   2. stage a batch of nodes: per node and dimension, the 2m window values
//      and the tile-local coordinate of each tap (-1 when the tap falls
//      outside the tile, which also encodes periodic wrap-around);
//   3. each warp spreads whole nodes, lane = (tap along dim 1, row slot),
//      accumulating into the tile with shared-memory atomics;
//   4. write the tile to the grid once with plain coalesced stores (tiles
//      with a single task: no zero fill of the grid and no global atomics),
//      or add it with global atomics (tiles split over several tasks, whose
//      region was zeroed first).
#include "nfft_internal.cuh"

namespace nfft {
namespace {

constexpr int kSpreadThreads = 256;
constexpr int kStage = 32;  // nodes staged per batch

template <int D, int L, typename T>
struct Stage {
  int16_t loc[kStage][D][L];
  T w[kStage][D][L];
  T cr[kStage];
  T ci[kStage];
};

template <int D, int L, typename T>
__device__ __forceinline__ void stage_nodes(const Geom<T>& G, const Nodes<T>& Nd, const T* cs, const int32_t* entries,
                                            int eb, int ee, const int lo[3], const int ext[3], const T* fhat,
                                            Stage<D, L, T>& S) {
  const int n = ee - eb;
  for (int q = threadIdx.x; q < kStage * D * L; q += blockDim.x) {
    const int s = q / (D * L);
    const int r = q - s * (D * L);
    const int d = r / L;
    const int l = r - d * L;
    if (s < n) {
      const int i = entries[eb + s];
      const int t = Nd.ti[int64_t(d) * Nd.M + i];
      const T e = Nd.te[int64_t(d) * Nd.M + i];
      S.w[s][d][l] = tap_weight<T>(G, cs, e, l);
      const int gg = G.small_grid ? wrap_any(t - G.m + 1 + l, G.Nt[d]) : wrap_once(t - G.m + 1 + l, G.Nt[d]);
      const int lc = gg - lo[d];
      S.loc[s][d][l] = int16_t((lc >= 0 && lc < ext[d]) ? lc : -1);
    } else {
      S.w[s][d][l] = T(0);
      S.loc[s][d][l] = -1;
    }
  }
  for (int s = threadIdx.x; s < kStage; s += blockDim.x) {
    if (s < n) {
      const int64_t j = Nd.perm[entries[eb + s]];
      S.cr[s] = fhat[2 * j];
      S.ci[s] = fhat[2 * j + 1];
    } else {
      S.cr[s] = T(0);
      S.ci[s] = T(0);
    }
  }
}

template <int D, int L, typename T>
__global__ void __launch_bounds__(kSpreadThreads) spread_tile_kernel(Geom<T> G, Nodes<T> Nd,
                                                                      const int4* __restrict__ tasks,
                                                                      const int32_t* __restrict__ entries,
                                                                      const T* __restrict__ fhat,
                                                                      T* __restrict__ g) {
  constexpr int RY = (D == 1) ? 1 : (32 / L);
  constexpr int NSTEP = (D == 1) ? 1 : (L + RY - 1) / RY;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T cs[kMaxDeg * kMaxL];
  __shared__ Stage<D, L, T> S;
  const int4 task = tasks[blockIdx.x];
  const int tile = task.x;
  const int tcoord[3] = {tile % G.ntiles[0], (tile / G.ntiles[0]) % G.ntiles[1], tile / (G.ntiles[0] * G.ntiles[1])};
  int lo[3], ext[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    lo[d] = tcoord[d] * G.bs[d];
    ext[d] = min(G.bs[d], G.Nt[d] - lo[d]);
  }
  const int bs0 = G.bs[0], bs01 = G.bs[0] * G.bs[1];
  const int npts = G.bs[0] * G.bs[1] * G.bs[2];
  T* acc_r = reinterpret_cast<T*>(smem_raw);
  T* acc_i = acc_r + npts;
  for (int q = threadIdx.x; q < npts; q += blockDim.x) {
    acc_r[q] = T(0);
    acc_i[q] = T(0);
  }
  if (G.mode == WIN_POLY) {
    const int n = (2 * G.m + 1) * L;
    for (int q = threadIdx.x; q < n; q += blockDim.x) cs[q] = G.coeffs[q];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int ix = lane % L;
  const int ry = lane / L;
  const bool xact = (D == 1) ? (lane < L) : (ry < RY);
  for (int eb = task.y; eb < task.z; eb += kStage) {
    const int ee = min(task.z, eb + kStage);
    stage_nodes<D, L, T>(G, Nd, cs, entries, eb, ee, lo, ext, fhat, S);
    __syncthreads();
    const int n = ee - eb;
    for (int s = warp; s < n; s += nwarps) {
      const int lx = xact ? int(S.loc[s][0][ix]) : -1;
      const T wx = S.w[s][0][ix];
      const T cr = S.cr[s] * wx, ci = S.ci[s] * wx;
      if constexpr (D == 1) {
        if (lx >= 0) {
          atomicAdd(acc_r + lx, cr);
          atomicAdd(acc_i + lx, ci);
        }
      } else {
        int rowoff[NSTEP];
        T vr[NSTEP], vi[NSTEP];
#pragma unroll
        for (int st = 0; st < NSTEP; ++st) {
          const int iy = st * RY + ry;
          const int ly = (lx >= 0 && iy < L) ? int(S.loc[s][1][iy < L ? iy : 0]) : -1;
          const T wy = S.w[s][1][iy < L ? iy : 0];
          rowoff[st] = ly >= 0 ? lx + bs0 * ly : -1;
          vr[st] = cr * wy;
          vi[st] = ci * wy;
        }
        if constexpr (D == 2) {
#pragma unroll
          for (int st = 0; st < NSTEP; ++st) {
            if (rowoff[st] >= 0) {
              atomicAdd(acc_r + rowoff[st], vr[st]);
              atomicAdd(acc_i + rowoff[st], vi[st]);
            }
          }
        } else {
#pragma unroll 2
          for (int iz = 0; iz < L; ++iz) {
            const int lz = S.loc[s][D - 1][iz];
            if (lz < 0) continue;  // uniform across the warp
            const T wz = S.w[s][D - 1][iz];
            const int pz = lz * bs01;
#pragma unroll
            for (int st = 0; st < NSTEP; ++st) {
              if (rowoff[st] >= 0) {
                atomicAdd(acc_r + pz + rowoff[st], vr[st] * wz);
                atomicAdd(acc_i + pz + rowoff[st], vi[st] * wz);
              }
            }
          }
        }
      }
    }
    __syncthreads();
  }
  // write the tile once
  const bool multi = task.w != 0;
  for (int q = threadIdx.x; q < npts; q += blockDim.x) {
    const int x = q % G.bs[0];
    const int y = (q / G.bs[0]) % G.bs[1];
    const int z = q / bs01;
    if (x >= ext[0] || y >= ext[1] || z >= ext[2]) continue;
    const int64_t gi = int64_t(lo[0] + x) + int64_t(G.Nt[0]) * (int64_t(lo[1] + y) + int64_t(G.Nt[1]) * (lo[2] + z));
    using C = typename Cplx<T>::type;
    C v;
    v.x = acc_r[q];
    v.y = acc_i[q];
    if (multi) {
      atomicAdd(g + 2 * gi, v.x);
      atomicAdd(g + 2 * gi + 1, v.y);
    } else {
      reinterpret_cast<C*>(g)[gi] = v;
    }
  }
}

// Zero the tiles that several tasks add into.
template <typename T>
__global__ void zero_tiles_kernel(Geom<T> G, const int32_t* __restrict__ tiles, T* __restrict__ g) {
  const int tile = tiles[blockIdx.x];
  const int tc[3] = {tile % G.ntiles[0], (tile / G.ntiles[0]) % G.ntiles[1], tile / (G.ntiles[0] * G.ntiles[1])};
  int lo[3], ext[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = tc[d] * G.bs[d];
    ext[d] = min(G.bs[d], G.Nt[d] - lo[d]);
  }
  const int npts = ext[0] * ext[1] * ext[2];
  for (int q = threadIdx.x; q < npts; q += blockDim.x) {
    const int x = q % ext[0];
    const int y = (q / ext[0]) % ext[1];
    const int z = q / (ext[0] * ext[1]);
    const int64_t gi = int64_t(lo[0] + x) + int64_t(G.Nt[0]) * (int64_t(lo[1] + y) + int64_t(G.Nt[1]) * (lo[2] + z));
    g[2 * gi] = T(0);
    g[2 * gi + 1] = T(0);
  }
}

template <int D, int L, typename T>
int spread_launch(nfft_plan* p, const void* fhat, void* g) {
  Geom<T> G = make_geom<T>(p);
  Nodes<T> Nd = make_nodes<T>(p);
  const size_t smem = size_t(2) * sizeof(T) * size_t(p->bs[0] * p->bs[1] * p->bs[2]);
  auto kern = spread_tile_kernel<D, L, T>;
  const size_t static_smem = sizeof(Stage<D, L, T>) + sizeof(T) * kMaxDeg * kMaxL;
  if (smem + static_smem > 227 * 1024) {
    set_error("spreading tile of %lld points does not fit in shared memory",
              (long long)(p->bs[0] * p->bs[1] * p->bs[2]));
    return NFFT_ERR_UNSUPPORTED;
  }
  NFFT_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  if (p->n_multi > 0) {
    zero_tiles_kernel<T><<<unsigned(p->n_multi), 256, 0, p->stream>>>(G, p->multi_tiles, static_cast<T*>(g));
    NFFT_LAUNCH_CHECK();
  }
  if (p->n_tasks > 0) {
    kern<<<unsigned(p->n_tasks), kSpreadThreads, smem, p->stream>>>(G, Nd, p->tasks, p->entries,
                                                                   static_cast<const T*>(fhat), static_cast<T*>(g));
    NFFT_LAUNCH_CHECK();
  }
  return NFFT_OK;
}

template <int D, int L, typename T>
int spread_dispatch_c(nfft_plan* p, const void* fhat, int, void* g, int) {
  return spread_launch<D, L, T>(p, fhat, g);
}

template <int D, typename T> int spread_dispatch_l(nfft_plan* p, const void* fhat, int fr, void* g, int gr) {
  switch (p->m) {
    case 2: return spread_dispatch_c<D, 4, T>(p, fhat, fr, g, gr);
    case 3: return spread_dispatch_c<D, 6, T>(p, fhat, fr, g, gr);
    case 4: return spread_dispatch_c<D, 8, T>(p, fhat, fr, g, gr);
    case 5: return spread_dispatch_c<D, 10, T>(p, fhat, fr, g, gr);
    case 6: return spread_dispatch_c<D, 12, T>(p, fhat, fr, g, gr);
    case 7: return spread_dispatch_c<D, 14, T>(p, fhat, fr, g, gr);
    case 8: return spread_dispatch_c<D, 16, T>(p, fhat, fr, g, gr);
  }
  set_error("m = %d not supported (2..8)", p->m);
  return NFFT_ERR_UNSUPPORTED;
}

template <typename T> int spread_dispatch(nfft_plan* p, const void* fhat, int fr, void* g, int gr) {
  switch (p->D) {
    case 1: return spread_dispatch_l<1, T>(p, fhat, fr, g, gr);
    case 2: return spread_dispatch_l<2, T>(p, fhat, fr, g, gr);
    case 3: return spread_dispatch_l<3, T>(p, fhat, fr, g, gr);
  }
  return NFFT_ERR_UNSUPPORTED;
}

}  // namespace

int launch_spread(nfft_plan* p, const void* fhat, int fhat_real, void* g, int g_real) {
  return p->precision == 32 ? spread_dispatch<float>(p, fhat, fhat_real, g, g_real)
                            : spread_dispatch<double>(p, fhat, fhat_real, g, g_real);
}

}  // namespace nfft
