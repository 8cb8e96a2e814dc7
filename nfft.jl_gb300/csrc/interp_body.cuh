// Gather body of one node (D >= 2), shared by the single-plan kernel
// (interp.cu) and the batched persistent kernel (batch.cu).
#pragma once

#include "warpnode.cuh"

namespace nfft {
namespace {

template <int D, int L, typename T, bool TABLE>
__device__ __forceinline__ void interp_node(const Geom<T>& G, const Nodes<T>& Nd, const PolyRegs<D, L, T>& P,
                                            int64_t i, int lane, const typename Cplx<T>::type* __restrict__ g,
                                            typename Cplx<T>::type* __restrict__ fhat) {
  using C = typename Cplx<T>::type;
  using LN = Lanes<D, L>;
  const int m = G.m;
  const bool small = G.small_grid;
  const int ix = lane % L, ry = lane / L;
  const bool xact = ry < LN::RY;
  const int Nt0 = G.Nt[0], Nt1 = G.Nt[1];
  const int4 nd = __ldg(Nd.node4 + i);
  T W[LN::NW];
  node_weights<D, L, T, TABLE>(Nd, P, i, lane, W);
  const int gx = small ? wrap_any(nd.x + G.sh[0] - m + 1 + ix, Nt0) : wrap_once(nd.x + G.sh[0] - m + 1 + ix, Nt0);
  const T wx = wsel<D, L>(W, ix);
  int row[LN::NSTEP];
  T wxy[LN::NSTEP];
#pragma unroll
  for (int s = 0; s < LN::NSTEP; ++s) {
    const int iy = s * LN::RY + ry;
    const bool ok = xact && iy < L;
    const int iyc = ok ? iy : 0;
    const int gy = small ? wrap_any(nd.y + G.sh[1] - m + 1 + iyc, Nt1) : wrap_once(nd.y + G.sh[1] - m + 1 + iyc, Nt1);
    row[s] = gy * Nt0 + gx;
    const T wy = wsel<D, L>(W, L + iyc);  // every lane shuffles
    wxy[s] = ok ? wx * wy : T(0);
  }
  T ar = T(0), ai = T(0);
  if constexpr (D == 2) {
#pragma unroll
    for (int s = 0; s < LN::NSTEP; ++s) {
      const C v = __ldg(g + row[s]);
      ar = fma(wxy[s], v.x, ar);
      ai = fma(wxy[s], v.y, ai);
    }
  } else {
    // all of the node's grid loads first (memory-level parallelism), then the sums
    C v[L][LN::NSTEP];
#pragma unroll
    for (int iz = 0; iz < L; ++iz) {
      const int gz = small ? wrap_any(nd.z + G.sh[2] - m + 1 + iz, G.Nt[2])
                           : wrap_once(nd.z + G.sh[2] - m + 1 + iz, G.Nt[2]);
      const C* gp = g + int64_t(gz) * G.plane;
#pragma unroll
      for (int s = 0; s < LN::NSTEP; ++s) v[iz][s] = __ldg(gp + row[s]);
    }
    // sum over z first, then weight by wx wy: 2.4 instead of 3 multiply-adds
    // per tap (what bounds the FP64 gather on GB300's FP64 units)
    T sr[LN::NSTEP], si[LN::NSTEP];
#pragma unroll
    for (int s = 0; s < LN::NSTEP; ++s) sr[s] = si[s] = T(0);
#pragma unroll
    for (int iz = 0; iz < L; ++iz) {
      const T wz = wsel<D, L>(W, 2 * L + iz);
#pragma unroll
      for (int s = 0; s < LN::NSTEP; ++s) {
        sr[s] = fma(wz, v[iz][s].x, sr[s]);
        si[s] = fma(wz, v[iz][s].y, si[s]);
      }
    }
#pragma unroll
    for (int s = 0; s < LN::NSTEP; ++s) {
      ar = fma(wxy[s], sr[s], ar);
      ai = fma(wxy[s], si[s], ai);
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

}  // namespace
}  // namespace nfft
