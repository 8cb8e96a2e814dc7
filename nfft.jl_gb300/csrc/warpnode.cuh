// Warp-per-node helpers shared by the gather, spreading and node-gradient
// kernels.
//
// A warp handles one node (D = 2, 3) or 32/G nodes (D = 1, G = 2m rounded up
// to a power of two).  Lane layout for D >= 2: lane = ix + L*ry with ix the
// tap along dimension 1 (contiguous grid addresses) and ry a row slot; taps
// along dimension 2 are visited in NSTEP steps of RY rows, taps along
// dimension 3 in a uniform loop.  The D*L window values of a node are held
// one per lane (lane q <-> dimension q / L, tap q % L; a second register for
// q >= 32) and exchanged with shuffles.
#pragma once

#include "nfft_internal.cuh"

namespace nfft {

template <int D, int L> struct Lanes {
  static constexpr int RY = (D == 1) ? 1 : (32 / L);
  static constexpr int NSTEP = (D == 1) ? 1 : (L + RY - 1) / RY;
  static constexpr int NW = (D * L + 31) / 32;  // weight registers per lane
  static constexpr int G1 = L <= 2 ? 2 : L <= 4 ? 4 : L <= 8 ? 8 : L <= 16 ? 16 : 32;  // D = 1 group
  static constexpr int NPW = 32 / G1;           // D = 1 nodes per warp
  static constexpr int DEG = L + 1;             // polynomial coefficients (degree 2m)
};

template <typename T> __device__ __forceinline__ T shfl_w(T v, int src) { return __shfl_sync(0xFFFFFFFFu, v, src); }

// Weight q of the current node (q compile-time after unrolling).
template <int D, int L, typename T> __device__ __forceinline__ T wsel(const T (&W)[Lanes<D, L>::NW], int q) {
  if constexpr (Lanes<D, L>::NW == 1) {
    return shfl_w(W[0], q);
  } else {
    T a = shfl_w(W[0], q & 31);
    T b = shfl_w(W[1], q & 31);
    return q < 32 ? a : b;
  }
}

// Polynomial coefficients of the columns this lane evaluates (POLYNOMIAL
// mode): column (lane + 32 r) % L, degree 2m (src/precomputation.jl:302-320).
template <int D, int L, typename T> struct PolyRegs {
  T c[Lanes<D, L>::NW][Lanes<D, L>::DEG];
  __device__ __forceinline__ void load(const T* __restrict__ coeffs, int lane) {
#pragma unroll
    for (int r = 0; r < Lanes<D, L>::NW; ++r) {
      const int l = (lane + 32 * r) % L;
#pragma unroll
      for (int i = 0; i < Lanes<D, L>::DEG; ++i) c[r][i] = __ldg(coeffs + l * Lanes<D, L>::DEG + i);
    }
  }
  // evalpoly(e - 1/2, coeffs[:, l]) by Horner
  __device__ __forceinline__ T eval(int r, T e) const {
    const T t = e - T(0.5);
    T v = c[r][Lanes<D, L>::DEG - 1];
#pragma unroll
    for (int i = Lanes<D, L>::DEG - 2; i >= 0; --i) v = fma(v, t, c[r][i]);
    return v;
  }
};

// The node's window values, one (or two) per lane.
template <int D, int L, typename T, bool TABLE>
__device__ __forceinline__ void node_weights(const Nodes<T>& Nd, const PolyRegs<D, L, T>& P, int64_t i, int lane,
                                             T (&W)[Lanes<D, L>::NW]) {
  constexpr int DL = D * L;
#pragma unroll
  for (int r = 0; r < Lanes<D, L>::NW; ++r) {
    const int q = lane + 32 * r;
    W[r] = T(0);
    if (q < DL) {
      if constexpr (TABLE) {
        W[r] = __ldg(Nd.wtab + i * DL + q);
      } else {
        const int d = q / L;
        W[r] = P.eval(r, __ldg(Nd.frac4 + 4 * i + d));
      }
    }
  }
}

__device__ __forceinline__ int4 load_node(const Nodes<float>& Nd, int64_t i) { return __ldg(Nd.node4 + i); }
__device__ __forceinline__ int4 load_node(const Nodes<double>& Nd, int64_t i) { return __ldg(Nd.node4 + i); }

}  // namespace nfft
