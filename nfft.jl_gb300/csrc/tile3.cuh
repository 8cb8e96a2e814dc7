// Fixed 3-D tile shapes (m = 4) shared by the shape-specialised spreading
// (spread_tile3.cuh) and gather (interp.cu) kernels: the tile padded by the
// window, laid out in shared memory as a TMA box of the grid, and the host
// side that encodes the grid's tensor map.
//
// The padded tile of a tile with origin (o0, o1, o2) covers grid x from
// o0 - m (even: one leading column outside the window, so that the box starts
// on a 16-byte boundary) and grid y, z from o - m + 1; its rows have a
// constant pitch (>= the padded width, = 8 mod 16 complex values, so the two
// row pairs a half-warp touches fall in distinct banks).  A tile whose box
// lies inside the grid moves between grid and shared memory with one bulk
// tensor copy; a tile whose box wraps around the grid is moved per point.
#pragma once

#include <cuda.h>  // CUtensorMap (encoded on the host through the runtime's driver entry point)

#include <mutex>

#include "nfft_internal.cuh"

namespace nfft {
namespace {

template <int BX, int BY, int BZ> struct Tile3 {
  static constexpr int L = 8;
  static constexpr int P0 = BX + L;                      // columns, from grid x o0 - m
  static constexpr int PITCH = P0 + ((8 - P0 % 16) + 16) % 16;  // >= P0, = 8 mod 16: conflict-free row pairs
  static constexpr int P1 = BY + L - 1;
  static constexpr int P2 = BZ + L - 1;
  static constexpr int PLANE = PITCH * P1;
  static constexpr int NACC = PLANE * P2;                // float2 accumulators
  static constexpr int THREADS = 256;
  static constexpr int NB = 32;                          // nodes per staged batch
  static constexpr size_t ACC_BYTES = (size_t(NACC) * 8 + 127) & ~size_t(127);
  static constexpr size_t SMEM = ACC_BYTES + size_t(NB) * (16 + 8 + 8 * L + 4 * 3 * L + 4 * L * L);
  static_assert(PITCH <= 128 && P1 <= 256 && P2 <= 256, "TMA box extents");
};

// mbarrier operations on a shared-memory barrier at address addr.
__device__ __forceinline__ void mbar_init(unsigned addr, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned addr, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(addr), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned addr, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(addr), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase with the given parity: false after 2^22 polls.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned addr, unsigned parity) {
  for (int it = 0; it < (1 << 22); ++it)
    if (mbar_try_wait(addr, parity)) return true;
  return false;
}

// The grid region of a tile's padded box lies inside the grid (no wrap):
// the box is added with one bulk tensor reduction.
template <int BX, int BY, int BZ>
__device__ __forceinline__ bool tile3_interior(const Geom<float>& G, int o0, int o1, int o2) {
  using TC = Tile3<BX, BY, BZ>;
  const int x = o0 - 4, y = o1 - 3, z = o2 - 3;
  return x >= 0 && y >= 0 && z >= 0 && x + TC::PITCH <= G.Nt[0] && y + TC::P1 <= G.Nt[1] && z + TC::P2 <= G.Nt[2];
}

// Host: the tile shapes with compiled kernels (m = 4, FP32, blockSize[3] = 8).
inline bool tile3_shape(const nfft_plan* p) {
  if (p->D != 3 || p->m != 4 || p->precision != 32 || p->bs[2] != 8) return false;
  const int64_t bx = p->bs[0], by = p->bs[1];
  return (bx == 16 && by == 8) || (bx == 16 && by == 16) || (bx == 32 && by == 8) || (bx == 8 && by == 8);
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library does not link the driver library itself); null if unavailable.
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(f);
  });
  return fn;
}

// Tensor map of the FP32 grid g (2 Ntilde[0] floats x Ntilde[1] x Ntilde[2])
// with the padded-tile box of Tile3<BX, BY, BZ>, cached on the plan per grid
// and shape (two entries: the plan's forward and adjoint grids).  Null when it
// cannot be made (no driver entry point, grid not 16-byte aligned, box larger
// than the grid): the kernels then move tiles point by point.
template <int BX, int BY, int BZ> const CUtensorMap* tile3_map(nfft_plan* p, void* g) {
  using TC = Tile3<BX, BY, BZ>;
  const int64_t key = (int64_t(BX) << 20) | (int64_t(BY) << 10) | BZ;
  for (int i = 0; i < 2; ++i)
    if (p->tmap_grid[i] == g && p->tmap_key[i] == key) return &p->tmap[i];
  EncodeTiledFn fn = encode_tiled();
  if (!fn || (reinterpret_cast<uintptr_t>(g) & 15) != 0) return nullptr;
  if (p->Nt[0] < TC::PITCH || p->Nt[1] < TC::P1 || p->Nt[2] < TC::P2) return nullptr;
  const int slot = p->tmap_next;
  p->tmap_grid[slot] = nullptr;
  const cuuint64_t dims[3] = {cuuint64_t(2 * p->Nt[0]), cuuint64_t(p->Nt[1]), cuuint64_t(p->Nt[2])};
  const cuuint64_t strides[2] = {cuuint64_t(8 * p->Nt[0]), cuuint64_t(8 * p->Nt[0] * p->Nt[1])};
  const cuuint32_t box[3] = {cuuint32_t(2 * TC::PITCH), cuuint32_t(TC::P1), cuuint32_t(TC::P2)};
  const cuuint32_t es[3] = {1, 1, 1};
  if (fn(&p->tmap[slot], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, g, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
         CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
      CUDA_SUCCESS)
    return nullptr;
  p->tmap_grid[slot] = g;
  p->tmap_key[slot] = key;
  p->tmap_next = slot ^ 1;
  return &p->tmap[slot];
}

}  // namespace
}  // namespace nfft
