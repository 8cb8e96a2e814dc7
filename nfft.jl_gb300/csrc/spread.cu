// Spreading (convolve_transpose!): g[tap] += prod_d phi_d * fHat[j] over the
// (2m)^D window taps of every node, src/convolution.jl:349-520.
//
// The GB300 form of NFFT.jl's blocked adjoint (private padded block per
// block, then a locked wrap-add into g, :356-443):
//   * nodes are bin-sorted by home tile (bs[0] x bs[1] x bs[2] grid points);
//     one CTA per task = one home tile or a chunk of a hot tile;
//   * the CTA accumulates into the tile padded by 2m-1 points in shared
//     memory, so every tap of every node lands inside it: no per-tap bounds
//     tests and no wrap-around in the hot loop;
//   * D >= 2 (spread_owned_kernel): warp w owns the slices of the padded tile
//     along the last dimension with index = w mod 8 (x-y planes for D = 3, x
//     rows for D = 2).  Each tile point then has exactly one writer, so the
//     accumulation is a plain read-modify-write of a complex value (measured
//     ~17x the throughput of shared-memory float atomics on GB300), and can
//     carry a Kahan compensation term (compensated = 1).  Nodes are staged in
//     shared memory in batches (window values, x*y weight products, value);
//   * D = 1 (spread_pad1_kernel): 32/G nodes per warp, shared-memory atomics;
//     compensated (spread_line_kahan_kernel): one warp per task, lane l owns
//     the padded positions x = l mod 32, Kahan read-modify-writes;
//   * the padded tile is added to the zeroed grid with vector global atomics
//     (red.global.add.v2), wrapping periodically; all-zero points are skipped.
// The lock of the reference becomes the L2 atomics of the flush.
#include "spread_body.cuh"
#include "spread_tile3.cuh"

namespace nfft {
namespace {

// fHat in bin-sorted order (node4[i].w = input index), for coalesced staging.
// blockIdx.y: column of a multi-column launch (input fhat + y fcol, output out + y M)
template <typename T>
__global__ void sort_values_kernel(const int4* __restrict__ node4, const typename Cplx<T>::type* __restrict__ fhat,
                                   typename Cplx<T>::type* __restrict__ out, int64_t M, int64_t fcol = 0) {
  fhat += blockIdx.y * fcol;
  out += blockIdx.y * M;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < M; i += int64_t(gridDim.x) * blockDim.x)
    out[i] = __ldg(fhat + __ldg(node4 + i).w);
}

// fHat of every column in bin-sorted order (grid-stride, a few CTAs per SM).
template <typename T>
int sort_values(const nfft_plan* p, const typename Cplx<T>::type* fhat, typename Cplx<T>::type* out, int ncols,
                int64_t fcol) {
  int dev = 0, sms = 1;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                cudaSuccess || sms < 1)
    sms = 1;
  int64_t nb = (p->M + 255) / 256;
  const int64_t cap = (int64_t(sms) * 32 + ncols - 1) / ncols;
  if (nb > cap) nb = cap;
  if (nb < 1) nb = 1;
  sort_values_kernel<T><<<dim3(unsigned(nb), unsigned(ncols)), 256, 0, p->stream>>>(p->node4, fhat, out, p->M, fcol);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

template <int BX, int BY, int BZ>
int tile3_launch(nfft_plan* p, const Geom<float>& G, const Nodes<float>& Nd, const float2* fs, float* gp, int ncols,
                 int64_t fcol, int64_t gcol_t) {
  using TC = Tile3<BX, BY, BZ>;
  const CUtensorMap* map = (ncols == 1 && p->spread_tma) ? tile3_map<BX, BY, BZ>(p, gp) : nullptr;
  const int use_tma = map ? 1 : 0;
  CUtensorMap none{};
  auto kern = p->wtab ? spread_tile3_kernel<BX, BY, BZ, true> : spread_tile3_kernel<BX, BY, BZ, false>;
  NFFT_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(TC::SMEM)));
  kern<<<dim3(unsigned(p->n_tasks), unsigned(ncols)), TC::THREADS, TC::SMEM, p->stream>>>(
      map ? *map : none, use_tma, G, Nd, p->tasks, fs, gp, ncols > 1 ? fcol : 0, gcol_t);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

// The one-step staging kernel for table windows: values fhat + c fcol in the
// caller's order, read through the bin-sorted nodes' input indices.
template <int BX, int BY, int BZ>
int tile3_rec_launch(nfft_plan* p, const Geom<float>& G, const Nodes<float>& Nd, const float2* fhat, float* gp,
                     int ncols, int64_t fcol, int64_t gcol_t) {
  using TC = Tile3<BX, BY, BZ>;
  using TR = Tile3Rec<BX, BY, BZ>;
  const CUtensorMap* map = (ncols == 1 && p->spread_tma) ? tile3_map<BX, BY, BZ>(p, gp) : nullptr;
  CUtensorMap none{};
  // a zeroed buffer of the largest padded tile, copied into shared memory to
  // clear each CTA's tile (allocated once per plan)
  static_assert(TC::NACC * 8 <= 128 * 1024, "zero tile buffer");
  if (!p->zero_tile && p->spread_zero_copy) {
    if (cudaMalloc(&p->zero_tile, 128 * 1024) != cudaSuccess ||
        cudaMemsetAsync(p->zero_tile, 0, 128 * 1024, p->stream) != cudaSuccess) {
      cudaFree(p->zero_tile);
      p->zero_tile = nullptr;
      p->spread_zero_copy = false;  // plain stores clear the tile
      cudaGetLastError();
    }
  }
  WinCoeffs8 wc{};
  if (!p->wtab)
    for (int q = 0; q < 8 * 9; ++q) wc.c[q] = float(p->coeffs_host[q]);
  auto kr = p->wtab ? spread_tile3_rec_kernel<BX, BY, BZ, true> : spread_tile3_rec_kernel<BX, BY, BZ, false>;
  NFFT_CUDA_TRY(cudaFuncSetAttribute(kr, cudaFuncAttributeMaxDynamicSharedMemorySize, int(TR::SMEM)));
  kr<<<dim3(unsigned(p->n_tasks), unsigned(ncols)), TC::THREADS, TR::SMEM, p->stream>>>(
      map ? *map : none, map ? 1 : 0, G, Nd, p->tasks, fhat, gp, ncols > 1 ? fcol : 0, gcol_t,
      p->spread_zero_copy ? static_cast<const float4*>(p->zero_tile) : nullptr, p->dflag + 1, wc);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

// The one-step kernel when the plan's tiles have a shape-specialised form
// (no value sort); -1 = not applicable.
int spread_tile3_user(nfft_plan* p, const Geom<float>& G, const Nodes<float>& Nd, const float2* fhat, float* gp,
                      int ncols, int64_t fcol, int64_t gcol_t) {
  if (!p->spread_tile3 || !p->spread_rec || (!p->wtab && !p->frac4) || p->D != 3 || p->m != 4 ||
      p->prm.compensated ||
      p->spread_layout != 1 || p->bs[2] != 8)
    return -1;
  const int64_t bx = p->bs[0], by = p->bs[1];
  if (bx == 16 && by == 8) return tile3_rec_launch<16, 8, 8>(p, G, Nd, fhat, gp, ncols, fcol, gcol_t);
  if (bx == 16 && by == 16) return tile3_rec_launch<16, 16, 8>(p, G, Nd, fhat, gp, ncols, fcol, gcol_t);
  if (bx == 32 && by == 8) return tile3_rec_launch<32, 8, 8>(p, G, Nd, fhat, gp, ncols, fcol, gcol_t);
  if (bx == 8 && by == 8) return tile3_rec_launch<8, 8, 8>(p, G, Nd, fhat, gp, ncols, fcol, gcol_t);
  return -1;
}

// The shape-specialised 3-D kernel when the plan's tiles have one of its
// shapes (FP32, m = 4, uncompensated, 8-warp layout); -1 = not applicable.
int spread_tile3(nfft_plan* p, const Geom<float>& G, const Nodes<float>& Nd, const float2* fs, float* gp, int ncols,
                 int64_t fcol, int64_t gcol_t) {
  if (!p->spread_tile3 || p->D != 3 || p->m != 4 || p->prm.compensated || p->spread_layout != 1) return -1;
  const int64_t bx = p->bs[0], by = p->bs[1], bz = p->bs[2];
  if (bz != 8) return -1;
  if (bx == 16 && by == 8) return tile3_launch<16, 8, 8>(p, G, Nd, fs, gp, ncols, fcol, gcol_t);
  if (bx == 16 && by == 16) return tile3_launch<16, 16, 8>(p, G, Nd, fs, gp, ncols, fcol, gcol_t);
  if (bx == 32 && by == 8) return tile3_launch<32, 8, 8>(p, G, Nd, fs, gp, ncols, fcol, gcol_t);
  if (bx == 8 && by == 8) return tile3_launch<8, 8, 8>(p, G, Nd, fs, gp, ncols, fcol, gcol_t);
  return -1;
}

// ncols columns in one launch (blockIdx.y): values fhat + c fcol, grids
// g + c gcol (complex elements; the grids must be contiguous, gcol = |Ntilde|),
// bin-sorted values in `sorted` (M x ncols); ncols = 1 uses the plan's own scratch.
template <int D, int L, typename T>
int spread_launch(nfft_plan* p, const void* fhat, void* g, int ncols, int64_t fcol, int64_t gcol, void* sorted) {
  Geom<T> G = make_geom<T>(p);
  Nodes<T> Nd = make_nodes<T>(p);
  using C = typename Cplx<T>::type;
  const size_t gbytes = size_t(p->Nt[0] * p->Nt[1] * p->Nt[2]) * sizeof(T) * 2;
  if (!p->skip_memset) NFFT_CUDA_TRY(cudaMemsetAsync(g, 0, gbytes * size_t(ncols), p->stream));
  if (p->n_tasks == 0) return NFFT_OK;
  const C* fp = static_cast<const C*>(fhat);
  T* gp = static_cast<T*>(g);
  const int64_t gcol_t = 2 * gcol;  // in T units
  if (ncols > 1 && (p->prm.compensated || (D == 3 && p->spread_layout == 2))) {
    set_error("multi-column spreading supports the default (uncompensated, 8-warp) tiles only");
    return NFFT_ERR_UNSUPPORTED;
  }
  if constexpr (D == 1) {
    if (p->prm.compensated) {
      const size_t smem = ((sizeof(typename Acc<T, true>::type) * size_t(p->bs[0] + L - 1) + 31) & ~size_t(31)) +
                          sizeof(T) * size_t(2 * 32 * L + L * (L + 1));
      if (smem > 227 * 1024) {
        set_error("compensated spreading row of %zu bytes does not fit in shared memory; use a smaller blockSize",
                  smem);
        return NFFT_ERR_UNSUPPORTED;
      }
      auto kern = p->wtab ? spread_line_kahan_kernel<L, T, true> : spread_line_kahan_kernel<L, T, false>;
      NFFT_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
      kern<<<unsigned(p->n_tasks), 32, smem, p->stream>>>(G, Nd, p->tasks, fp, gp);
      NFFT_LAUNCH_CHECK();
      return NFFT_OK;
    }
    const size_t smem = 2 * sizeof(T) * size_t(p->bs[0] + L - 1);
    if (smem > 227 * 1024) {
      set_error("spreading row of %zu bytes does not fit in shared memory; use a smaller blockSize", smem);
      return NFFT_ERR_UNSUPPORTED;
    }
    auto kern = p->wtab ? spread_pad1_kernel<L, T, true> : spread_pad1_kernel<L, T, false>;
    NFFT_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    kern<<<dim3(unsigned(p->n_tasks), unsigned(ncols)), kSpreadThreads, smem, p->stream>>>(G, Nd, p->tasks, fp, gp,
                                                                                          fcol, gcol_t);
  } else {
    const bool comp = p->prm.compensated != 0;
    const size_t smem = owned_smem<D, L, T>(p, comp);
    if (smem > 227 * 1024) {
      set_error("padded spreading tile (%zu bytes) does not fit in shared memory; use a smaller blockSize", smem);
      return NFFT_ERR_UNSUPPORTED;
    }
    auto kern = comp ? (p->wtab ? spread_owned_kernel<D, L, T, true, true> : spread_owned_kernel<D, L, T, false, true>)
                     : (p->wtab ? spread_owned_kernel<D, L, T, true, false> : spread_owned_kernel<D, L, T, false, false>);
    int threads = OwnedCfg<D, L>::THREADS;
    if constexpr (D == 3) {
      if (!comp && p->spread_layout == 2) {  // 16 warps: slice group x row parity
        kern = p->wtab ? spread_owned_kernel<D, L, T, true, false, 2> : spread_owned_kernel<D, L, T, false, false, 2>;
        threads = OwnedCfg<D, L, 2>::THREADS;
      }
    }
    if constexpr (D == 3 && L == 8 && sizeof(T) == 4) {  // values read in the caller's order
      const int rc = spread_tile3_user(p, G, Nd, fp, gp, ncols, fcol, gcol_t);
      if (rc != -1) return rc;
    }
    NFFT_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    C* fs = static_cast<C*>(ncols > 1 ? sorted : p->fsorted);
    int rc = sort_values<T>(p, fp, fs, ncols, fcol);
    if (rc) return rc;
    if constexpr (D == 3 && L == 8 && sizeof(T) == 4) {
      rc = spread_tile3(p, G, Nd, fs, gp, ncols, p->M, gcol_t);
      if (rc != -1) return rc;
    }
    kern<<<dim3(unsigned(p->n_tasks), unsigned(ncols)), threads, smem, p->stream>>>(G, Nd, p->tasks, fs, gp,
                                                                                   p->spread_pitch, p->M, gcol_t);
  }
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

#define NFFT_SPREAD_ARGS p, fhat, g, ncols, fcol, gcol, sorted
template <int D, typename T>
int spread_dispatch_l(nfft_plan* p, const void* fhat, void* g, int ncols, int64_t fcol, int64_t gcol, void* sorted) {
  switch (p->m) {
    case 2: return spread_launch<D, 4, T>(NFFT_SPREAD_ARGS);
    case 3: return spread_launch<D, 6, T>(NFFT_SPREAD_ARGS);
    case 4: return spread_launch<D, 8, T>(NFFT_SPREAD_ARGS);
    case 5: return spread_launch<D, 10, T>(NFFT_SPREAD_ARGS);
    case 6: return spread_launch<D, 12, T>(NFFT_SPREAD_ARGS);
    case 7: return spread_launch<D, 14, T>(NFFT_SPREAD_ARGS);
    case 8: return spread_launch<D, 16, T>(NFFT_SPREAD_ARGS);
  }
  set_error("m = %d not supported (2..8)", p->m);
  return NFFT_ERR_UNSUPPORTED;
}

template <typename T>
int spread_dispatch(nfft_plan* p, const void* fhat, void* g, int ncols, int64_t fcol, int64_t gcol, void* sorted) {
  switch (p->D) {
    case 1: return spread_dispatch_l<1, T>(NFFT_SPREAD_ARGS);
    case 2: return spread_dispatch_l<2, T>(NFFT_SPREAD_ARGS);
    case 3: return spread_dispatch_l<3, T>(NFFT_SPREAD_ARGS);
  }
  return NFFT_ERR_UNSUPPORTED;
}
#undef NFFT_SPREAD_ARGS

}  // namespace

// Row pitch (in accumulator elements) of the padded tile: the smallest pitch
// >= the padded row length for which every shared-memory access phase of a
// warp step (lanes = L taps along x times the row slots) hits distinct banks.
int spread_pitch_for(int D, int m, int P0, int elem_bytes, int ny) {
  const int L = 2 * m;
  // lane -> (column ix, row slot ry); D = 3 rows are ny pitches apart (ny = 2:
  // row-parity ownership), D = 2 rows of one warp are 2 slices = 2 pitches apart
  const int RY = D == 3 ? 32 / L : (D == 2 ? (L + 1) / 2 : 1);
  const int rowmul = D == 2 ? 2 : (D == 3 ? ny : 1);
  const int words = elem_bytes / 4;       // 32-bit words per element
  const int lanes_per_phase = 32 / words;  // lanes served per shared-memory wavefront
  for (int pitch = P0; pitch < P0 + 64; ++pitch) {
    bool ok = true;
    for (int ph = 0; ph < words && ok; ++ph) {
      int used[32] = {};
      for (int l = ph * lanes_per_phase; l < (ph + 1) * lanes_per_phase && ok; ++l) {
        const int ix = l % L, ry = l / L;
        if (ry >= RY) continue;
        for (int w = 0; w < words; ++w) {
          const int bank = ((ix + pitch * rowmul * ry) * words + w) % 32;
          if (used[bank]++) ok = false;
        }
      }
    }
    if (ok) return pitch;
  }
  return P0;
}

int launch_spread(nfft_plan* p, const void* fhat, int, void* g, int) {
  return p->precision == 32 ? spread_dispatch<float>(p, fhat, g, 1, 0, 0, nullptr)
                            : spread_dispatch<double>(p, fhat, g, 1, 0, 0, nullptr);
}

int launch_spread_cols(nfft_plan* p, const void* fhat, void* g, int ncols, int64_t fcol, int64_t gcol,
                       void* sorted) {
  return p->precision == 32 ? spread_dispatch<float>(p, fhat, g, ncols, fcol, gcol, sorted)
                            : spread_dispatch<double>(p, fhat, g, ncols, fcol, gcol, sorted);
}

}  // namespace nfft
