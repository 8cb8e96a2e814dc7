/*
 * nfft_gb300.h -- C ABI of the GB300 (sm_103a) NFFT plan.
 *
 * This is the boundary a host binding (Julia ccall, Python ctypes) calls.  It
 * replaces the GPU plan of NFFT.jl's GPUArrays extension
 * (ext/NFFTGPUArraysExt/implementation.jl) behind the AbstractNFFTs plan
 * interface (AbstractNFFTs/src/interface.jl:170-243).  Each entry point names
 * the reference interface it stands in for.
 *
 * Conventions (identical to NFFT.jl's):
 *  - nodes k: D x M, column-major (coordinate index fastest), each coordinate
 *    in [-1/2, 1/2];
 *  - images f and oversampled grids g: column-major (dimension 1 fastest);
 *  - complex values interleaved (re, im) of the plan's real type;
 *  - forward:  fHat[j] = sum_n f[n] exp(-2 pi i k_j . (n - N/2)),
 *    adjoint:  f[n]    = sum_j fHat[j] exp(+2 pi i k_j . (n - N/2)),
 *    computed as B F D and D^H F^H B^H (docs/src/background.md:64-85).
 *
 * Data pointers passed to the transform calls are DEVICE pointers, except
 * where a call says otherwise.  All transform calls are asynchronous on the
 * plan's stream.  A plan is not safe for concurrent calls (it owns its
 * oversampled grid, like NFFTPlan.tmpVec); independent plans are.
 */
#ifndef NFFT_GB300_H
#define NFFT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nfft_plan nfft_plan;

/* Status codes.  The Julia binding maps them onto the reference's exceptions:
 * INVALID_ARG and NODE_OUT_OF_RANGE -> ArgumentError (src/utils.jl:46-55,
 * src/convolution.jl:47-53), DIM_MISMATCH -> DimensionMismatch
 * (src/utils.jl:98-105), UNSUPPORTED -> error() (src/windowFunctions.jl:16,
 * src/precomputation.jl:401). */
typedef enum {
  NFFT_OK = 0,
  NFFT_ERR_INVALID_ARG = 1,
  NFFT_ERR_DIM_MISMATCH = 2,
  NFFT_ERR_NODE_OUT_OF_RANGE = 3,
  NFFT_ERR_ALLOC = 4,
  NFFT_ERR_CUDA = 5,
  NFFT_ERR_CUFFT = 6,
  NFFT_ERR_TIMEOUT = 7,
  NFFT_ERR_UNSUPPORTED = 8,
  NFFT_ERR_NO_NODES = 9
} nfft_status;

/* Window functions, src/windowFunctions.jl:4-19. */
enum {
  NFFT_WINDOW_KAISER_BESSEL = 0,
  NFFT_WINDOW_GAUSS = 1,
  NFFT_WINDOW_SPLINE = 2,
  NFFT_WINDOW_KAISER_BESSEL_REV = 3,
  NFFT_WINDOW_COSH_TYPE = 4
};

/* PrecomputeFlags, AbstractNFFTs/src/misc.jl:13-19.  On the device FULL
 * evaluates the window function itself per tap (no stored sparse matrix),
 * TENSOR and POLYNOMIAL evaluate the fitted polynomial of
 * src/precomputation.jl:302-320 per tap, LINEAR interpolates the
 * LUT of src/precomputation.jl:291-300. */
enum {
  NFFT_PRECOMPUTE_FULL = 1,
  NFFT_PRECOMPUTE_TENSOR = 2,
  NFFT_PRECOMPUTE_LINEAR = 3,
  NFFT_PRECOMPUTE_POLYNOMIAL = 4
};

enum { NFFT_F32 = 32, NFFT_F64 = 64 };

/* NFFTParams (src/implementation.jl:3-14).  m and sigma are final values:
 * the host binding applies accuracyParams (AbstractNFFTs/src/misc.jl:66-81)
 * before calling. */
typedef struct {
  int32_t m;                /* window half width (taps per dimension: 2m), 2..8 */
  double sigma;             /* oversampling factor; Ntilde = (ceil(sigma*N) / 2) * 2 */
  int32_t window;           /* NFFT_WINDOW_* */
  int32_t precompute;       /* NFFT_PRECOMPUTE_* */
  int32_t blocking;         /* 1: bin-sorted tiled kernels; 0: per-node kernels
                               with global atomics (the plain path) */
  int32_t sort_nodes;       /* sortNodes: 1 = the host binding sorts the caller's
                               k in place with nfft_sort_nodes before
                               nfft_set_nodes (the reference's in-place
                               sortslices); nfft_set_nodes itself never
                               reorders k */
  int32_t store_deconv_idx; /* accepted for interface parity; deconvolution is
                               fused with padding/cropping */
  int64_t block_size[3];    /* tile (block) size per dimension; 0 = automatic */
  int32_t compensated;      /* 1: compensated (Kahan) spreading tiles */
  int32_t timing;           /* 1: record per-stage device times (TimingStats) */
} nfft_params;

/* Plan geometry as NFFTPlan exposes it (N, NOut, J, Ntilde, params). */
typedef struct {
  int32_t precision;        /* 32 or 64 */
  int32_t D;
  int64_t N[3];
  int64_t Ntilde[3];
  int64_t M;                /* J, number of nodes */
  int32_t m;
  double sigma;
  int32_t window;
  int32_t precompute;
  int64_t lut_size;         /* LUTSize, src/precomputation.jl:14-17 */
  int64_t block_size[3];
  int64_t num_tiles;
  int64_t num_spread_tasks; /* after nfft_set_nodes */
  int64_t num_spread_entries;
  int64_t scratch_bytes;    /* device bytes held by the plan */
} nfft_info;

/* Fill defaults of NFFTParams for the GPU plan (m = 4, sigma = 2,
 * kaiser_bessel, POLYNOMIAL, blocking). */
void nfft_params_default(nfft_params* params);

/* plan_nfft(CuArray, k, N; kwargs...) without the nodes:
 * AbstractNFFTs.plan_nfft(::NFFTBackend, ::Type{<:AbstractGPUArray}, ...)
 * (ext/NFFTGPUArraysExt/implementation.jl:21-59).  Builds Ntilde
 * (src/precomputation.jl:3-56), the cuFFT plans, the deconvolution factors
 * (src/precomputation.jl:347-358, on the device in FP64) and the window
 * tables.  stream may be NULL (legacy default stream). */
int nfft_plan_create(nfft_plan** plan, int precision, int D, const int64_t* N, int64_t M,
                     const nfft_params* params, void* stream);

/* Finalizer; frees every device buffer the plan holds. */
int nfft_plan_destroy(nfft_plan* plan);

/* copy(p): an independent plan with the same nodes
 * (src/implementation.jl:45-66). */
int nfft_plan_copy(const nfft_plan* plan, nfft_plan** out);

/* Rebind the plan to another stream (CUDA.jl's task-local stream). */
int nfft_set_stream(nfft_plan* plan, void* stream);

/* nodes!(p, k) (AbstractNFFTs/src/interface.jl:208-213,
 * src/implementation.jl:108-141): checks the nodes like checkNodes
 * (src/utils.jl:46-55), reduces them to grid index and fractional offset,
 * bins them with a stable device radix sort (src/precomputation.jl:487-520)
 * and builds the spreading task list.  k is D x M of the plan's real type;
 * k_on_device selects a device or a host pointer.  Synchronises the stream. */
int nfft_set_nodes(nfft_plan* plan, const void* k, int k_on_device);

/* k .= sortslices(k, dims=2), the sortNodes = true step of plan_nfft and
 * nodes! (src/precomputation.jl:52-54, src/implementation.jl:112-114):
 * sorts the columns of the D x M node array k (precision 32 or 64) in place
 * in lexicographic order (dimension 1 first; isless per coordinate, -0.0
 * before 0.0) with a stable device radix sort.  k is a device or a host
 * pointer (k_on_device).  The nodes are checked like checkNodes first
 * (src/utils.jl:46-55): invalid nodes return NFFT_ERR_NODE_OUT_OF_RANGE and
 * leave k untouched.  Synchronous on stream (NULL: legacy default stream). */
int nfft_sort_nodes(int precision, int D, int64_t M, void* k, int k_on_device, void* stream);

/* mul!(fHat, p, f) (src/implementation.jl:155-172,
 * ext/NFFTGPUArraysExt/implementation.jl:97-115): fused pad + apodize,
 * forward FFT, gather interpolation. */
int nfft_forward(nfft_plan* plan, const void* f, void* fhat);

/* mul!(f, adjoint(p), fHat) (src/implementation.jl:176-193,
 * ext/NFFTGPUArraysExt/implementation.jl:118-136): spreading, backward
 * (unnormalised) FFT, fused crop + apodize. */
int nfft_adjoint(nfft_plan* plan, const void* fhat, void* f);

/* convolve!(p, g, fHat) (AbstractNFFTs/src/interface.jl:221-232,
 * src/convolution.jl:20-53).  g has size Ntilde.  A flag of 1 marks a real
 * array (the sampling-density client, NFFTTools/src/samplingDensity.jl:105-112);
 * complex g with real fHat is rejected (ArgumentError). */
int nfft_convolve(nfft_plan* plan, const void* g, int g_real, void* fhat, int fhat_real);

/* convolve_transpose!(p, fHat, g) (AbstractNFFTs/src/interface.jl:235-243,
 * src/convolution.jl:115-149).  Complex fHat with real g is rejected. */
int nfft_convolve_transpose(nfft_plan* plan, const void* fhat, int fhat_real, void* g, int g_real);

/* deconvolve!(p, f, g) (src/deconvolution.jl:2-45): writes the whole
 * oversampled grid g (zeros outside the image). */
int nfft_deconvolve(nfft_plan* plan, const void* f, void* g);

/* deconvolve_transpose!(p, g, f) (src/deconvolution.jl:49-92). */
int nfft_deconvolve_transpose(nfft_plan* plan, const void* g, void* f);

/* Node gradient (no reference counterpart: the reference rrules return
 * NoTangent for k, AbstractNFFTs/ext/AbstractNFFTsChainRulesCoreExt.jl:45,61).
 * dk[d, j] = Re( conj(w[j]) * d(A(k) v)_j / dk[d, j] ), with A the forward
 * NFFT; v has size N, w has length M, dk is D x M of the real type.  For a
 * loss of y = A f use (v, w) = (f, ybar); for a loss of x = A^H y use
 * (v, w) = (xbar, y). */
int nfft_grad_nodes(nfft_plan* plan, const void* v, const void* w, void* dk);

/* Tile-shape autotuner (no reference counterpart; the reference's blockSize
 * keyword is chosen by hand, src/precomputation.jl:59-77).  Re-bins the
 * plan's nodes for a set of candidate tile shapes (and, for D = 3, the two
 * warp layouts of nfft_set_tiling), times one spreading and one gather pass
 * per candidate on the plan's stream, and keeps the fastest.
 * With use_cache = 1 the choice is looked up in / stored to the file named by
 * the environment variable NFFT_GB300_TUNE_CACHE, keyed by (D, Ntilde,
 * log2 M, m, precision, SM count, precompute, compensated).  Synchronises. */
int nfft_autotune(nfft_plan* plan, int use_cache);

/* Re-tile the plan (blockSize) and re-bin its nodes.  Synchronises. */
int nfft_set_block_size(nfft_plan* plan, const int64_t* block_size);

/* nfft_set_block_size plus the D = 3 spreading warp layout (no reference
 * counterpart): row_parity_warps = 1 runs 8 warps per tile, each owning the
 * x-y slices of one residue mod 8; 2 runs 16 warps, each owning one residue
 * mod 8 and one row parity (for larger tiles).  Ignored for D < 3 and for
 * compensated plans.  Synchronises. */
int nfft_set_tiling(nfft_plan* plan, const int64_t* block_size, int row_parity_warps);

/* Plan geometry and sizes. */
int nfft_get_info(const nfft_plan* plan, nfft_info* info);

/* Device pointer of the plan's oversampled grid (NFFTPlan.tmpVec). */
void* nfft_grid(nfft_plan* plan);

/* TimingStats (AbstractNFFTs/src/misc.jl:22-30): device seconds of the last
 * transforms as {pre, conv, fft, deconv, conv_adjoint, fft_adjoint,
 * deconv_adjoint}.  Synchronises the stream. */
int nfft_get_timing(nfft_plan* plan, double out[7]);

/* Stage totals over all transforms since the last nfft_timing_reset (same
 * order as nfft_get_timing, pre excluded) and the number of forward
 * (calls[0]) and adjoint (calls[1]) transforms they cover.  Synchronises. */
int nfft_get_timing_totals(nfft_plan* plan, double totals[7], int64_t calls[2]);

/* Clear the stage totals. */
int nfft_timing_reset(nfft_plan* plan);

/* Integer outputs of the binning, copied to host buffers (the reference's
 * nodesInBlock, src/precomputation.jl:487-520): perm[i] = node at sorted
 * position i (0-based), tile_start (num_tiles+1) = CSR offsets of the tiles,
 * grid_index (D x M) = first grid index of each node's window per
 * dimension, (trunc(k*Ntilde) - m + 1) mod Ntilde.  Any pointer may be NULL. */
int nfft_get_binning(nfft_plan* plan, int32_t* perm, int32_t* tile_start, int32_t* grid_index);

/* Deconvolution factors 1/phi-hat per dimension (windowHatInvLUT,
 * src/precomputation.jl:347-358), copied to a host buffer of N[0]+..+N[D-1]
 * values of the plan's real type. */
int nfft_get_deconv_factors(nfft_plan* plan, void* out);

/* Node binning without any device allocation.  No counterpart in the
 * reference: it is the binning step of nfft_set_nodes (node check, reduction
 * to grid index, stable radix sort by tile -- the nodesInBlock order of
 * src/precomputation.jl:487-520) for callers that cannot call cudaMalloc at
 * that point, e.g. a host framework whose caching allocator already owns the
 * device memory, or a latency-critical pipeline that must not take the
 * implicit device synchronisation of cudaMalloc/cudaFree.  The caller passes
 * the nodes k (device, D x M of the real type), perm (device, M int32: node
 * at sorted position i) and tile_start (device, num_tiles+1 int32 CSR
 * offsets), with num_tiles = prod_d ceil(Ntilde[d] / block_size[d]).
 * Scratch is a static 16 MiB device array that every GPU loading the
 * library holds until exit; the limits are M <= 262144 nodes and
 * num_tiles <= 262144, larger requests fail with NFFT_ERR_UNSUPPORTED.  The
 * first call on a device looks up the array's device address (make it before
 * any stream capture).  All calls share the array: calls that overlap on the
 * GPU race.  Synchronises the stream once (node check). */
int nfft_bin_nodes_noalloc(int precision, int D, const int64_t* Ntilde, const int64_t* block_size, int64_t M,
                           const void* k, int32_t* perm, int32_t* tile_start, void* stream);

/* Batched plans (no reference counterpart: NFFT.jl transforms one plan per
 * mul! call, src/implementation.jl:145-204, and a set of plans is a loop of
 * such calls).  A batch runs the forward (or adjoint) transforms of many
 * plans of uneven N and M as one launch per stage over all plans -- pad,
 * the plans' FFTs, gather (forward); value sort, spreading with tasks of all
 * plans taken from one counter, the plans' FFTs, crop (adjoint) -- captured
 * once per direction into a CUDA graph on `stream` and replayed.  Members
 * need nodes, blocking = 1, compensated = 0, D = 2 or 3, and the same
 * precision, D, m and window-evaluation mode (POLYNOMIAL or table); their
 * grids and tile shapes may differ.  The batch uses the plans' grids and
 * sets their stream to `stream`; a member may not be used elsewhere while
 * the batch's call is in flight, and must outlive the batch.  After
 * nfft_set_nodes (or a block-size change) on a member the batch refuses to
 * run: create it again.  A NULL stream (legacy default) makes the batch use
 * a blocking stream of its own, ordered with the legacy stream. */
typedef struct nfft_batch nfft_batch;
int nfft_batch_create(nfft_batch** batch, nfft_plan* const* plans, int nplans, void* stream);
int nfft_batch_destroy(nfft_batch* batch);
/* f[i]: image of plan i (N_i complex), fhat[i]: its M_i node values. */
int nfft_batch_forward(nfft_batch* batch, const void* const* f, void* const* fhat);
int nfft_batch_adjoint(nfft_batch* batch, const void* const* fhat, void* const* f);

/* Directional plans: NFFTPlan(k, N; dims) (src/implementation.jl:73-104,
 * src/directional.jl) -- the NFFT along the contiguous dimensions
 * dim_lo..dim_hi (0-based, inclusive) of a D-dimensional array (D <= 3), every
 * other index a batch column.  k is (dim_hi-dim_lo+1) x M; node values are
 * arrays of size NOut = N with the dims range replaced by M (column-major).
 * precompute is LINEAR and the loops unblocked, as in the reference; params
 * supplies m, sigma and the window.  forward: f (N) -> fhat (NOut);
 * adjoint: fhat (NOut) -> f (N).  nfft_dplan_set_nodes checks the nodes
 * like checkNodes and synchronises the stream. */
typedef struct nfft_dplan nfft_dplan;
int nfft_dplan_create(nfft_dplan** plan, int precision, int D, const int64_t* N, int dim_lo, int dim_hi, int64_t M,
                      const nfft_params* params, void* stream);
int nfft_dplan_destroy(nfft_dplan* plan);
int nfft_dplan_set_nodes(nfft_dplan* plan, const void* k, int k_on_device);
int nfft_dplan_set_stream(nfft_dplan* plan, void* stream);
int nfft_dplan_forward(nfft_dplan* plan, const void* f, void* fhat);
int nfft_dplan_adjoint(nfft_dplan* plan, const void* fhat, void* f);

/* Toeplitz tools (NFFTTools/src/Toeplitz.jl): the Gram operator A^H A of a
 * plan with image size N as a convolution with a kernel lambda on the 2N
 * grid.  An nfft_toeplitz object owns the 2N-grid workspace and transforms
 * for one image size N (D <= 3) and precision; fft_mode 0 takes the fused
 * pruned-FFT path where every 2N_d is a power of two in [64, 1024] and D >= 2
 * (cuFFT otherwise), 1 always cuFFT.  Arrays are column-major complex T:
 * y has N points, lambda 2N.  All calls are asynchronous on `stream`. */
typedef struct nfft_toeplitz nfft_toeplitz;
int nfft_toeplitz_create(nfft_toeplitz** tz, int precision, int D, const int64_t* N, int fft_mode, void* stream);
int nfft_toeplitz_destroy(nfft_toeplitz* tz);
int nfft_toeplitz_set_stream(nfft_toeplitz* tz, void* stream);
/* 1 when nfft_toeplitz_apply runs the fused path. */
int nfft_toeplitz_is_fused(const nfft_toeplitz* tz, int* fused);
/* calculateToeplitzKernel!(lambda, p, tr, fftplan) after nodes!(p, tr)
 * (Toeplitz.jl:129-135; the allocating form :86-93): lambda =
 * FFT(fftshift(adjoint(p) * ones(J))).  p: a plan with nodes and size 2N of
 * the same precision; it runs on its own stream, ordered before this
 * object's stream. */
int nfft_toeplitz_kernel(nfft_toeplitz* tz, nfft_plan* plan, void* lambda);
/* calculateToeplitzKernel_explicit (Toeplitz.jl:142-164): lambda from the
 * exact sums over the D x M nodes k (T, host or device memory), accumulated
 * in FP64. */
int nfft_toeplitz_kernel_explicit(nfft_toeplitz* tz, const void* k, int64_t M, int k_on_device, void* lambda);
/* convolveToeplitzKernel!(y, lambda) (Toeplitz.jl:230-244), y in place:
 * y <- crop(IFFT(lambda . FFT(pad(y)))), IFFT normalised by 1/|2N|. */
int nfft_toeplitz_apply(nfft_toeplitz* tz, const void* lambda, void* y);

/* Direct (exact) transforms of src/direct.jl on the device, sums in FP64:
 * NDFTPlan (:99-151), NDCTPlan (:153-199), NDSTPlan (:202-249), NNDFTPlan
 * (:252-287).  N: the plan's N (D <= 4; the NDST's image is N - 1 per
 * dimension; the NNDFT's N[0] is the number of points y).  k: D x M nodes,
 * y: D x N[0] points (NNDFT), both T on the device.  adjoint = 0: image ->
 * M node values (NDFT/NNDFT sign -1); 1: the adjoint (sign +1) or, for the
 * NDCT/NDST, the transpose.  complex_data: interleaved complex T in and out
 * (required for NDFT/NNDFT), else real T.  Asynchronous on `stream`. */
enum { NFFT_NDFT = 0, NFFT_NDCT = 1, NFFT_NDST = 2, NFFT_NNDFT = 3 };
int nfft_direct(int kind, int precision, int D, const int64_t* N, int64_t M, const void* k, const void* y,
                int adjoint, int complex_data, const void* in, void* out, void* stream);

/* NFCT / NFST plans (the AbstractNFCTPlan / AbstractNFSTPlan types of
 * AbstractNFFTs/src/interface.jl:73-90; NFFT.jl itself computes them only
 * directly, src/direct.jl:153-249): kind NFFT_NDCT or NFFT_NDST, real data of
 * type T.  NFCT: f has N points, n_d = 0..N_d-1; NFST: f has N - 1 points,
 * n_d = 1..N_d-1 (size_in = N .- 1, as NDSTPlan).  Computed by the NFFT of
 * size 2N (params as for nfft_plan_create) of the even / odd extension of f;
 * the transpose folds the adjoint NFFT.  Nodes as for nfft_set_nodes. */
typedef struct nfft_tplan nfft_tplan;
int nfft_tplan_create(nfft_tplan** plan, int kind, int precision, int D, const int64_t* N, int64_t M,
                      const nfft_params* params, void* stream);
int nfft_tplan_destroy(nfft_tplan* plan);
int nfft_tplan_set_stream(nfft_tplan* plan, void* stream);
int nfft_tplan_set_nodes(nfft_tplan* plan, const void* k, int k_on_device);
/* mul!(fHat, p, f): real f -> real fHat (M) */
int nfft_tplan_forward(nfft_tplan* plan, const void* f, void* fhat);
/* mul!(f, transpose(p), fHat): real fHat (M) -> real f */
int nfft_tplan_transpose(nfft_tplan* plan, const void* fhat, void* f);

/* Fast NNFFT plans (nonequispaced in both domains: the transform of
 * NNDFTPlan, src/direct.jl:252-287; AbstractNNFFTPlan of AbstractNFFTs):
 * fHat_j = sum_l c_l exp(-2 pi i k_j . y_l) with nodes k (D x M, |k| <= 1/2)
 * and points y (D x Ny, any finite values).  Computed by spreading c at y / N1
 * with a plan of size N1 = 2 ceil(max |y| + m / sigma) + 2, a forward NFFT of
 * size sigma N1 at k / sigma1 and a division by the window transform; params
 * as for nfft_plan_create.  nfft_nnplan_set_nodes (re)builds the two plans
 * and synchronises. */
typedef struct nfft_nnplan nfft_nnplan;
int nfft_nnplan_create(nfft_nnplan** plan, int precision, int D, int64_t M, int64_t Ny, const nfft_params* params,
                       void* stream);
int nfft_nnplan_destroy(nfft_nnplan* plan);
int nfft_nnplan_set_stream(nfft_nnplan* plan, void* stream);
int nfft_nnplan_set_nodes(nfft_nnplan* plan, const void* k, const void* y, int on_device);
/* c (Ny complex) -> fhat (M complex) */
int nfft_nnplan_forward(nfft_nnplan* plan, const void* c, void* fhat);
/* fhat (M complex) -> c (Ny complex) */
int nfft_nnplan_adjoint(nfft_nnplan* plan, const void* fhat, void* c);

/* Wait for the plan's stream.  Returns NFFT_ERR_TIMEOUT (once) if a kernel
 * of the plan gave up waiting for a bulk tensor copy into shared memory
 * (bounded waits: the kernel skips the work it was waiting for instead of
 * spinning forever). */
int nfft_sync(nfft_plan* plan);

/* Number of kernels this library has launched in the calling process. */
int64_t nfft_kernel_launch_count(void);

const char* nfft_status_string(int status);

/* Message of the last failing call on this host thread. */
const char* nfft_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* NFFT_GB300_H */
