// sortNodes = true: k .= sortslices(k, dims=2) (src/precomputation.jl:52-54,
// src/implementation.jl:112-114), the caller's D x M node array sorted in
// place by columns in lexicographic order (dimension 1 first; Julia's isless
// on each coordinate, so -0.0 sorts before 0.0).
//
// GB300 form: an LSD sort over the coordinates with the library's stable
// radix sort (sort.cu).  Each coordinate becomes an order-preserving unsigned
// key (sign bit set: all bits inverted; else the sign bit set), and the
// permutation is sorted stably by the key of the last dimension first, the
// first dimension last (FP64 keys in two 32-bit passes, low word first), so
// ties keep the order of the less significant coordinates.  The columns are
// then gathered by the permutation.  Nodes are checked like checkNodes
// (src/utils.jl:46-55) first; invalid nodes leave k untouched.
#include "nfft_internal.cuh"

#include <utility>

namespace nfft {
namespace {

__device__ __forceinline__ uint32_t ordered32(uint32_t u) { return (u & 0x80000000u) ? ~u : (u | 0x80000000u); }
__device__ __forceinline__ uint64_t ordered64(uint64_t u) {
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// key[i] = word `word` of the ordered bits of k[d, perm[i]]; val[i] = perm[i]
template <typename T>
__global__ void lex_key_kernel(const T* __restrict__ k, int D, int64_t M, int d, int word,
                               const int32_t* __restrict__ perm, uint32_t* __restrict__ key,
                               int32_t* __restrict__ val) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= M) return;
  const int32_t j = perm ? perm[i] : int32_t(i);
  const T x = k[int64_t(j) * D + d];
  if constexpr (sizeof(T) == 4) {
    key[i] = ordered32(__float_as_uint(x));
  } else {
    const uint64_t o = ordered64(static_cast<uint64_t>(__double_as_longlong(x)));
    key[i] = word ? uint32_t(o >> 32) : uint32_t(o);
  }
  val[i] = j;
}

template <typename T>
__global__ void gather_columns_kernel(const T* __restrict__ k, int D, int64_t M, const int32_t* __restrict__ perm,
                                      T* __restrict__ out) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= M) return;
  const int64_t j = perm[i];
  for (int d = 0; d < D; ++d) out[i * D + d] = k[j * D + d];
}

struct Buf {
  void* p = nullptr;
  ~Buf() {
    if (p) cudaFree(p);
  }
  bool alloc(size_t n) { return cudaMalloc(&p, n ? n : 1) == cudaSuccess; }
};

template <typename T> int sort_nodes_t(int D, int64_t M, void* k, int k_on_device, cudaStream_t s) {
  const size_t bytes = sizeof(T) * size_t(D) * size_t(M);
  Buf kd, kout, key, val, key2, val2, scr, flag;
  const size_t sb = radix_sort_scratch_bytes(M);
  if (!kd.alloc(bytes) || !kout.alloc(bytes) || !key.alloc(4 * size_t(M)) || !val.alloc(4 * size_t(M)) ||
      !key2.alloc(4 * size_t(M)) || !val2.alloc(4 * size_t(M)) || !scr.alloc(sb) || !flag.alloc(sizeof(int))) {
    set_error("cudaMalloc of the node sort buffers failed");
    return NFFT_ERR_ALLOC;
  }
  NFFT_CUDA_TRY(cudaMemcpyAsync(kd.p, k, bytes, k_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  // checkNodes before anything is reordered
  NFFT_CUDA_TRY(cudaMemsetAsync(flag.p, 0, sizeof(int), s));
  int rc = launch_check_node_values(sizeof(T) == 4 ? 32 : 64, kd.p, int64_t(D) * M, static_cast<int*>(flag.p), s);
  if (rc) return rc;
  int hflag = 0;
  NFFT_CUDA_TRY(cudaMemcpyAsync(&hflag, flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  NFFT_CUDA_TRY(cudaStreamSynchronize(s));
  if (hflag) {
    set_error("Nodes k need to be within the range [-1/2, 1/2)");
    return NFFT_ERR_NODE_OUT_OF_RANGE;
  }
  const unsigned nb = unsigned((M + 255) / 256);
  const int32_t* perm = nullptr;  // identity before the first pass
  const int words = sizeof(T) == 4 ? 1 : 2;
  for (int d = D - 1; d >= 0; --d) {
    for (int w = 0; w < words; ++w) {
      lex_key_kernel<T><<<nb, 256, 0, s>>>(static_cast<const T*>(kd.p), D, M, d, w, perm,
                                           static_cast<uint32_t*>(key.p), static_cast<int32_t*>(val.p));
      NFFT_LAUNCH_CHECK();
      uint32_t* ko = nullptr;
      int32_t* vo = nullptr;
      rc = radix_sort_pairs(static_cast<uint32_t*>(key.p), static_cast<int32_t*>(val.p),
                            static_cast<uint32_t*>(key2.p), static_cast<int32_t*>(val2.p), M, 32, scr.p, sb, s, &ko,
                            &vo);
      if (rc) return rc;
      // the sorted permutation must not be overwritten by the next key pass
      if (vo == static_cast<int32_t*>(val.p)) {
        std::swap(val.p, val2.p);
        std::swap(key.p, key2.p);
      }
      perm = vo;
    }
  }
  gather_columns_kernel<T><<<nb, 256, 0, s>>>(static_cast<const T*>(kd.p), D, M, perm, static_cast<T*>(kout.p));
  NFFT_LAUNCH_CHECK();
  NFFT_CUDA_TRY(cudaMemcpyAsync(k, kout.p, bytes, k_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
  NFFT_CUDA_TRY(cudaStreamSynchronize(s));
  return NFFT_OK;
}

}  // namespace
}  // namespace nfft

extern "C" int nfft_sort_nodes(int precision, int D, int64_t M, void* k, int k_on_device, void* stream) {
  using namespace nfft;
  if ((precision != 32 && precision != 64) || D < 1 || D > 3 || M < 0 || M > int64_t(INT32_MAX)) {
    set_error("nfft_sort_nodes: precision must be 32 or 64, 1 <= D <= 3 and 0 <= M < 2^31");
    return NFFT_ERR_INVALID_ARG;
  }
  if (M > 0 && !k) {
    set_error("null argument");
    return NFFT_ERR_INVALID_ARG;
  }
  if (M <= 1) return NFFT_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return precision == 32 ? sort_nodes_t<float>(D, M, k, k_on_device, s) : sort_nodes_t<double>(D, M, k, k_on_device, s);
}
