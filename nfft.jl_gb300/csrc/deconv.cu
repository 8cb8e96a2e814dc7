// Fused deconvolution (apodization) with zero padding / cropping.
//
// pad_apodize   replaces fill!(tmpVec, 0) + deconvolve! of mul!
//               (src/implementation.jl:159-160, src/deconvolution.jl:22-45): one
//               pass writes every point of the oversampled grid, f[n] times the
//               separable factors 1/phi-hat at g[(n - N/2) mod Ntilde], zeros
//               elsewhere.
// crop_apodize  replaces deconvolve_transpose! (src/deconvolution.jl:69-92).
#include "nfft_internal.cuh"

namespace nfft {
namespace {

template <typename T> struct Grid3 {
  int N0, N1, N2;
  int Nt0, Nt1, Nt2;
  const T* inv0;
  const T* inv1;
  const T* inv2;
};

// One thread writes two consecutive grid points of a row (Ntilde[0] is even).
template <typename T>
__global__ void __launch_bounds__(256) pad_apodize_kernel(Grid3<T> G, const typename Cplx<T>::type* __restrict__ f,
                                                          typename Cplx<T>::type* __restrict__ g, int64_t npairs) {
  using C = typename Cplx<T>::type;
  const int half = G.Nt0 >> 1;
  for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < npairs;
       q += int64_t(gridDim.x) * blockDim.x) {
    const int64_t row = q / half;
    const int gx = int(q - row * half) * 2;
    const int gy = int(row % G.Nt1);
    const int gz = int(row / G.Nt1);
    // n = (g + N/2) mod Ntilde is an image index iff n < N
    const int ny = wrap_once(gy + G.N1 / 2, G.Nt1);
    const int nz = wrap_once(gz + G.N2 / 2, G.Nt2);
    C v0 = {T(0), T(0)}, v1 = {T(0), T(0)};
    if (ny < G.N1 && nz < G.N2) {
      const T s = __ldg(G.inv1 + ny) * __ldg(G.inv2 + nz);
      const int64_t frow = int64_t(G.N0) * (ny + int64_t(G.N1) * nz);
      const int nx0 = wrap_once(gx + G.N0 / 2, G.Nt0);
      const int nx1 = wrap_once(gx + 1 + G.N0 / 2, G.Nt0);
      if (nx0 < G.N0) {
        C a = f[frow + nx0];
        T w = __ldg(G.inv0 + nx0) * s;
        v0.x = a.x * w;
        v0.y = a.y * w;
      }
      if (nx1 < G.N0) {
        C a = f[frow + nx1];
        T w = __ldg(G.inv0 + nx1) * s;
        v1.x = a.x * w;
        v1.y = a.y * w;
      }
    }
    C* out = g + row * G.Nt0 + gx;
    out[0] = v0;
    out[1] = v1;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) crop_apodize_kernel(Grid3<T> G, const typename Cplx<T>::type* __restrict__ g,
                                                           typename Cplx<T>::type* __restrict__ f, int64_t n) {
  using C = typename Cplx<T>::type;
  for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < n; q += int64_t(gridDim.x) * blockDim.x) {
    const int64_t row = q / G.N0;
    const int nx = int(q - row * G.N0);
    const int ny = int(row % G.N1);
    const int nz = int(row / G.N1);
    const int gx = wrap_once(nx - G.N0 / 2, G.Nt0);
    const int gy = wrap_once(ny - G.N1 / 2, G.Nt1);
    const int gz = wrap_once(nz - G.N2 / 2, G.Nt2);
    C a = g[gx + int64_t(G.Nt0) * (gy + int64_t(G.Nt1) * gz)];
    const T w = __ldg(G.inv0 + nx) * __ldg(G.inv1 + ny) * __ldg(G.inv2 + nz);
    C r;
    r.x = a.x * w;
    r.y = a.y * w;
    f[q] = r;
  }
}

template <typename T> Grid3<T> make_grid3(const nfft_plan* p) {
  Grid3<T> G;
  G.N0 = int(p->N[0]);
  G.N1 = int(p->N[1]);
  G.N2 = int(p->N[2]);
  G.Nt0 = int(p->Nt[0]);
  G.Nt1 = int(p->Nt[1]);
  G.Nt2 = int(p->Nt[2]);
  const T* inv = static_cast<const T*>(p->cur_center ? p->inv_c : p->inv);
  G.inv0 = inv;
  // singleton dimensions read the "one" entry stored after the real factors
  const T* one = inv + (p->N[0] + (p->D > 1 ? p->N[1] : 0) + (p->D > 2 ? p->N[2] : 0));
  G.inv1 = p->D > 1 ? inv + p->N[0] : one;
  G.inv2 = p->D > 2 ? inv + p->N[0] + p->N[1] : one;
  return G;
}

unsigned grid_for(int64_t work) {
  int64_t b = (work + 255) / 256;
  const int64_t cap = 152 * 32;
  if (b > cap) b = cap;
  return unsigned(b < 1 ? 1 : b);
}

template <typename T> int pad_t(const nfft_plan* p, const void* f, void* g) {
  Grid3<T> G = make_grid3<T>(p);
  const int64_t npairs = p->Nt[0] * p->Nt[1] * p->Nt[2] / 2;
  using C = typename Cplx<T>::type;
  pad_apodize_kernel<T><<<grid_for(npairs), 256, 0, p->stream>>>(G, static_cast<const C*>(f), static_cast<C*>(g),
                                                                  npairs);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

template <typename T> int crop_t(const nfft_plan* p, const void* g, void* f) {
  Grid3<T> G = make_grid3<T>(p);
  const int64_t n = p->N[0] * p->N[1] * p->N[2];
  using C = typename Cplx<T>::type;
  crop_apodize_kernel<T><<<grid_for(n), 256, 0, p->stream>>>(G, static_cast<const C*>(g), static_cast<C*>(f), n);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

template <typename T> __global__ void real_to_complex_kernel(const T* __restrict__ in, T* __restrict__ out, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    out[2 * i] = in[i];
    out[2 * i + 1] = T(0);
  }
}

template <typename T> __global__ void real_part_kernel(const T* __restrict__ in, T* __restrict__ out, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    out[i] = in[2 * i];
}

}  // namespace

// Real arrays of the optional convolve interface (the sampling-density
// client) go through these conversions around the complex kernels.
int launch_real_to_complex(const nfft_plan* p, const void* in, void* out, int64_t n) {
  if (n == 0) return NFFT_OK;
  if (p->precision == 32)
    real_to_complex_kernel<float><<<grid_for(n), 256, 0, p->stream>>>(static_cast<const float*>(in), static_cast<float*>(out), n);
  else
    real_to_complex_kernel<double><<<grid_for(n), 256, 0, p->stream>>>(static_cast<const double*>(in), static_cast<double*>(out), n);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

int launch_real_part(const nfft_plan* p, const void* in, void* out, int64_t n) {
  if (n == 0) return NFFT_OK;
  if (p->precision == 32)
    real_part_kernel<float><<<grid_for(n), 256, 0, p->stream>>>(static_cast<const float*>(in), static_cast<float*>(out), n);
  else
    real_part_kernel<double><<<grid_for(n), 256, 0, p->stream>>>(static_cast<const double*>(in), static_cast<double*>(out), n);
  NFFT_LAUNCH_CHECK();
  return NFFT_OK;
}

int launch_pad_apodize(const nfft_plan* p, const void* f, void* g) {
  return p->precision == 32 ? pad_t<float>(p, f, g) : pad_t<double>(p, f, g);
}

int launch_crop_apodize(const nfft_plan* p, const void* g, void* f) {
  return p->precision == 32 ? crop_t<float>(p, g, f) : crop_t<double>(p, g, f);
}

}  // namespace nfft
