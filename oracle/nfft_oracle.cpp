// Oracle: CPU restatement of NFFT.jl's blocked NFFT convolution and of its
// direct NDFT.  TEST INFRASTRUCTURE ONLY: it is loaded by tests/, by
// __graft_entry__.smoke() and by bench.py's CPU-baseline leg, always as the
// checker or as the timed CPU reference, never as part of the GPU product.
//
// Each routine cites the reference file:line it restates (paths relative to
// the NFFT.jl repository root).  Arrays are column-major like Julia: nodes
// k are D x M with the coordinate index fastest, grids have dimension 1
// fastest, complex values are interleaved (re, im).
//
// The restatement treats D < 3 as 3-D with singleton trailing dimensions
// (one tap of weight 1, block size 1, no padding), which leaves the sums
// unchanged.
#include <cstdint>
#include <cstring>
#include <cmath>
#include <cfloat>
#include <vector>
#include <limits>
#include <cstdlib>
#include <algorithm>
#include <omp.h>

namespace {

constexpr double PI = 3.14159265358979323846;

// Window modes (how per-tap window values are obtained).
enum { MODE_POLY = 0, MODE_LINEAR = 1, MODE_EXACT = 2 };
// Window ids, matching the C-ABI enum.
enum { WIN_KB = 0, WIN_GAUSS = 1, WIN_SPLINE = 2, WIN_KB_REV = 3, WIN_COSH = 4 };

// Modified Bessel I0 from its power series (FP64); used by the exact
// kaiser_bessel_rev window (src/windowFunctions.jl:41-49).
double bessel_i0(double x) {
  double q = 0.25 * x * x, term = 1.0, sum = 1.0;
  for (int k = 1; k < 500; ++k) {
    term *= q / (double(k) * double(k));
    sum += term;
    if (term < 1e-17 * sum) break;
  }
  return sum;
}

// Cardinal B-spline, src/windowFunctions.jl:75-87.
double cbspline(int m, double k) {
  if (m == 1) return (k >= 0 && k < 1) ? 1.0 : 0.0;
  return k / (m - 1) * cbspline(m - 1, k) + (m - k) / (m - 1) * cbspline(m - 1, k - 1);
}

// Window functions phi(x, Ntilde, m, sigma), src/windowFunctions.jl:21-134.
double window_phi(int win, double k, double Nt, int m, double sigma) {
  const double ak = std::fabs(k), mbyN = m / Nt;
  switch (win) {
    case WIN_KB: {  // :21-34
      const double b = PI * (2.0 - 1.0 / sigma);
      if (ak < mbyN) {
        const double arg = std::sqrt(double(m) * m - Nt * Nt * k * k);
        return std::sinh(b * arg) / (arg * PI);
      } else if (ak > mbyN) {
        return 0.0;
      }
      return b / PI;
    }
    case WIN_GAUSS: {  // :60-68
      const double b = m / PI;
      if (ak < mbyN) return 1.0 / std::sqrt(PI * b) * std::exp(-(Nt * k) * (Nt * k) / b);
      return 0.0;
    }
    case WIN_SPLINE:  // :89-96
      if (ak < mbyN) return cbspline(2 * m, Nt * k + m);
      return 0.0;
    case WIN_KB_REV: {  // :41-49
      const double b = PI * (2.0 - 1.0 / sigma);
      if (ak < mbyN) {
        const double r = Nt * k / m;
        return 0.5 / m * bessel_i0(m * b * std::sqrt(1.0 - r * r));
      }
      return 0.0;
    }
    case WIN_COSH: {  // :104-116
      const double beta = PI * m * (2.0 - 1.0 / sigma);
      if (ak < mbyN) {
        const double arg = (Nt * k) / m;
        const double alpha = std::sqrt(1.0 - arg * arg);
        return 1.0 / (std::cosh(beta) - 1.0) * (std::cosh(beta * alpha) - 1.0) / alpha;
      }
      return 0.0;
    }
  }
  return 0.0;
}

template <typename T> struct Plan {
  int D = 0;
  int64_t Nt[3] = {1, 1, 1};   // oversampled grid (Ntilde)
  int64_t bs[3] = {1, 1, 1};   // block size
  int64_t nb[3] = {1, 1, 1};   // number of blocks per dimension
  int64_t L[3] = {1, 1, 1};    // taps per dimension (2m, or 1 for singleton dims)
  int64_t pad[3] = {0, 0, 0};  // block padding (m, or 0)
  int64_t P[3] = {1, 1, 1};    // padded block extent bs + 2*pad
  int m = 0;
  int64_t M = 0;
  int64_t nblocks = 0;
  std::vector<int64_t> block_start;  // nblocks+1, CSR of nodesInBlock
  std::vector<int64_t> nodes;        // M node ids in block order (stable)
  std::vector<int64_t> trunc;        // 3 x M, original order: trunc(k_shift * Ntilde)
  std::vector<int64_t> bin;          // M, original order: linear block id
  std::vector<T> win;                // (3 * Lmax) x M in block order (window tensor)
  int64_t Lmax = 1;
};

// Horner evaluation in FP64 of a polynomial whose coefficients were stored
// in T, as Julia's evalpoly does after promotion (src/precomputation.jl:206-216).
inline double evalpoly(double x, const double* c, int n) {
  double ex = c[n - 1];
  for (int i = n - 2; i >= 0; --i) ex = x * ex + c[i];
  return ex;
}

// Per-node, per-dimension offset for the polynomial argument, mirroring the
// mixed-precision expression `kscale - off - m + 1 - 0.5` of
// src/precomputation.jl:538-541 and :580-582 (T arithmetic up to the FP64
// literal 0.5).
template <typename T> inline double poly_arg(T kscale, int64_t off, int m) {
  T a = kscale - T(off);
  a = a - T(m);
  a = a + T(1);
  return double(a) - 0.5;
}

template <typename T>
Plan<T>* plan_new(int D, const int64_t* Nt, int m, const int64_t* bs, int64_t M, const T* k,
                  int mode, const double* coeffs, const double* lut, int64_t lut_size, int window,
                  double sigma) {
  auto* p = new Plan<T>();
  p->D = D;
  p->m = m;
  p->M = M;
  for (int d = 0; d < D; ++d) {
    p->Nt[d] = Nt[d];
    p->bs[d] = bs[d];
    p->nb[d] = (Nt[d] + bs[d] - 1) / bs[d];  // ceil(Ntilde/blockSize), :490
    p->L[d] = 2 * m;
    p->pad[d] = m;
    p->P[d] = bs[d] + 2 * m;  // blockSizePadded, :491
  }
  p->nblocks = p->nb[0] * p->nb[1] * p->nb[2];
  p->Lmax = 2 * m;

  // shiftNodes! (src/utils.jl:32-44) then the block index
  // unsafe_trunc(Int, k*Ntilde) ÷ blockSize (src/precomputation.jl:495-503).
  p->trunc.assign(3 * M, 0);
  p->bin.assign(M, 0);
  std::vector<T> kscale(3 * M, T(0));
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < M; ++j) {
    int64_t b[3] = {0, 0, 0};
    for (int d = 0; d < D; ++d) {
      T x = k[d + int64_t(D) * j];
      if (x < T(0)) x += T(1);
      if (x == T(1)) x -= std::numeric_limits<T>::epsilon();
      T ks = x * T(Nt[d]);
      int64_t t = int64_t(ks);  // trunc toward zero; ks >= 0
      if (t >= Nt[d]) t = Nt[d] - 1;  // guard: k_shift*Ntilde rounded up to Ntilde
      kscale[3 * j + d] = ks;
      p->trunc[3 * j + d] = t;
      b[d] = t / bs[d];
    }
    p->bin[j] = b[0] + p->nb[0] * (b[1] + p->nb[1] * b[2]);
  }
  // Two-pass count + push: nodes of a block stay in input order (:494-504).
  p->block_start.assign(p->nblocks + 1, 0);
  for (int64_t j = 0; j < M; ++j) p->block_start[p->bin[j] + 1]++;
  for (int64_t b = 0; b < p->nblocks; ++b) p->block_start[b + 1] += p->block_start[b];
  p->nodes.assign(M, 0);
  {
    std::vector<int64_t> fill(p->block_start.begin(), p->block_start.end() - 1);
    for (int64_t j = 0; j < M; ++j) p->nodes[fill[p->bin[j]]++] = j;
  }

  // Window tensor in block order: _precomputeWindowTensor (:556-591) for the
  // polynomial, shiftedWindowEntries (:168-190) for the linear LUT, the
  // window function itself (:130-136) for the exact mode.
  const int64_t Lm = p->Lmax;
  p->win.assign(size_t(3 * Lm) * size_t(M), T(0));
  const int deg = 2 * m + 1;
  const double scale = (mode == MODE_LINEAR) ? double(lut_size / m) : 0.0;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < M; ++i) {
    const int64_t j = p->nodes[i];
    T* w = &p->win[size_t(3 * Lm) * size_t(i)];
    for (int d = 0; d < 3; ++d) {
      if (d >= D) { w[d * Lm] = T(1); continue; }
      const T ks = kscale[3 * j + d];
      const int64_t t = p->trunc[3 * j + d];
      if (mode == MODE_POLY) {
        const double x = poly_arg<T>(ks, t - m + 1, m);
        for (int l = 0; l < 2 * m; ++l) w[d * Lm + l] = T(evalpoly(x, coeffs + size_t(deg) * l, deg));
      } else if (mode == MODE_LINEAR) {
        // idx = (kscale - off) * (LUTSize ÷ m), :543-545
        const int64_t off = t - m + 1;
        const double idx = double(T(ks - T(off))) * scale;
        const double fi = std::floor(idx);
        const int64_t ii = int64_t(fi);
        const double a = idx - fi;
        const int64_t sc = lut_size / m;
        for (int l = 0; l < 2 * m; ++l) {
          const int64_t i1 = std::llabs(ii - l * sc);
          const int64_t i2 = std::llabs(ii - l * sc + 1);
          w[d * Lm + l] = T(lut[i1] + a * (lut[i2] - lut[i1]));
        }
      } else {
        const int64_t off = t - m + 1;
        for (int l = 0; l < 2 * m; ++l) {
          const double x = (double(ks) - double(off + l)) / double(Nt[d]);
          w[d * Lm + l] = T(window_phi(window, x, double(Nt[d]), m, sigma));
        }
      }
    }
  }
  return p;
}

// convolve_blocking!: toBlock! + calcOneNode! per block
// (src/convolution.jl:229-344).
template <typename T> void convolve(const Plan<T>* p, const T* g, T* fhat) {
  const int64_t P0 = p->P[0], P1 = p->P[1], P2 = p->P[2];
  const int64_t Lm = p->Lmax;
#pragma omp parallel
  {
    std::vector<T> block(size_t(2) * P0 * P1 * P2);
#pragma omp for schedule(dynamic, 1)
    for (int64_t b = 0; b < p->nblocks; ++b) {
      const int64_t s = p->block_start[b], e = p->block_start[b + 1];
      if (s == e) continue;
      const int64_t bi[3] = {b % p->nb[0], (b / p->nb[0]) % p->nb[1], b / (p->nb[0] * p->nb[1])};
      int64_t off[3];
      for (int d = 0; d < 3; ++d) off[d] = bi[d] * p->bs[d] - p->pad[d];
      // toBlock!: block[i] = g[(i + b*bs - m) mod Ntilde] (:248-299)
      for (int64_t i2 = 0; i2 < P2; ++i2) {
        const int64_t g2 = ((i2 + off[2]) % p->Nt[2] + p->Nt[2]) % p->Nt[2];
        for (int64_t i1 = 0; i1 < P1; ++i1) {
          const int64_t g1 = ((i1 + off[1]) % p->Nt[1] + p->Nt[1]) % p->Nt[1];
          for (int64_t i0 = 0; i0 < P0; ++i0) {
            const int64_t g0 = ((i0 + off[0]) % p->Nt[0] + p->Nt[0]) % p->Nt[0];
            const int64_t gi = g0 + p->Nt[0] * (g1 + p->Nt[1] * g2);
            const int64_t li = i0 + P0 * (i1 + P1 * i2);
            block[2 * li] = g[2 * gi];
            block[2 * li + 1] = g[2 * gi + 1];
          }
        }
      }
      for (int64_t i = s; i < e; ++i) {
        const int64_t j = p->nodes[i];
        const T* w = &p->win[size_t(3 * Lm) * size_t(i)];
        int64_t base[3];
        for (int d = 0; d < 3; ++d) base[d] = p->trunc[3 * j + d] - p->m + 1 + p->pad[d] - bi[d] * p->bs[d];
        for (int d = p->D; d < 3; ++d) base[d] = 0;
        // calcOneNode!: nested separable sum, innermost over dim 1 (:315-344)
        T r3 = 0, i3 = 0;
        for (int64_t l2 = 0; l2 < p->L[2]; ++l2) {
          T r2 = 0, i2v = 0;
          for (int64_t l1 = 0; l1 < p->L[1]; ++l1) {
            T r1 = 0, i1v = 0;
            const int64_t row = P0 * ((base[1] + l1) + P1 * (base[2] + l2));
            for (int64_t l0 = 0; l0 < p->L[0]; ++l0) {
              const int64_t li = base[0] + l0 + row;
              r1 += w[l0] * block[2 * li];
              i1v += w[l0] * block[2 * li + 1];
            }
            r2 += w[Lm + l1] * r1;
            i2v += w[Lm + l1] * i1v;
          }
          r3 += w[2 * Lm + l2] * r2;
          i3 += w[2 * Lm + l2] * i2v;
        }
        fhat[2 * j] = r3;
        fhat[2 * j + 1] = i3;
      }
    }
  }
}

// _convolve_transpose_blocking!: private block fill (fillOneNode!) and a
// locked wrap-add into g (addBlock!), src/convolution.jl:356-520.
template <typename T> void convolve_transpose(const Plan<T>* p, const T* fhat, T* g) {
  const int64_t P0 = p->P[0], P1 = p->P[1], P2 = p->P[2];
  const int64_t Lm = p->Lmax;
  const int64_t ng = p->Nt[0] * p->Nt[1] * p->Nt[2];
  std::memset(g, 0, sizeof(T) * 2 * size_t(ng));
#pragma omp parallel
  {
    std::vector<T> block(size_t(2) * P0 * P1 * P2);
#pragma omp for schedule(dynamic, 1)
    for (int64_t b = 0; b < p->nblocks; ++b) {
      const int64_t s = p->block_start[b], e = p->block_start[b + 1];
      if (s == e) continue;
      std::fill(block.begin(), block.end(), T(0));
      const int64_t bi[3] = {b % p->nb[0], (b / p->nb[0]) % p->nb[1], b / (p->nb[0] * p->nb[1])};
      for (int64_t i = s; i < e; ++i) {
        const int64_t j = p->nodes[i];
        const T* w = &p->win[size_t(3 * Lm) * size_t(i)];
        int64_t base[3];
        for (int d = 0; d < 3; ++d) base[d] = p->trunc[3 * j + d] - p->m + 1 + p->pad[d] - bi[d] * p->bs[d];
        for (int d = p->D; d < 3; ++d) base[d] = 0;
        const T fr = fhat[2 * j], fi = fhat[2 * j + 1];
        // fillOneNode!: innerWin = w1 .* fHat, prodWin = product of outer windows
        for (int64_t l2 = 0; l2 < p->L[2]; ++l2) {
          const T pw2 = w[2 * Lm + l2];
          for (int64_t l1 = 0; l1 < p->L[1]; ++l1) {
            const T pw1 = pw2 * w[Lm + l1];
            const int64_t row = P0 * ((base[1] + l1) + P1 * (base[2] + l2));
            for (int64_t l0 = 0; l0 < p->L[0]; ++l0) {
              const int64_t li = base[0] + l0 + row;
              block[2 * li] += (w[l0] * fr) * pw1;
              block[2 * li + 1] += (w[l0] * fi) * pw1;
            }
          }
        }
      }
      int64_t off[3];
      for (int d = 0; d < 3; ++d) off[d] = bi[d] * p->bs[d] - p->pad[d];
      // addBlock! under the plan-wide lock (:371-373, :379-443)
#pragma omp critical(nfft_oracle_addblock)
      for (int64_t i2 = 0; i2 < P2; ++i2) {
        const int64_t g2 = ((i2 + off[2]) % p->Nt[2] + p->Nt[2]) % p->Nt[2];
        for (int64_t i1 = 0; i1 < P1; ++i1) {
          const int64_t g1 = ((i1 + off[1]) % p->Nt[1] + p->Nt[1]) % p->Nt[1];
          for (int64_t i0 = 0; i0 < P0; ++i0) {
            const int64_t g0 = ((i0 + off[0]) % p->Nt[0] + p->Nt[0]) % p->Nt[0];
            const int64_t gi = g0 + p->Nt[0] * (g1 + p->Nt[1] * g2);
            const int64_t li = i0 + P0 * (i1 + P1 * i2);
            g[2 * gi] += block[2 * li];
            g[2 * gi + 1] += block[2 * li + 1];
          }
        }
      }
    }
  }
}

// Deconvolution with zero padding, _deconvolve_alloc_free!
// (src/deconvolution.jl:22-45): g[(n - N÷2) mod Ntilde] = f[n] * prod invphihat.
template <typename T>
void deconvolve(int D, const int64_t* N, const int64_t* Nt, const T* const* inv, const T* f, T* g) {
  int64_t n3[3] = {1, 1, 1}, t3[3] = {1, 1, 1};
  for (int d = 0; d < D; ++d) { n3[d] = N[d]; t3[d] = Nt[d]; }
  const int64_t ng = t3[0] * t3[1] * t3[2];
  std::memset(g, 0, sizeof(T) * 2 * size_t(ng));
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t i2 = 0; i2 < n3[2]; ++i2)
    for (int64_t i1 = 0; i1 < n3[1]; ++i1) {
      const int64_t g2 = (i2 - n3[2] / 2 + t3[2]) % t3[2];
      const int64_t g1 = (i1 - n3[1] / 2 + t3[1]) % t3[1];
      T s12 = T(1);
      if (D > 1) s12 *= inv[1][i1];
      if (D > 2) s12 *= inv[2][i2];
      for (int64_t i0 = 0; i0 < n3[0]; ++i0) {
        const int64_t g0 = (i0 - n3[0] / 2 + t3[0]) % t3[0];
        const int64_t fi = i0 + n3[0] * (i1 + n3[1] * i2);
        const int64_t gi = g0 + t3[0] * (g1 + t3[1] * g2);
        T v0 = f[2 * fi] * inv[0][i0], v1 = f[2 * fi + 1] * inv[0][i0];
        g[2 * gi] = v0 * s12;
        g[2 * gi + 1] = v1 * s12;
      }
    }
}

// Cropping deconvolution, _deconvolve_transpose_alloc_free!
// (src/deconvolution.jl:69-92).
template <typename T>
void deconvolve_transpose(int D, const int64_t* N, const int64_t* Nt, const T* const* inv, const T* g, T* f) {
  int64_t n3[3] = {1, 1, 1}, t3[3] = {1, 1, 1};
  for (int d = 0; d < D; ++d) { n3[d] = N[d]; t3[d] = Nt[d]; }
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t i2 = 0; i2 < n3[2]; ++i2)
    for (int64_t i1 = 0; i1 < n3[1]; ++i1) {
      const int64_t g2 = (i2 - n3[2] / 2 + t3[2]) % t3[2];
      const int64_t g1 = (i1 - n3[1] / 2 + t3[1]) % t3[1];
      T s12 = T(1);
      if (D > 1) s12 *= inv[1][i1];
      if (D > 2) s12 *= inv[2][i2];
      for (int64_t i0 = 0; i0 < n3[0]; ++i0) {
        const int64_t g0 = (i0 - n3[0] / 2 + t3[0]) % t3[0];
        const int64_t fi = i0 + n3[0] * (i1 + n3[1] * i2);
        const int64_t gi = g0 + t3[0] * (g1 + t3[1] * g2);
        T v0 = g[2 * gi] * inv[0][i0], v1 = g[2 * gi + 1] * inv[0][i0];
        f[2 * fi] = v0 * s12;
        f[2 * fi + 1] = v1 * s12;
      }
    }
}

}  // namespace

extern "C" {

int oracle_num_threads() { return omp_get_max_threads(); }
void oracle_set_num_threads(int n) { omp_set_num_threads(n); }

double oracle_window_phi(int win, double x, double Nt, int m, double sigma) {
  return window_phi(win, x, Nt, m, sigma);
}

#define ORACLE_API(SUF, T)                                                                         \
  void* oracle_plan_new_##SUF(int D, const int64_t* Nt, int m, const int64_t* bs, int64_t M,        \
                              const T* k, int mode, const double* coeffs, const double* lut,        \
                              int64_t lut_size, int window, double sigma) {                         \
    return plan_new<T>(D, Nt, m, bs, M, k, mode, coeffs, lut, lut_size, window, sigma);             \
  }                                                                                                \
  void oracle_plan_free_##SUF(void* p) { delete static_cast<Plan<T>*>(p); }                         \
  int64_t oracle_plan_nblocks_##SUF(void* p) { return static_cast<Plan<T>*>(p)->nblocks; }          \
  void oracle_plan_blocks_##SUF(void* vp, int64_t* block_start, int64_t* nodes, int64_t* bin,       \
                                int64_t* trunc) {                                                  \
    auto* p = static_cast<Plan<T>*>(vp);                                                           \
    std::memcpy(block_start, p->block_start.data(), sizeof(int64_t) * (p->nblocks + 1));           \
    std::memcpy(nodes, p->nodes.data(), sizeof(int64_t) * p->M);                                   \
    std::memcpy(bin, p->bin.data(), sizeof(int64_t) * p->M);                                       \
    for (int64_t j = 0; j < p->M; ++j)                                                             \
      for (int d = 0; d < p->D; ++d) trunc[d + p->D * j] = p->trunc[3 * j + d];                    \
  }                                                                                                \
  void oracle_convolve_##SUF(void* p, const T* g, T* fhat) {                                       \
    convolve<T>(static_cast<Plan<T>*>(p), g, fhat);                                                \
  }                                                                                                \
  void oracle_convolve_transpose_##SUF(void* p, const T* fhat, T* g) {                             \
    convolve_transpose<T>(static_cast<Plan<T>*>(p), fhat, g);                                      \
  }                                                                                                \
  void oracle_deconvolve_##SUF(int D, const int64_t* N, const int64_t* Nt, const T* inv0,          \
                               const T* inv1, const T* inv2, const T* f, T* g) {                    \
    const T* inv[3] = {inv0, inv1, inv2};                                                          \
    deconvolve<T>(D, N, Nt, inv, f, g);                                                            \
  }                                                                                                \
  void oracle_deconvolve_transpose_##SUF(int D, const int64_t* N, const int64_t* Nt,               \
                                         const T* inv0, const T* inv1, const T* inv2, const T* g,  \
                                         T* f) {                                                   \
    const T* inv[3] = {inv0, inv1, inv2};                                                          \
    deconvolve_transpose<T>(D, N, Nt, inv, g, f);                                                  \
  }

ORACLE_API(f32, float)
ORACLE_API(f64, double)

// Direct NDFT forward on a subset of nodes, src/direct.jl:99-123:
// fhat[j] = sum_n f[n] exp(-2 pi i k_j . (n - N÷2)).  The D-dimensional sum
// is factored dimension by dimension (separable phases), in FP64.
void oracle_ndft_forward(int D, const int64_t* N, int64_t Msel, const double* k, const double* f,
                         double* out) {
  int64_t n3[3] = {1, 1, 1};
  for (int d = 0; d < D; ++d) n3[d] = N[d];
#pragma omp parallel
  {
    std::vector<double> ph[3];
    for (int d = 0; d < 3; ++d) ph[d].resize(2 * n3[d]);
    std::vector<double> acc1(2 * n3[1] * n3[2]);
#pragma omp for schedule(dynamic, 1)
    for (int64_t j = 0; j < Msel; ++j) {
      for (int d = 0; d < 3; ++d) {
        for (int64_t n = 0; n < n3[d]; ++n) {
          if (d >= D) { ph[d][2 * n] = 1.0; ph[d][2 * n + 1] = 0.0; continue; }
          const double arg = -2.0 * PI * k[d + D * j] * double(n - n3[d] / 2);
          ph[d][2 * n] = std::cos(arg);
          ph[d][2 * n + 1] = std::sin(arg);
        }
      }
      double sr = 0, si = 0;
      for (int64_t i2 = 0; i2 < n3[2]; ++i2) {
        double r2 = 0, q2 = 0;
        for (int64_t i1 = 0; i1 < n3[1]; ++i1) {
          const double* fr = f + 2 * n3[0] * (i1 + n3[1] * i2);
          double r1 = 0, q1 = 0;
          for (int64_t i0 = 0; i0 < n3[0]; ++i0) {
            const double a = fr[2 * i0], b = fr[2 * i0 + 1];
            const double c = ph[0][2 * i0], s = ph[0][2 * i0 + 1];
            r1 += a * c - b * s;
            q1 += a * s + b * c;
          }
          const double c = ph[1][2 * i1], s = ph[1][2 * i1 + 1];
          r2 += r1 * c - q1 * s;
          q2 += r1 * s + q1 * c;
        }
        const double c = ph[2][2 * i2], s = ph[2][2 * i2 + 1];
        sr += r2 * c - q2 * s;
        si += r2 * s + q2 * c;
      }
      out[2 * j] = sr;
      out[2 * j + 1] = si;
    }
  }
}

// Direct adjoint NDFT at selected output indices (linear, column-major),
// src/direct.jl:126-151: f[n] = sum_j fhat[j] exp(+2 pi i k_j . (n - N÷2)).
void oracle_ndft_adjoint(int D, const int64_t* N, int64_t M, const double* k, const double* fhat,
                         int64_t nsel, const int64_t* sel, double* out) {
  int64_t n3[3] = {1, 1, 1};
  for (int d = 0; d < D; ++d) n3[d] = N[d];
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t s = 0; s < nsel; ++s) {
    const int64_t li = sel[s];
    double fr[3] = {0, 0, 0};
    fr[0] = double(li % n3[0] - n3[0] / 2);
    fr[1] = double((li / n3[0]) % n3[1] - n3[1] / 2);
    fr[2] = double(li / (n3[0] * n3[1]) - n3[2] / 2);
    double sr = 0, si = 0;
    for (int64_t j = 0; j < M; ++j) {
      double arg = 0;
      for (int d = 0; d < D; ++d) arg += k[d + D * j] * fr[d];
      const double a = 2.0 * PI * arg;
      const double c = std::cos(a), sn = std::sin(a);
      const double x = fhat[2 * j], y = fhat[2 * j + 1];
      sr += x * c - y * sn;
      si += x * sn + y * c;
    }
    out[2 * s] = sr;
    out[2 * s + 1] = si;
  }
}

}  // extern "C"
