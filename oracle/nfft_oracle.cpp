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
}  // extern "C"

// Direct NDFT forward on a subset of nodes, src/direct.jl:99-123:
// fhat[j] = sum_n f[n] exp(-2 pi i k_j . (n - N÷2)), in FP64.
//
// The D-dimensional sum is contracted one (virtual) dimension at a time with
// per-node phase tables (separable phases).  A dimension longer than 4096 is
// split into two virtual dimensions n = v + B u (B = 2048), whose phases are
// exp(-2 pi i k (v - N÷2)) and exp(-2 pi i k B u), so a 1-D image of 2^22
// points needs tables of 2 x 2048 entries per node.  Nodes are processed in
// blocks of 8 so that each image row is read once per block.
namespace {

constexpr int kMaxV = 6;

struct VDims {
  int nv = 0;
  int64_t n[kMaxV];      // virtual extents, fastest first
  int dim[kMaxV];        // source dimension of the virtual dimension
  double scale[kMaxV];   // image coordinate = scale * i + off
  double off[kMaxV];
};

// Split the image dimensions into virtual dimensions of at most `maxlen` points
// (a longer extent must be divisible by the chosen base).
VDims make_vdims(int D, const int64_t* N, int64_t maxlen, int64_t base) {
  VDims V;
  for (int d = 0; d < D; ++d) {
    int64_t rest = N[d];
    double sc = 1.0, of = -double(N[d] / 2);
    while (rest > maxlen && rest % base == 0) {
      V.n[V.nv] = base; V.dim[V.nv] = d; V.scale[V.nv] = sc; V.off[V.nv] = of; ++V.nv;
      sc *= double(base); of = 0.0; rest /= base;
    }
    V.n[V.nv] = rest; V.dim[V.nv] = d; V.scale[V.nv] = sc; V.off[V.nv] = of; ++V.nv;
  }
  return V;
}

// exp(sign 2 pi i x t) for t = scale*i + off, i = 0..n-1, written to (c[i*stride], s[i*stride]).
// Exact seeds every 32 entries (fractional part of x*t formed with an FMA
// residual), complex multiplication by exp(sign 2 pi i x scale) in between
// (relative error below 1e-14).
void phase_table(double x, double sign, double scale, double off, int64_t n, double* c, double* s, int64_t stride) {
  auto seed = [&](double t, double& cr, double& ci) {
    const double p = x * t;
    const double e = std::fma(x, t, -p);
    const double fr = (p - std::nearbyint(p)) + e;
    cr = std::cos(2.0 * PI * fr);
    ci = sign * std::sin(2.0 * PI * fr);
  };
  double wr, wi;
  seed(scale, wr, wi);
  for (int64_t i0 = 0; i0 < n; i0 += 32) {
    double cr, ci;
    seed(scale * double(i0) + off, cr, ci);
    const int64_t i1 = std::min<int64_t>(n, i0 + 32);
    for (int64_t i = i0; i < i1; ++i) {
      c[i * stride] = cr;
      s[i * stride] = ci;
      const double t = cr * wr - ci * wi;
      ci = cr * wi + ci * wr;
      cr = t;
    }
  }
}

}  // namespace

extern "C" {
void oracle_ndft_forward(int D, const int64_t* N, int64_t Msel, const double* k, const double* f,
                         double* out) {
  constexpr int NB = 8;
  const VDims V = make_vdims(D, N, 4096, 2048);
  int64_t rows = 1;
  for (int v = 1; v < V.nv; ++v) rows *= V.n[v];
  const int64_t n0 = V.n[0];
  const int64_t nblk = (Msel + NB - 1) / NB;
#pragma omp parallel
  {
    std::vector<double> tc[kMaxV], ts[kMaxV];
    for (int v = 0; v < V.nv; ++v) {
      tc[v].assign(V.n[v] * NB, 0.0);
      ts[v].assign(V.n[v] * NB, 0.0);
    }
#pragma omp for schedule(dynamic, 1)
    for (int64_t b = 0; b < nblk; ++b) {
      const int64_t j0 = b * NB;
      const int nb = int(std::min<int64_t>(NB, Msel - j0));
      for (int v = 0; v < V.nv; ++v)
        for (int jj = 0; jj < NB; ++jj) {
          if (jj < nb) {
            phase_table(k[V.dim[v] + int64_t(D) * (j0 + jj)], -1.0, V.scale[v], V.off[v], V.n[v],
                        tc[v].data() + jj, ts[v].data() + jj, NB);
          } else {
            for (int64_t i = 0; i < V.n[v]; ++i) tc[v][i * NB + jj] = ts[v][i * NB + jj] = 0.0;
          }
        }
      // acc[v] holds the partial sum over virtual dimensions < v of the current row
      double ar[kMaxV][NB] = {}, ai[kMaxV][NB] = {};
      int64_t idx[kMaxV] = {};
      for (int64_t r = 0; r < rows; ++r) {
        const double* fr = f + 2 * n0 * r;
        double r1[NB] = {}, q1[NB] = {};
        for (int64_t i0 = 0; i0 < n0; ++i0) {
          const double a = fr[2 * i0], bb = fr[2 * i0 + 1];
          const double* cc = &tc[0][i0 * NB];
          const double* ss = &ts[0][i0 * NB];
          for (int jj = 0; jj < NB; ++jj) {
            r1[jj] += a * cc[jj] - bb * ss[jj];
            q1[jj] += a * ss[jj] + bb * cc[jj];
          }
        }
        for (int jj = 0; jj < NB; ++jj) {
          ar[0][jj] = r1[jj];
          ai[0][jj] = q1[jj];
        }
        // fold level v into level v+1 while the odometer wraps
        int v = 1;
        for (; v < V.nv; ++v) {
          const double* cc = &tc[v][idx[v] * NB];
          const double* ss = &ts[v][idx[v] * NB];
          for (int jj = 0; jj < NB; ++jj) {
            ar[v][jj] += ar[v - 1][jj] * cc[jj] - ai[v - 1][jj] * ss[jj];
            ai[v][jj] += ar[v - 1][jj] * ss[jj] + ai[v - 1][jj] * cc[jj];
            ar[v - 1][jj] = ai[v - 1][jj] = 0.0;
          }
          if (++idx[v] < V.n[v]) break;
          idx[v] = 0;
        }
      }
      const int top = V.nv - 1;
      for (int jj = 0; jj < nb; ++jj) {
        out[2 * (j0 + jj)] = ar[top][jj];
        out[2 * (j0 + jj) + 1] = ai[top][jj];
      }
    }
  }
}

// Direct adjoint NDFT at selected outputs, src/direct.jl:126-151:
// f[n] = sum_j fhat[j] exp(+2 pi i k_j . (n - N÷2)) for the column-major
// linear indices sel, in FP64.  The phase of a (node, output) pair is a
// product of per-node table entries, one per virtual dimension of at most
// 256 points (n = v + 256 u + 256^2 w ...), so each pair costs a few complex
// products.  Threads take blocks of 64 nodes, build the blocks' tables
// (node index fastest) and add every selected output's sum over the block
// to a private accumulator; the accumulators are added in thread order.
void oracle_ndft_adjoint_sel(int D, const int64_t* N, int64_t M, const double* k, const double* fhat,
                             int64_t nsel, const int64_t* sel, double* out) {
  constexpr int NB = 64;
  const VDims V = make_vdims(D, N, 256, 256);
  std::vector<int32_t> vidx(size_t(nsel) * V.nv);
  for (int64_t s = 0; s < nsel; ++s) {
    int64_t r = sel[s];
    for (int v = 0; v < V.nv; ++v) {
      vidx[s * V.nv + v] = int32_t(r % V.n[v]);
      r /= V.n[v];
    }
  }
  const int nth = omp_get_max_threads();
  std::vector<double> part(size_t(nth) * 2 * nsel, 0.0);
  const int64_t nblk = (M + NB - 1) / NB;
#pragma omp parallel num_threads(nth)
  {
    double* acc = part.data() + size_t(omp_get_thread_num()) * 2 * nsel;
    std::vector<double> tc[kMaxV], ts[kMaxV];
    for (int v = 0; v < V.nv; ++v) {
      tc[v].assign(V.n[v] * NB, 0.0);
      ts[v].assign(V.n[v] * NB, 0.0);
    }
    double hr[NB], hi[NB];
#pragma omp for schedule(static)
    for (int64_t b = 0; b < nblk; ++b) {
      const int64_t j0 = b * NB;
      const int nb = int(std::min<int64_t>(NB, M - j0));
      for (int jj = 0; jj < NB; ++jj) {
        hr[jj] = jj < nb ? fhat[2 * (j0 + jj)] : 0.0;
        hi[jj] = jj < nb ? fhat[2 * (j0 + jj) + 1] : 0.0;
      }
      for (int v = 0; v < V.nv; ++v)
        for (int jj = 0; jj < NB; ++jj) {
          const double x = jj < nb ? k[V.dim[v] + int64_t(D) * (j0 + jj)] : 0.0;
          phase_table(x, 1.0, V.scale[v], V.off[v], V.n[v], tc[v].data() + jj, ts[v].data() + jj, NB);
        }
      // fold the node values into the last table: a pair then costs nv - 1 complex products
      {
        const int v = V.nv - 1;
        for (int64_t i = 0; i < V.n[v]; ++i)
          for (int jj = 0; jj < NB; ++jj) {
            const double c = tc[v][i * NB + jj], sn = ts[v][i * NB + jj];
            tc[v][i * NB + jj] = hr[jj] * c - hi[jj] * sn;
            ts[v][i * NB + jj] = hr[jj] * sn + hi[jj] * c;
          }
      }
      for (int64_t s = 0; s < nsel; ++s) {
        const int32_t* ix = &vidx[s * V.nv];
        double pr[NB], pi[NB];
        {
          const int v = V.nv - 1;
          const double* cc = &tc[v][int64_t(ix[v]) * NB];
          const double* ss = &ts[v][int64_t(ix[v]) * NB];
          for (int jj = 0; jj < NB; ++jj) {
            pr[jj] = cc[jj];
            pi[jj] = ss[jj];
          }
        }
        for (int v = V.nv - 2; v >= 0; --v) {
          const double* cc = &tc[v][int64_t(ix[v]) * NB];
          const double* ss = &ts[v][int64_t(ix[v]) * NB];
          for (int jj = 0; jj < NB; ++jj) {
            const double t = pr[jj] * cc[jj] - pi[jj] * ss[jj];
            pi[jj] = pr[jj] * ss[jj] + pi[jj] * cc[jj];
            pr[jj] = t;
          }
        }
        double sr = 0.0, si = 0.0;
        for (int jj = 0; jj < NB; ++jj) {
          sr += pr[jj];
          si += pi[jj];
        }
        acc[2 * s] += sr;
        acc[2 * s + 1] += si;
      }
    }
  }
  for (int64_t s = 0; s < nsel; ++s) {
    double sr = 0.0, si = 0.0;
    for (int t = 0; t < nth; ++t) {
      sr += part[size_t(t) * 2 * nsel + 2 * s];
      si += part[size_t(t) * 2 * nsel + 2 * s + 1];
    }
    out[2 * s] = sr;
    out[2 * s + 1] = si;
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
