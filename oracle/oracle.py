"""Oracle: CPU restatement of NFFT.jl's NFFT plan (params, windows, deconvolution
factors, blocked convolution, FFT) and of its direct NDFT.

TEST INFRASTRUCTURE ONLY.  This module is imported by ``tests/``, by
``__graft_entry__.smoke()`` and by the CPU-baseline leg of ``bench.py``, always as
the checker (or as the timed CPU reference), never by the GPU product path.

Parity status: the reference is a Julia package and no Julia toolchain exists
here, so no output of the reference itself can be produced.  The restatement is
pinned instead by the reference's own known-answer tests: the NDFT accuracy
tolerances of ``test/accuracy.jl:41-73`` and ``test/gpu.jl:17-50``, the
closed-form sampling-density weights of ``test/samplingDensity.jl:10-27`` and the
published m=4 accuracy of ``benchmark/paper/img/accuracy_m_D2_.tex:36``.

Layout conventions follow Julia: ``k`` has logical shape (D, M); image arrays have
logical shape N and are stored column-major (dimension 1 fastest).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import threading

import numpy as np
import scipy.fft
import scipy.special

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libnfft_oracle.so")
_lib = None
_lib_lock = threading.Lock()

# Precompute flags, AbstractNFFTs/src/misc.jl:13-19
FULL, TENSOR, LINEAR, POLYNOMIAL = 1, 2, 3, 4
WINDOWS = {"kaiser_bessel": 0, "gauss": 1, "spline": 2, "kaiser_bessel_rev": 3, "cosh_type": 4}
_MODE_POLY, _MODE_LINEAR, _MODE_EXACT = 0, 1, 2


def build(force: bool = False) -> str:
    """Compile the C++ restatement with g++/OpenMP into oracle/_build."""
    src = os.path.join(_HERE, "nfft_oracle.cpp")
    if not force and os.path.exists(_LIB_PATH) and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src):
        return _LIB_PATH
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c++17", "-o", tmp, src])
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    with _lib_lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            vp, i64p, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.c_void_p
            for suf in ("f32", "f64"):
                f = getattr(L, f"oracle_plan_new_{suf}")
                f.restype = vp
                f.argtypes = [ctypes.c_int, i64p, ctypes.c_int, i64p, ctypes.c_int64, dp, ctypes.c_int,
                              dp, dp, ctypes.c_int64, ctypes.c_int, ctypes.c_double]
                getattr(L, f"oracle_plan_free_{suf}").argtypes = [vp]
                getattr(L, f"oracle_plan_nblocks_{suf}").restype = ctypes.c_int64
                getattr(L, f"oracle_plan_nblocks_{suf}").argtypes = [vp]
                getattr(L, f"oracle_plan_blocks_{suf}").argtypes = [vp, i64p, i64p, i64p, i64p]
                getattr(L, f"oracle_convolve_{suf}").argtypes = [vp, dp, dp]
                getattr(L, f"oracle_convolve_transpose_{suf}").argtypes = [vp, dp, dp]
                getattr(L, f"oracle_deconvolve_{suf}").argtypes = [ctypes.c_int, i64p, i64p, dp, dp, dp, dp, dp]
                getattr(L, f"oracle_deconvolve_transpose_{suf}").argtypes = [ctypes.c_int, i64p, i64p, dp, dp, dp, dp, dp]
            L.oracle_ndft_forward.argtypes = [ctypes.c_int, i64p, ctypes.c_int64, dp, dp, dp]
            L.oracle_ndft_adjoint.argtypes = [ctypes.c_int, i64p, ctypes.c_int64, dp, dp, ctypes.c_int64, i64p, dp]
            L.oracle_ndft_adjoint_sel.argtypes = [ctypes.c_int, i64p, ctypes.c_int64, dp, dp, ctypes.c_int64, i64p,
                                                  dp]
            L.oracle_window_phi.restype = ctypes.c_double
            L.oracle_window_phi.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_double]
            L.oracle_num_threads.restype = ctypes.c_int
            L.oracle_set_num_threads.argtypes = [ctypes.c_int]
            _lib = L
    return _lib


def _i64(a):
    a = np.ascontiguousarray(a, dtype=np.int64)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


# ---------------------------------------------------------------- parameters

def reltol_to_params(reltol):
    """AbstractNFFTs/src/misc.jl:44-48."""
    w = math.ceil(math.log10(1.0 / reltol)) + 1
    return w // 2, 2.0


def params_to_reltol(m, sigma):
    """AbstractNFFTs/src/misc.jl:50-53."""
    return 10.0 ** (-(2 * m - 1))


def accuracy_params(m=None, sigma=None, reltol=None):
    """accuracyParams, AbstractNFFTs/src/misc.jl:66-81: reltol wins; m and sigma
    are honoured only when both are given; default reltol 1e-9."""
    if reltol is not None:
        m_, s_ = reltol_to_params(reltol)
        return m_, s_, reltol
    if m is not None and sigma is not None:
        return int(m), float(sigma), params_to_reltol(m, sigma)
    reltol = 1e-9
    m_, s_ = reltol_to_params(reltol)
    return m_, s_, reltol


_M2K = [1, 3, 7, 9, 14, 17, 20, 23, 24]


def lut_size(m):
    """LUTSize = 2^K * m with K from the m2K table, src/precomputation.jl:14-17."""
    K = _M2K[min(m + 1, len(_M2K)) - 1]
    return (2 ** K) * m


def oversampled(N, sigma):
    """Ntilde = (ceil(sigma*N) ÷ 2) * 2, src/precomputation.jl:25-27."""
    return tuple((math.ceil(sigma * n) // 2) * 2 for n in N)


def default_block_size(Nt):
    """_blockSize, src/precomputation.jl:59-77."""
    D = len(Nt)
    if D == 1:
        return (min(1024, Nt[0]),)
    if D == 2:
        return tuple(min(64, n) for n in Nt)
    return tuple(min(16, Nt[d]) if d < 3 else 1 for d in range(D))


def init_params(N, m=None, sigma=None, reltol=None, block_size=None):
    """initParams, src/precomputation.jl:3-56 (full-dimensional plans)."""
    m_, s_, r_ = accuracy_params(m, sigma, reltol)
    Nt = oversampled(N, s_)
    s_ = Nt[0] / N[0]  # sigma recomputed from the first dimension, :30
    bs = tuple(block_size) if block_size is not None else default_block_size(Nt)
    return dict(m=m_, sigma=s_, reltol=r_, Nt=Nt, block_size=bs, LUTSize=lut_size(m_))


# ------------------------------------------------------------------ windows

def window_phi(window, x, Nt, m, sigma):
    """phi for one window, scalar FP64 (src/windowFunctions.jl)."""
    return lib().oracle_window_phi(WINDOWS[window], float(x), float(Nt), int(m), float(sigma))


def window_hat(window, n, Nt, m, sigma):
    """phi-hat, vectorised FP64 (src/windowFunctions.jl:36-134)."""
    n = np.asarray(n, dtype=np.float64)
    pi = np.pi
    if window == "kaiser_bessel":  # :36-39
        b = pi * (2 - 1 / sigma)
        return scipy.special.i0(m * np.sqrt(b * b - (2 * pi * n / Nt) ** 2))
    if window == "gauss":  # :70-73
        b = m / pi
        return np.exp(-((pi * n / Nt) ** 2) * b)
    if window == "spline":  # :98-100
        return np.sinc(n / Nt) ** (2 * m)
    if window == "kaiser_bessel_rev":  # :51-57, real(sinc(arg/pi)) with arg = sqrt(complex(.))
        b = pi * (2 - 1 / sigma)
        a2 = (2 * pi * m * n / Nt) ** 2 - (m * b) ** 2
        arg = np.sqrt(a2.astype(np.complex128))
        return np.real(np.sinc(arg / pi))
    if window == "cosh_type":  # :118-134
        beta = pi * m * (2 - 1 / sigma)
        gamma = beta / (2 * pi)
        zeta = pi / (np.cosh(beta) - 1) * m
        arg = m * n / Nt
        out = np.empty_like(arg)
        lo = np.abs(arg) < gamma
        hi = np.abs(arg) > gamma
        eq = ~(lo | hi)
        out[lo] = zeta * (scipy.special.i0(np.sqrt(beta ** 2 - (2 * pi * arg[lo]) ** 2)) - scipy.special.j0(2 * pi * arg[lo]))
        out[hi] = zeta * (scipy.special.j0(np.sqrt((2 * pi * arg[hi]) ** 2 - beta ** 2)) - scipy.special.j0(2 * pi * arg[hi]))
        out[eq] = zeta * (1 - scipy.special.j0(beta))
        return out
    raise ValueError(f"Window {window} not yet implemented!")


def poly_coefficients(window, m, sigma):
    """precomputePolyInterp, src/precomputation.jl:302-320: for each of the 2m
    tap columns a least-squares fit (V' \\ samples) of a degree-2m polynomial to
    phi(m - (l - 0.5) + t), t on 2(2m+1) equispaced points in [-0.5, 0.5].
    Returns an FP64 array of shape (2m+1, 2m)."""
    deg = 2 * m + 1
    K = 2 * m
    ns = 2 * deg
    kk = np.linspace(-0.5, 0.5, ns)
    V = np.ones((deg, ns))
    for r in range(1, deg):
        V[r] = V[r - 1] * kk
    out = np.empty((deg, K))
    for l in range(1, K + 1):
        y = (m - (l - 0.5)) + kk
        samples = np.array([window_phi(window, yy, 1, m, sigma) for yy in y])
        out[:, l - 1] = np.linalg.lstsq(V.T, samples, rcond=None)[0]
    return out


def linear_lut(window, m, sigma, K):
    """precomputeLinInterp, src/precomputation.jl:291-300: phi((l-1)*m/K), l=1..K+2."""
    step = m / K
    return np.array([window_phi(window, l * step, 1, m, sigma) for l in range(K + 2)])


def chebyshev_interp(fun, a, b, n, x):
    """Degree n-1 interpolant of ``fun`` through n first-kind Chebyshev points on
    [a, b], evaluated at ``x`` (Clenshaw).  Restates the ChebyshevInterpolator of
    BasicInterpolators.jl (an unvendored dependency, compat 0.6.5/0.7) used at
    src/precomputation.jl:351; its exact node kind is not pinned by any test."""
    i = np.arange(1, n + 1)
    theta = np.pi * (2 * i - 1) / (2 * n)
    xi = np.cos(theta)
    y = fun(0.5 * (b - a) * (xi + 1) + a)
    kk = np.arange(n)
    c = (2.0 / n) * (np.cos(np.outer(kk, theta)) @ y)
    c[0] *= 0.5
    t = (2.0 * np.asarray(x, dtype=np.float64) - (a + b)) / (b - a)
    b1 = np.zeros_like(t)
    b2 = np.zeros_like(t)
    for ck in c[:0:-1]:
        b1, b2 = 2 * t * b1 - b2 + ck, b1
    return t * b1 - b2 + c[0]


def sort_nodes_lex(k):
    """k .= sortslices(k, dims=2) (src/precomputation.jl:52-54,
    src/implementation.jl:112-114): the columns of the D x M node array sorted
    in place in lexicographic order, dimension 1 first, each coordinate by
    Julia's isless (-0.0 before 0.0; nodes are checked before, so no NaN).
    Returns the permutation (new column i = old column perm[i])."""
    keys = []
    for d in reversed(range(k.shape[0])):
        keys.append(~np.signbit(k[d]))  # ties of equal values: -0.0 first
        keys.append(k[d])
    perm = np.lexsort(keys)
    k[...] = k[:, perm]
    return perm


def index_offset(n):
    """indexOffset, src/precomputation.jl:345."""
    return (-1 - n // 2) if n % 2 == 0 else (-1 - (n - 1) // 2)


def deconv_factors(window, N, Nt, m, sigma, exact=False):
    """precomputeWindowHatInvLUT, src/precomputation.jl:347-358: per dimension,
    1 / cheb(j), j = 1..N_d, cheb a 30-point Chebyshev interpolant of
    phi-hat(j + indexOffset(N_d)) on [1, N_d].  FP64."""
    out = []
    for d in range(len(N)):
        kap = lambda x, d=d: window_hat(window, x + index_offset(N[d]), Nt[d], m, sigma)
        j = np.arange(1, N[d] + 1, dtype=np.float64)
        if exact or N[d] == 1:
            out.append(1.0 / kap(j))
        else:
            out.append(1.0 / chebyshev_interp(kap, 1.0, float(N[d]), 30, j))
    return out


# --------------------------------------------------------------------- plan

class OraclePlan:
    """FP32/FP64 restatement of NFFTPlan with blocking (src/implementation.jl:73-106,
    155-193)."""

    def __init__(self, k, N, *, m=None, sigma=None, reltol=None, window="kaiser_bessel",
                 precompute=TENSOR, blockSize=None, dtype=np.float64, fft_workers=None, sortNodes=False):
        k = np.asarray(k)
        if k.ndim == 1:
            k = k.reshape(1, -1)
        self.D = k.shape[0]
        self.N = tuple(int(n) for n in N)
        if len(self.N) != self.D:
            raise ValueError(f"Nodes x have dimension {self.D} != {len(self.N)}")
        self.dtype = np.dtype(dtype)
        self.cdtype = np.complex64 if self.dtype == np.float32 else np.complex128
        pr = init_params(self.N, m, sigma, reltol, blockSize)
        self.m, self.sigma, self.Nt, self.block_size = pr["m"], pr["sigma"], pr["Nt"], pr["block_size"]
        self.LUTSize = pr["LUTSize"]
        self.window = window
        self.precompute = precompute
        self.M = k.shape[1]
        self.fft_workers = fft_workers if fft_workers is not None else (os.cpu_count() or 1)
        kk = np.ascontiguousarray(k.T.astype(self.dtype))  # column-major D x M
        if not np.all(np.abs(kk) <= 0.5):  # checkNodes, src/utils.jl:46-55
            raise ValueError("Nodes k need to be within the range [-1/2, 1/2)")
        if sortNodes:  # k .= sortslices(k, dims=2) on the caller's array, src/precomputation.jl:52-54
            kd = np.array(k, dtype=self.dtype)
            sort_nodes_lex(kd)
            if k.flags.writeable:
                k[...] = kd
            kk = np.ascontiguousarray(kd.T)
        self.k = kk
        self.coeffs = poly_coefficients(window, self.m, self.sigma)
        # polynomial coefficients are stored in T (Matrix{T}, :306)
        coeffs_t = self.coeffs.astype(self.dtype).astype(np.float64)
        coeffs_c = np.ascontiguousarray(coeffs_t.T)  # column l contiguous
        lut = np.zeros(1)
        if precompute == LINEAR:
            mode = _MODE_LINEAR
            lut = linear_lut(window, self.m, self.sigma, self.LUTSize).astype(self.dtype).astype(np.float64)
        elif precompute == FULL:
            mode = _MODE_EXACT
        else:
            mode = _MODE_POLY
        self._lut = lut
        self._coeffs_c = coeffs_c
        inv = deconv_factors(window, self.N, self.Nt, self.m, self.sigma)
        self.inv = [np.ascontiguousarray(v.astype(self.dtype)) for v in inv]
        L = lib()
        self._suf = "f32" if self.dtype == np.float32 else "f64"
        Nt_a, Nt_p = _i64(self.Nt)
        bs_a, bs_p = _i64(self.block_size)
        self._h = getattr(L, f"oracle_plan_new_{self._suf}")(
            self.D, Nt_p, self.m, bs_p, self.M, kk.ctypes.data, mode, coeffs_c.ctypes.data,
            lut.ctypes.data, self.LUTSize, WINDOWS[window], self.sigma)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            getattr(lib(), f"oracle_plan_free_{self._suf}")(h)
            self._h = None

    # --- integer outputs of the blocking (src/precomputation.jl:487-520)
    def blocks(self):
        L = lib()
        nb = getattr(L, f"oracle_plan_nblocks_{self._suf}")(self._h)
        bstart = np.zeros(nb + 1, np.int64)
        nodes = np.zeros(self.M, np.int64)
        bins = np.zeros(self.M, np.int64)
        trunc = np.zeros(self.D * self.M, np.int64)
        getattr(L, f"oracle_plan_blocks_{self._suf}")(
            self._h, *(a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)) for a in (bstart, nodes, bins, trunc)))
        return dict(block_start=bstart, nodes=nodes, bins=bins, trunc=trunc.reshape(self.M, self.D).T.copy())

    # --- the four stages (AbstractNFFTs optional interface)
    def convolve(self, g):
        g = np.ascontiguousarray(np.asarray(g).ravel(order="F").astype(self.cdtype))
        out = np.zeros(self.M, self.cdtype)
        getattr(lib(), f"oracle_convolve_{self._suf}")(self._h, g.ctypes.data, out.ctypes.data)
        return out

    def convolve_transpose(self, fhat):
        fhat = np.ascontiguousarray(np.asarray(fhat).astype(self.cdtype))
        g = np.zeros(int(np.prod(self.Nt)), self.cdtype)
        getattr(lib(), f"oracle_convolve_transpose_{self._suf}")(self._h, fhat.ctypes.data, g.ctypes.data)
        return g.reshape(self.Nt, order="F")

    def _inv_ptrs(self):
        ptrs = [v.ctypes.data for v in self.inv] + [self.inv[0].ctypes.data] * (3 - self.D)
        return ptrs

    def deconvolve(self, f):
        f = np.ascontiguousarray(np.asarray(f).ravel(order="F").astype(self.cdtype))
        g = np.empty(int(np.prod(self.Nt)), self.cdtype)
        N_a, N_p = _i64(self.N)
        T_a, T_p = _i64(self.Nt)
        getattr(lib(), f"oracle_deconvolve_{self._suf}")(self.D, N_p, T_p, *self._inv_ptrs(), f.ctypes.data, g.ctypes.data)
        return g.reshape(self.Nt, order="F")

    def deconvolve_transpose(self, g):
        g = np.ascontiguousarray(np.asarray(g).ravel(order="F").astype(self.cdtype))
        f = np.empty(int(np.prod(self.N)), self.cdtype)
        N_a, N_p = _i64(self.N)
        T_a, T_p = _i64(self.Nt)
        getattr(lib(), f"oracle_deconvolve_transpose_{self._suf}")(self.D, N_p, T_p, *self._inv_ptrs(), g.ctypes.data, f.ctypes.data)
        return f.reshape(self.N, order="F")

    def _fft(self, g, sign):
        # FFTW plan_fft! (sign -1) / plan_bfft! (sign +1), both unnormalised,
        # src/implementation.jl:87-88; here pocketfft through scipy.fft.
        flat = np.asarray(g).ravel(order="F")
        c = flat.reshape(self.Nt[::-1])  # same memory, C order
        if sign < 0:
            r = scipy.fft.fftn(c, workers=self.fft_workers, overwrite_x=True)
        else:
            r = scipy.fft.ifftn(c, norm="forward", workers=self.fft_workers, overwrite_x=True)
        return r.astype(self.cdtype, copy=False).ravel().reshape(self.Nt, order="F")

    def forward(self, f):
        """mul!(fHat, p, f), src/implementation.jl:155-172."""
        g = self.deconvolve(f)
        g = self._fft(g, -1)
        return self.convolve(g)

    def adjoint(self, fhat):
        """mul!(f, adjoint(p), fHat), src/implementation.jl:176-193."""
        g = self.convolve_transpose(fhat)
        g = self._fft(g, +1)
        return self.deconvolve_transpose(g)


# --------------------------------------------------------------------- NDFT

def ndft_forward(k, f, subset=None):
    """Direct NDFT, src/direct.jl:99-123, FP64; optionally only at node indices
    ``subset``.  k: (D, M), f: logical shape N."""
    k = np.asarray(k, dtype=np.float64)
    if k.ndim == 1:
        k = k.reshape(1, -1)
    D = k.shape[0]
    N = f.shape
    if subset is not None:
        k = k[:, np.asarray(subset)]
    kk = np.ascontiguousarray(k.T)
    fc = np.ascontiguousarray(np.asarray(f).ravel(order="F").astype(np.complex128))
    out = np.zeros(kk.shape[0], np.complex128)
    N_a, N_p = _i64(N)
    lib().oracle_ndft_forward(D, N_p, kk.shape[0], kk.ctypes.data, fc.ctypes.data, out.ctypes.data)
    return out


def ndft_adjoint(k, N, fhat, subset=None, method=None):
    """Direct adjoint NDFT, src/direct.jl:126-151, FP64; with ``subset`` (linear
    column-major indices) only those outputs are returned (flat).

    ``method``: "direct" evaluates cos/sin for every (node, output) pair (the
    default without a subset); "table" builds per-node phase tables of at most
    256 entries per (virtual) dimension and multiplies their entries (the
    default with a subset: ~20 flops per pair, used for the full-size NDFT
    subsets)."""
    k = np.asarray(k, dtype=np.float64)
    if k.ndim == 1:
        k = k.reshape(1, -1)
    D = k.shape[0]
    N = tuple(N)
    kk = np.ascontiguousarray(k.T)
    fh = np.ascontiguousarray(np.asarray(fhat).astype(np.complex128))
    sel = np.arange(int(np.prod(N)), dtype=np.int64) if subset is None else np.asarray(subset, np.int64)
    sel_a, sel_p = _i64(sel)
    out = np.zeros(sel.size, np.complex128)
    N_a, N_p = _i64(N)
    if method is None:
        method = "direct" if subset is None else "table"
    fn = lib().oracle_ndft_adjoint if method == "direct" else lib().oracle_ndft_adjoint_sel
    fn(D, N_p, kk.shape[0], kk.ctypes.data, fh.ctypes.data, sel.size, sel_p, out.ctypes.data)
    if subset is None:
        return out.reshape(N, order="F")
    return out


# The NFFT.jl TENSOR series of the paper's accuracy figure at D = 2, N = 512^2,
# J = |N|, sigma = 2 (benchmark/paper/img/accuracy_m_D2_.tex:40-43 forward,
# :87-90 adjoint): mean relative l2 error over the script's P = 10 runs.
PAPER_D2_TENSOR = {
    "forward": {3: 7.662783919423607e-6, 4: 5.747972034947691e-8, 5: 6.130420281952177e-10,
                6: 8.923266708493597e-12},
    "adjoint": {3: 6.932655431859695e-6, 4: 6.318935476675504e-8, 5: 7.001282121332577e-10,
                6: 7.660093463898552e-12},
}


def paper_d2_runs(nruns=10, seed=1):
    """The inputs of benchmark/paper/accuracyNew.jl:29-45 at D = 2 (N = 512^2,
    J = |N|, sigma = 2), run by run: nodes rand(2, J) - 1/2, fHat =
    randn(ComplexF64, J) (each part N(0, 1/2)), f = rand(ComplexF64, N) (each
    part U[0, 1)).  Each run yields (k, f, fhat, truth_forward, truth_adjoint),
    the ground truth from an FP64 FULL-precompute plan at m = 8: the script
    used NFFT3 at m = 12, and both sit at the ~2e-14 floor of the figure
    (accuracy_m_D2_.tex:45-47), far below the m <= 6 errors compared."""
    rng = np.random.default_rng(seed)
    N = (512, 512)
    J = N[0] * N[1]
    for _ in range(nruns):
        k = rng.random((2, J)) - 0.5
        fhat = (rng.standard_normal(J) + 1j * rng.standard_normal(J)) / math.sqrt(2)
        f = rng.random(N) + 1j * rng.random(N)
        g = OraclePlan(k, N, m=8, sigma=2.0, precompute=FULL)
        yield k, f, fhat, g.forward(f), g.adjoint(fhat)


def rel_l2(x, ref):
    """||x - ref|| / ||ref|| in FP64: raw window sums reach 1e21 in 3-D (the
    window is unnormalised), so FP32 squares would overflow."""
    x = np.asarray(x).ravel()
    ref = np.asarray(ref).ravel()
    up = np.complex128 if (np.iscomplexobj(x) or np.iscomplexobj(ref)) else np.float64
    x = x.astype(up)
    ref = ref.astype(up)
    return float(np.linalg.norm(x - ref) / np.linalg.norm(ref))


def sdc(plan, iters=20):
    """Sampling density compensation, restating NFFTTools sdc!
    (NFFTTools/src/samplingDensity.jl:93-155) on an OraclePlan with the real
    convolve / convolve_transpose of the optional interface."""
    rdt = plan.dtype
    weights = np.ones(plan.M, rdt)
    scaling = None
    for i in range(iters):
        workg = np.real(plan.convolve_transpose(weights.astype(plan.cdtype))).astype(rdt)
        if i == 0:
            scaling = workg.max()
        workg = workg / scaling
        wt = np.real(plan.convolve(workg.astype(plan.cdtype))).astype(rdt) / scaling
        if np.any(wt <= 0):
            raise ValueError("non-positive weights")
        weights = weights / wt
    u = np.ones(plan.N, plan.cdtype)
    workf = plan.forward(u) * weights
    workv = plan.adjoint(workf)
    c = np.real(workv.sum()) / np.sum(np.abs(workv) ** 2)
    return (weights * c).astype(rdt)


# ----------------------------------------------------------------- Toeplitz

def toeplitz_kernel(shape, tr, m=4, sigma=2.0, window="kaiser_bessel", dtype=np.float64, precompute=TENSOR):
    """calculateToeplitzKernel (NFFTTools/src/Toeplitz.jl:86-93): FFT of the
    fftshifted adjoint NFFT of ones on a plan of size 2 .* shape."""
    shape = tuple(int(n) for n in shape)
    p = OraclePlan(tr, tuple(2 * n for n in shape), m=m, sigma=sigma, window=window, dtype=dtype,
                   precompute=precompute)
    eig = p.adjoint(np.ones(p.M, p.cdtype))
    return np.fft.fftn(np.fft.fftshift(eig.astype(np.complex128)))


def toeplitz_kernel_explicit(shape, tr):
    """calculateToeplitzKernel_explicit (Toeplitz.jl:142-164): the exact sums
    getMatrixElement(idx) = sum_j exp(-2 pi i k_j . (shape_os/2 + 1 - idx))
    = the adjoint NDFT of ones on the 2 .* shape grid, fftshifted and
    transformed; FP64."""
    shape_os = tuple(2 * int(n) for n in shape)
    tr = np.asarray(tr, dtype=np.float64)
    if tr.ndim == 1:
        tr = tr.reshape(1, -1)
    eig = ndft_adjoint(tr, shape_os, np.ones(tr.shape[1], np.complex128))
    return np.fft.fftn(np.fft.fftshift(eig))


def convolve_toeplitz(y, lam, dtype=np.complex128, workers=1):
    """convolveToeplitzKernel! (Toeplitz.jl:230-244): the image in the corner
    of a zero grid of lam's size, FFT, product, normalised inverse FFT, crop;
    computed in ``dtype`` (FP64 by default), returns a new array."""
    y = np.asarray(y)
    lam = np.asarray(lam)
    xos = np.zeros(lam.shape, dtype)
    xos[tuple(slice(0, n) for n in y.shape)] = y
    xos = scipy.fft.fftn(xos, workers=workers, overwrite_x=True)
    xos *= lam
    xos = scipy.fft.ifftn(xos, workers=workers, overwrite_x=True)
    return xos[tuple(slice(0, n) for n in y.shape)]


# ------------------------------------------------- NDCT / NDST / NNDFT

def _trig_factors(k, N, fun, shift):
    """Per-dimension factor matrices fun(2 pi k_dj (n + shift)), n = 0..N_d-1."""
    k = np.asarray(k, dtype=np.float64)
    if k.ndim == 1:
        k = k.reshape(1, -1)
    return [fun(2.0 * np.pi * np.outer(k[d], np.arange(N[d], dtype=np.float64) + shift)) for d in range(len(N))]


def _contract(mats, f):
    """g_j = sum_n f[n] prod_d mats[d][j, n_d] for f of logical shape N."""
    D = len(mats)
    letters = "abcd"[:D]
    expr = ",".join(f"j{c}" for c in letters) + "," + letters + "->j"
    return np.einsum(expr, *mats, f, optimize=True)


def _contract_t(mats, v):
    """f[n] = sum_j v_j prod_d mats[d][j, n_d]."""
    D = len(mats)
    letters = "abcd"[:D]
    expr = ",".join(f"j{c}" for c in letters) + ",j->" + letters
    return np.einsum(expr, *mats, v, optimize=True)


def ndct_forward(k, f):
    """NDCTPlan * f (src/direct.jl:153-174): fHat_j = sum_n f_n prod_d
    cos(2 pi k_dj n_d), n_d = 0..N_d-1; FP64."""
    f = np.asarray(f)
    return _contract(_trig_factors(k, f.shape, np.cos, 0.0), f.astype(np.result_type(f, np.float64)))


def ndct_transpose(k, N, fhat):
    """transpose(NDCTPlan) * fHat (src/direct.jl:177-199)."""
    fhat = np.asarray(fhat)
    return _contract_t(_trig_factors(k, tuple(N), np.cos, 0.0), fhat.astype(np.result_type(fhat, np.float64)))


def ndst_forward(k, f):
    """NDSTPlan * f (src/direct.jl:202-224): the input has N - 1 points per
    dimension, n_d = 1..N_d-1, factors sin(2 pi k_dj n_d); FP64."""
    f = np.asarray(f)
    return _contract(_trig_factors(k, f.shape, np.sin, 1.0), f.astype(np.result_type(f, np.float64)))


def ndst_transpose(k, N, fhat):
    """transpose(NDSTPlan) * fHat (src/direct.jl:227-249); N is the plan
    size, the output has N - 1 points per dimension."""
    fhat = np.asarray(fhat)
    Nm = tuple(int(n) - 1 for n in N)
    return _contract_t(_trig_factors(k, Nm, np.sin, 1.0), fhat.astype(np.result_type(fhat, np.float64)))


def nndft_forward(k, y, f):
    """NNDFTPlan * f (src/direct.jl:252-268): fHat_j = sum_l f_l
    exp(-2 pi i k_j . y_l); FP64."""
    k = np.atleast_2d(np.asarray(k, dtype=np.float64))
    y = np.atleast_2d(np.asarray(y, dtype=np.float64))
    return np.exp(-2j * np.pi * (k.T @ y)) @ np.asarray(f, dtype=np.complex128)


def nndft_adjoint(k, y, fhat):
    """adjoint(NNDFTPlan) * fHat (src/direct.jl:270-287)."""
    k = np.atleast_2d(np.asarray(k, dtype=np.float64))
    y = np.atleast_2d(np.asarray(y, dtype=np.float64))
    return np.exp(2j * np.pi * (y.T @ k)) @ np.asarray(fhat, dtype=np.complex128)


def ndft_forward_sep(k, f):
    """The NDFT of ndft_forward by per-dimension phase matrices (any D <= 4):
    exp(-2 pi i k_dj (n_d - N_d div 2)); FP64."""
    f = np.asarray(f)
    N = f.shape
    k = np.atleast_2d(np.asarray(k, dtype=np.float64))
    mats = [np.exp(-2j * np.pi * np.outer(k[d], np.arange(N[d]) - N[d] // 2)) for d in range(len(N))]
    return _contract(mats, f.astype(np.complex128))


def ndft_adjoint_sep(k, N, fhat):
    """The adjoint NDFT of ndft_adjoint by per-dimension phase matrices."""
    N = tuple(int(n) for n in N)
    k = np.atleast_2d(np.asarray(k, dtype=np.float64))
    mats = [np.exp(2j * np.pi * np.outer(k[d], np.arange(N[d]) - N[d] // 2)) for d in range(len(N))]
    return _contract_t(mats, np.asarray(fhat, dtype=np.complex128))
