"""NFFTTools clients on the GPU plan.

``sdc`` restates NFFTTools' sampling density compensation
(NFFTTools/src/samplingDensity.jl:59-155) on top of the plan's real-valued
``convolve!`` / ``convolve_transpose!`` and ``mul!``, the way NFFTTools uses the
reference's GPU plan (test/gpu.jl:52-65).

The Toeplitz tools (NFFTTools/src/Toeplitz.jl) mirror
``calculateToeplitzKernel``, ``calculateToeplitzKernel!``,
``calculateToeplitzKernel_explicit`` and ``convolveToeplitzKernel!`` on the
library's ``nfft_toeplitz_*`` entry points: the kernel lambda of the Gram
operator A^H A on the 2N grid, and its application to an image.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib as L
from . import plan as P


def sdc(p, iters=20, weights=None, weights_tmp=None, workg=None, workf=None, workv=None):
    """Density compensation weights (real, length J) with the final scaling
    c = real(sum(v)) / ||v||^2 of sdc! (:138-155).  The work buffers may be
    passed in to avoid allocation, as in the reference."""
    T = p.dtype
    dev = p.device
    if weights is None:
        weights = torch.ones(p.J, dtype=T, device=dev)
    if weights_tmp is None:
        weights_tmp = torch.empty_like(weights)
    if workg is None:
        workg = P.empty_image(p.Ñ, T, dev)
    if workf is None:
        workf = torch.empty(p.J, dtype=p.cdtype, device=dev)
    if workv is None:
        workv = P.empty_image(p.N, p.cdtype, dev)
    scaling = None
    for i in range(iters):
        p.convolve_transpose_(weights, workg)
        if i == 0:
            scaling = workg.max()
        workg.div_(scaling)
        p.convolve_(workg, weights_tmp)
        weights_tmp.div_(scaling)
        if bool((weights_tmp <= 0).any()):
            raise ValueError("non-positive weights")
        weights.div_(weights_tmp)
    u = workv
    u.fill_(1)
    p.forward_(workf, u)
    workf.mul_(weights)
    p.adjoint_(workv, workf)
    c = workv.sum().real / (workv.abs() ** 2).sum()
    weights.mul_(c)
    return weights


# ---------------------------------------------------------------- Toeplitz
class Toeplitz:
    """Workspace of the Toeplitz tools for one image size ``shape`` and
    precision: the 2N grid and transforms that ``convolveToeplitzKernel!``
    takes as ``fftplan, ifftplan, xOS1, xOS2`` (Toeplitz.jl:230-244) and
    ``calculateToeplitzKernel!`` as ``fftplan``.  ``fft="cufft"`` forces the
    cuFFT sequence; ``"auto"`` fuses the pruned transforms and the kernel
    product where the 2N sizes allow."""

    def __init__(self, shape, dtype=torch.complex64, device="cuda", fft="auto"):
        if isinstance(shape, int):
            shape = (shape,)
        self.shape = tuple(int(n) for n in shape)
        self.shape_os = tuple(2 * n for n in self.shape)
        if dtype in (torch.float32, np.float32, torch.complex64, np.complex64):
            self.cdtype, self.dtype, self.precision = torch.complex64, torch.float32, 32
        elif dtype in (torch.float64, np.float64, torch.complex128, np.complex128):
            self.cdtype, self.dtype, self.precision = torch.complex128, torch.float64, 64
        else:
            raise P.ArgumentError(f"unsupported element type {dtype}")
        if fft not in ("auto", "cufft"):
            raise P.ArgumentError("fft must be 'auto' or 'cufft'")
        dev = torch.device(device)
        if dev.type == "cuda" and dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        lib = L.load()
        D = len(self.shape)
        Narr = (ctypes.c_int64 * 3)(*(list(self.shape) + [1] * (3 - D)))
        h = ctypes.c_void_p()
        self._handle = None
        with torch.cuda.device(dev):
            stream = torch.cuda.current_stream(dev).cuda_stream
            P._check(lib.nfft_toeplitz_create(ctypes.byref(h), self.precision, D, Narr,
                                              0 if fft == "auto" else 1, ctypes.c_void_p(stream)))
        self._handle = h
        self._stream = stream

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                L.load().nfft_toeplitz_destroy(h)
            except Exception:
                pass
            self._handle = None

    @property
    def fused(self):
        """Whether ``convolve_`` runs the fused pruned-FFT path."""
        v = ctypes.c_int()
        P._check(L.load().nfft_toeplitz_is_fused(self._handle, ctypes.byref(v)))
        return bool(v.value)

    def _sync_stream(self):
        s = torch.cuda.current_stream(self.device).cuda_stream
        if s != self._stream:
            P._check(L.load().nfft_toeplitz_set_stream(self._handle, ctypes.c_void_p(s)))
            self._stream = s

    def _grid(self, x, shape, what):
        if not isinstance(x, torch.Tensor) or tuple(x.shape) != shape:
            raise P.DimensionMismatch(f"{what} must have size {shape}")
        if x.dtype != self.cdtype or x.device != self.device or not P._is_colmajor(x):
            raise P.ArgumentError(f"{what} must be a column-major {self.cdtype} tensor on {self.device}")
        return x

    def empty_kernel(self):
        return P.empty_image(self.shape_os, self.cdtype, self.device)

    def kernel_(self, lam, p):
        """lambda <- FFT(fftshift(adjoint(p) * ones(J))) for a plan ``p`` of
        size 2N with nodes (calculateToeplitzKernel!, Toeplitz.jl:129-135)."""
        lam = self._grid(lam, self.shape_os, "kernel")
        if tuple(p.N) != self.shape_os:
            raise P.DimensionMismatch(f"the plan's size {p.N} must be twice the image size {self.shape}")
        p._sync_stream()
        self._sync_stream()
        P._check(L.load().nfft_toeplitz_kernel(self._handle, p._handle, P._ptr(lam)))
        return lam

    def kernel_explicit_(self, lam, tr):
        """lambda from the exact sums (calculateToeplitzKernel_explicit,
        Toeplitz.jl:142-164), accumulated in FP64."""
        lam = self._grid(lam, self.shape_os, "kernel")
        kk = P.GB300NFFTPlan._nodes_array(tr)
        if kk.shape[0] != len(self.shape):
            raise P.ArgumentError(f"Nodes x have dimension {kk.shape[0]} != {len(self.shape)}")
        if isinstance(kk, torch.Tensor):
            kt = kk.to(device=self.device, dtype=self.dtype).t().contiguous()
        else:
            kt = torch.from_numpy(np.ascontiguousarray(kk.T)).to(device=self.device, dtype=self.dtype)
        self._sync_stream()
        P._check(L.load().nfft_toeplitz_kernel_explicit(self._handle, P._ptr(kt), int(kk.shape[1]), 1,
                                                         P._ptr(lam)))
        return lam

    def convolve_(self, y, lam):
        """y <- crop(IFFT(lambda . FFT(pad(y)))) in place
        (convolveToeplitzKernel!, Toeplitz.jl:230-244)."""
        lam = self._grid(lam, self.shape_os, "kernel")
        if not isinstance(y, torch.Tensor) or tuple(y.shape) != self.shape:
            raise P.DimensionMismatch(f"image must have size {self.shape}")
        self._sync_stream()
        if y.dtype == self.cdtype and y.device == self.device and P._is_colmajor(y):
            P._check(L.load().nfft_toeplitz_apply(self._handle, P._ptr(lam), P._ptr(y)))
            return y
        t = P.as_colmajor(y, self.shape, self.cdtype, self.device)
        if t.data_ptr() == y.data_ptr():
            t = t.clone()
        P._check(L.load().nfft_toeplitz_apply(self._handle, P._ptr(lam), P._ptr(t)))
        y.copy_(t)
        return y


def _toeplitz_for(shape, cdtype, device, toeplitz):
    if toeplitz is not None:
        if toeplitz.shape != tuple(shape) or toeplitz.cdtype != cdtype:
            raise P.DimensionMismatch("Toeplitz workspace of another size or precision")
        return toeplitz
    return Toeplitz(shape, cdtype, device)


def calculate_toeplitz_kernel(shape, tr, m=4, sigma=2.0, window="kaiser_bessel", toeplitz=None, device="cuda",
                              **kwargs):
    """calculateToeplitzKernel(shape, tr; m, σ, window) (Toeplitz.jl:86-93):
    the kernel (size 2 .* shape, complex of tr's type) of A^H A for the nodes
    ``tr`` (D x J).  ``kwargs`` go to the plan of size 2 .* shape."""
    if isinstance(shape, int):
        shape = (shape,)
    shape = tuple(int(n) for n in shape)
    p = P.plan_nfft(tr, tuple(2 * n for n in shape), m=m, sigma=sigma, window=window, device=device, **kwargs)
    tz = _toeplitz_for(shape, p.cdtype, p.device, toeplitz)
    lam = tz.empty_kernel()
    return tz.kernel_(lam, p)


def calculate_toeplitz_kernel_(lam, p, tr, toeplitz=None):
    """calculateToeplitzKernel!(f, p, tr, fftplan) (Toeplitz.jl:129-135):
    nodes!(p, tr), then the kernel into ``lam`` (size p.N = 2 .* shape)."""
    P.nodes_(p, tr)
    shape = tuple(n // 2 for n in p.N)
    tz = _toeplitz_for(shape, p.cdtype, p.device, toeplitz)
    return tz.kernel_(lam, p)


def calculate_toeplitz_kernel_explicit(shape, tr, toeplitz=None, device="cuda"):
    """calculateToeplitzKernel_explicit(shape, tr) (Toeplitz.jl:142-164)."""
    if isinstance(shape, int):
        shape = (shape,)
    shape = tuple(int(n) for n in shape)
    kk = P.GB300NFFTPlan._nodes_array(tr)
    single = kk.dtype in (np.float32, torch.float32)
    tz = _toeplitz_for(shape, torch.complex64 if single else torch.complex128, device, toeplitz)
    lam = tz.empty_kernel()
    return tz.kernel_explicit_(lam, kk)


def convolve_toeplitz_kernel_(y, lam, toeplitz=None):
    """convolveToeplitzKernel!(y, λ[, fftplan, ifftplan, xOS1, xOS2])
    (Toeplitz.jl:230-244): y <- A^H A y through the kernel, in place.  Pass
    a :class:`Toeplitz` as ``toeplitz`` to reuse its workspace (the
    reference's pre-allocated plans and buffers)."""
    if not isinstance(lam, torch.Tensor):
        raise P.ArgumentError("the kernel must be a device tensor")
    shape = tuple(n // 2 for n in lam.shape)
    tz = _toeplitz_for(shape, lam.dtype, lam.device, toeplitz)
    return tz.convolve_(y, lam)
