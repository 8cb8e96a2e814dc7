"""Python mirror of the AbstractNFFTs plan interface over the GB300 C ABI.

Names, argument meanings and errors follow the reference:

=============================  ==================================================
this module                    reference
=============================  ==================================================
``plan_nfft(k, N, **kw)``      ``plan_nfft(CuArray, k, N; kw...)``
                               (ext/NFFTGPUArraysExt/implementation.jl:21-59)
``mul_(fHat, p, f)``           ``mul!(fHat, p, f)`` (src/implementation.jl:155)
``mul_(f, adjoint(p), fHat)``  ``mul!(f, adjoint(p), fHat)`` (:176)
``p * f``, ``adjoint(p) * y``  ``*`` (AbstractNFFTs/src/derived.jl:174-208)
``nodes_(p, k)``               ``nodes!(p, k)`` (src/implementation.jl:108-141)
``convolve_`` etc.             optional interface (AbstractNFFTs/src/interface.jl:215-243)
``nfft``, ``nfft_adjoint``     AbstractNFFTs/src/derived.jl:134-166
``DimensionMismatch``,         Julia's exception types of the same names
``ArgumentError``
=============================  ==================================================

Arrays follow Julia's layout.  ``k`` has logical shape (D, M).  Images have
logical shape ``N`` and must be column-major (dimension 1 fastest), e.g. from
:func:`empty_image`; node vectors have shape (M,).  Device arrays are torch
CUDA tensors (the CuArray analogue); complex values are complex64 for Float32
plans and complex128 for Float64 plans.
"""
from __future__ import annotations

import ctypes
import enum
import math
import weakref
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib as L


class DimensionMismatch(ValueError):
    """Julia's DimensionMismatch (src/utils.jl:98-105)."""


class ArgumentError(ValueError):
    """Julia's ArgumentError (src/utils.jl:46-55, src/convolution.jl:47-53)."""


class NFFTError(RuntimeError):
    """A failure reported by the CUDA library (allocation, CUDA, cuFFT)."""


class PrecomputeFlags(enum.IntEnum):
    """AbstractNFFTs/src/misc.jl:13-19."""
    FULL = 1
    TENSOR = 2
    LINEAR = 3
    POLYNOMIAL = 4


FULL, TENSOR, LINEAR, POLYNOMIAL = (PrecomputeFlags.FULL, PrecomputeFlags.TENSOR, PrecomputeFlags.LINEAR,
                                    PrecomputeFlags.POLYNOMIAL)

WINDOWS = {"kaiser_bessel": 0, "gauss": 1, "spline": 2, "kaiser_bessel_rev": 3, "cosh_type": 4}


class TimingStats:
    """AbstractNFFTs/src/misc.jl:22-42 (device seconds) of the plan's latest
    calls.  The plan records CUDA events around its stages; the fields are
    read from those events when accessed, so timed calls stay asynchronous
    (reading a field waits for the calls recorded so far)."""

    FIELDS = ("pre", "conv", "fft", "deconv", "conv_adjoint", "fft_adjoint", "deconv_adjoint")

    def __init__(self, pre=0.0, conv=0.0, fft=0.0, deconv=0.0, conv_adjoint=0.0, fft_adjoint=0.0,
                 deconv_adjoint=0.0):
        self._vals = [float(pre), float(conv), float(fft), float(deconv), float(conv_adjoint), float(fft_adjoint),
                      float(deconv_adjoint)]
        self._source = None  # weak method of the plan returning the 7 values

    def _refresh(self):
        src = self._source() if self._source is not None else None
        if src is not None:
            vals = src()
            if vals is not None:
                self._vals = [float(v) for v in vals]

    def __repr__(self):
        return "TimingStats(" + ", ".join(f"{n}={getattr(self, n):.6g}" for n in self.FIELDS) + ")"


def _timing_field(i):
    def get(self):
        self._refresh()
        return self._vals[i]

    def put(self, v):
        self._vals[i] = float(v)

    return property(get, put)


for _i, _n in enumerate(TimingStats.FIELDS):
    setattr(TimingStats, _n, _timing_field(_i))


def reltol_to_params(reltol):
    """AbstractNFFTs/src/misc.jl:44-48."""
    w = math.ceil(math.log10(1.0 / reltol)) + 1
    return w // 2, 2.0


def params_to_reltol(m, sigma):
    """AbstractNFFTs/src/misc.jl:50-53."""
    return 10.0 ** (-(2 * m - 1))


def accuracy_params(m=None, sigma=None, reltol=None):
    """accuracyParams, AbstractNFFTs/src/misc.jl:66-81: reltol wins; m and
    sigma are honoured only together; the default is reltol = 1e-9."""
    if reltol is not None:
        m_, s_ = reltol_to_params(reltol)
        return m_, s_, reltol
    if m is not None and sigma is not None:
        return int(m), float(sigma), params_to_reltol(m, sigma)
    reltol = 1e-9
    m_, s_ = reltol_to_params(reltol)
    return m_, s_, reltol


@dataclass
class NFFTParams:
    """NFFTParams (src/implementation.jl:3-14) as the GPU plan uses them."""
    m: int = 4
    sigma: float = 2.0
    reltol: float = 1e-7
    window: str = "kaiser_bessel"
    LUTSize: int = 0
    precompute: PrecomputeFlags = PrecomputeFlags.POLYNOMIAL
    sortNodes: bool = False
    storeDeconvolutionIdx: bool = False
    blocking: bool = True
    blockSize: tuple = field(default_factory=tuple)
    compensated: bool = False


def _check(rc):
    if rc == L.NFFT_OK:
        return
    lib = L.load()
    msg = (lib.nfft_last_error() or b"").decode(errors="replace")
    if rc in (L.NFFT_ERR_INVALID_ARG, L.NFFT_ERR_NODE_OUT_OF_RANGE):
        raise ArgumentError(msg)
    if rc == L.NFFT_ERR_DIM_MISMATCH:
        raise DimensionMismatch(msg)
    if rc == L.NFFT_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise NFFTError(f"{lib.nfft_status_string(rc).decode()}: {msg}")


def empty_image(N, dtype=torch.complex64, device="cuda"):
    """A column-major tensor of logical shape N (Julia layout)."""
    N = tuple(int(n) for n in N)
    return torch.empty(N[::-1], dtype=dtype, device=device).permute(*reversed(range(len(N))))


def as_colmajor(x, N, dtype, device="cuda"):
    """Move ``x`` (numpy or torch, logical shape N) to a column-major device
    tensor of ``dtype``; copies only when needed."""
    N = tuple(int(n) for n in N)
    if tuple(x.shape) != N:
        raise DimensionMismatch("Data is not consistent with NFFTPlan")
    if isinstance(x, np.ndarray):
        x = torch.from_numpy(np.ascontiguousarray(np.asarray(x).ravel(order="F")).reshape(N[::-1]))
        x = x.permute(*reversed(range(len(N))))
    if tuple(x.shape) != N:
        raise DimensionMismatch("Data is not consistent with NFFTPlan")
    x = x.to(device=device, dtype=dtype)
    if not _is_colmajor(x):
        y = empty_image(N, dtype, device)
        y.copy_(x)
        x = y
    return x


def _is_colmajor(x):
    s = 1
    for n, st in zip(x.shape, x.stride()):
        if n > 1 and st != s:
            return False
        s *= n
    return True


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class _GridView:
    """__cuda_array_interface__ over the plan's oversampled grid."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (ptr, False),
                                         "version": 3, "strides": None}


class GB300NFFTPlan:
    """The GPU NFFT plan (mirror of NFFTPlan / GPU_NFFTPlan).

    Fields mirror the reference: ``N``, ``NOut``, ``J``, ``k``, ``Ñ`` (also
    ``Ntilde``), ``dims``, ``params``, ``tmpVec``.  One plan is not safe for
    concurrent calls (it owns ``tmpVec``); use :meth:`copy`.
    """

    def __init__(self, k, N, *, m=None, sigma=None, reltol=None, window="kaiser_bessel",
                 precompute=PrecomputeFlags.POLYNOMIAL, blocking=True, sortNodes=False,
                 storeDeconvolutionIdx=False, blockSize=None, compensated=False, timing=None,
                 fftflags=None, dims=None, device="cuda"):
        kk = self._nodes_array(k)
        D = kk.shape[0]
        if isinstance(N, int):
            N = (N,)
        N = tuple(int(n) for n in N)
        if dims is not None and tuple(range(len(N))) != tuple(np.atleast_1d(dims)) and \
                tuple(range(1, len(N) + 1)) != tuple(np.atleast_1d(dims)):
            raise NotImplementedError("GPU NFFT does not work along directions right now!")
        if len(N) != D:
            raise ArgumentError(f"Nodes x have dimension {D} != {len(N)}")
        if window not in WINDOWS:
            raise NotImplementedError(f"Window {window} not yet implemented!")
        m_, s_, r_ = accuracy_params(m, sigma, reltol)
        self.dtype = torch.float32 if kk.dtype in (np.float32, torch.float32) else torch.float64
        self.cdtype = torch.complex64 if self.dtype == torch.float32 else torch.complex128
        self.precision = 32 if self.dtype == torch.float32 else 64
        dev = torch.device(device)
        if dev.type == "cuda" and dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        self.N = N
        self.dims = tuple(range(1, D + 1))
        self.params = NFFTParams(m=m_, sigma=s_, reltol=r_, window=window, precompute=PrecomputeFlags(precompute),
                                 sortNodes=bool(sortNodes), storeDeconvolutionIdx=bool(storeDeconvolutionIdx),
                                 blocking=bool(blocking), blockSize=tuple(blockSize or ()),
                                 compensated=bool(compensated))
        self._timing = timing
        self._handle = None
        self._stream = None
        self._create(kk.shape[1])
        self.nodes_(kk)

    # ------------------------------------------------------------------ setup
    @staticmethod
    def _nodes_array(k):
        if isinstance(k, torch.Tensor):
            kk = k.detach()
            if kk.dim() == 1:
                kk = kk.reshape(1, -1)
            return kk
        kk = np.asarray(k)
        if kk.ndim == 1:
            kk = kk.reshape(1, -1)
        if kk.dtype not in (np.float32, np.float64):
            kk = kk.astype(np.float64)
        return kk

    def _create(self, M):
        lib = L.load()
        prm = L.nfft_params()
        lib.nfft_params_default(ctypes.byref(prm))
        p = self.params
        prm.m = p.m
        prm.sigma = p.sigma
        prm.window = WINDOWS[p.window]
        prm.precompute = int(p.precompute)
        prm.blocking = int(p.blocking)
        prm.sort_nodes = int(p.sortNodes)
        prm.store_deconv_idx = int(p.storeDeconvolutionIdx)
        for d, b in enumerate(p.blockSize[:3]):
            prm.block_size[d] = int(b)
        prm.compensated = int(p.compensated)
        prm.timing = 1 if self._timing is not None else 0
        Narr = (ctypes.c_int64 * 3)(*(list(self.N) + [1] * (3 - len(self.N))))
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            stream = torch.cuda.current_stream(self.device)
            _check(lib.nfft_plan_create(ctypes.byref(h), self.precision, len(self.N), Narr, int(M),
                                        ctypes.byref(prm), ctypes.c_void_p(stream.cuda_stream)))
        self._handle = h
        self._stream = stream.cuda_stream
        info = L.nfft_info()
        _check(lib.nfft_get_info(h, ctypes.byref(info)))
        self._info = info
        D = len(self.N)
        self.Ñ = tuple(int(info.Ntilde[d]) for d in range(D))
        self.Ntilde = self.Ñ
        self.params.sigma = float(info.sigma)
        self.params.LUTSize = int(info.lut_size)
        self.params.blockSize = tuple(int(info.block_size[d]) for d in range(D))
        self.J = int(M)
        self.NOut = (int(M),)
        ng = int(np.prod(self.Ñ))
        gp = lib.nfft_grid(h)
        view = _GridView(gp, (ng,), "<c8" if self.precision == 32 else "<c16")
        flat = torch.as_tensor(view, device=self.device)
        self.tmpVec = flat.reshape(self.Ñ[::-1]).permute(*reversed(range(D)))

    def _sync_stream(self):
        s = torch.cuda.current_stream(self.device).cuda_stream
        if s != self._stream:
            _check(L.load().nfft_set_stream(self._handle, ctypes.c_void_p(s)))
            self._stream = s

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                L.load().nfft_plan_destroy(h)
            except Exception:
                pass
            self._handle = None

    # -------------------------------------------------------------- interface
    def size_in(self):
        return self.N

    def size_out(self):
        return self.NOut

    def nodes_(self, k):
        """nodes!(p, k): replace the nodes (src/implementation.jl:108-141)."""
        kk = self._nodes_array(k)
        if kk.shape[0] != len(self.N):
            raise ArgumentError(f"Nodes x have dimension {kk.shape[0]} != {len(self.N)}")
        if kk.shape[1] != self.J:
            self._destroy_handle()
            self._create(kk.shape[1])
        lib = L.load()
        self._sync_stream()
        D, M = kk.shape
        if isinstance(kk, torch.Tensor):
            kt = kk.to(device=self.device, dtype=self.dtype).t().contiguous()  # column-major D x M
            if self.params.sortNodes:
                # k .= sortslices(k, dims=2): the caller's tensor is sorted in place
                _check(lib.nfft_sort_nodes(self.precision, D, M, _ptr(kt), 1, ctypes.c_void_p(self._stream)))
                kk.copy_(kt.t())
            rc = lib.nfft_set_nodes(self._handle, _ptr(kt), 1)
            self.k = kk
        else:
            kc = np.ascontiguousarray(kk.T.astype(np.float32 if self.precision == 32 else np.float64))
            if self.params.sortNodes:
                # k .= sortslices(k, dims=2): the caller's array is sorted in place
                _check(lib.nfft_sort_nodes(self.precision, D, M, ctypes.c_void_p(kc.ctypes.data), 0,
                                           ctypes.c_void_p(self._stream)))
                if kk.flags.writeable:
                    kk[...] = kc.T
            rc = lib.nfft_set_nodes(self._handle, ctypes.c_void_p(kc.ctypes.data), 0)
            self.k = np.asarray(kk, dtype=kc.dtype) if not self.params.sortNodes else np.ascontiguousarray(kc.T)
        _check(rc)
        self._timing_update()
        return self

    def _destroy_handle(self):
        if self._handle is not None and self._handle.value:
            L.load().nfft_plan_destroy(self._handle)
        self._handle = None

    def copy(self):
        """copy(p): an independent plan with the same nodes."""
        return GB300NFFTPlan(self.k, self.N, m=self.params.m, sigma=self.params.sigma, window=self.params.window,
                             precompute=self.params.precompute, blocking=self.params.blocking,
                             sortNodes=self.params.sortNodes,
                             blockSize=self.params.blockSize, compensated=self.params.compensated,
                             timing=self._timing, device=self.device)

    def _read_timing(self):
        if self._handle is None or not self._handle.value:
            return None
        t = (ctypes.c_double * 7)()
        _check(L.load().nfft_get_timing(self._handle, t))
        return tuple(t)

    def _timing_update(self):
        """Bind the plan's TimingStats to this plan's event records (no sync)."""
        if self._timing is not None and self._timing._source is None:
            self._timing._source = weakref.WeakMethod(self._read_timing)

    def _image(self, f):
        if not isinstance(f, torch.Tensor) or tuple(f.shape) != self.N:
            raise DimensionMismatch("Data is not consistent with NFFTPlan")
        if f.dtype != self.cdtype or f.device != self.device or not _is_colmajor(f):
            raise ArgumentError(f"image must be a column-major {self.cdtype} tensor on {self.device}")
        return f

    def _nodevec(self, v, dtype=None):
        dtype = dtype or self.cdtype
        if not isinstance(v, torch.Tensor) or tuple(v.shape) != self.NOut:
            raise DimensionMismatch("Data is not consistent with NFFTPlan")
        if v.dtype != dtype or v.device != self.device or not v.is_contiguous():
            raise ArgumentError(f"node vector must be a contiguous {dtype} tensor on {self.device}")
        return v

    def forward_(self, fHat, f):
        """mul!(fHat, p, f)."""
        f = self._image(f)
        fHat = self._nodevec(fHat)
        self._sync_stream()
        _check(L.load().nfft_forward(self._handle, _ptr(f), _ptr(fHat)))
        self._timing_update()
        return fHat

    def adjoint_(self, f, fHat):
        """mul!(f, adjoint(p), fHat)."""
        f = self._image(f)
        fHat = self._nodevec(fHat)
        self._sync_stream()
        _check(L.load().nfft_adjoint(self._handle, _ptr(fHat), _ptr(f)))
        self._timing_update()
        return f

    def __mul__(self, f):
        f = as_colmajor(f, self.N, self.cdtype, self.device)
        fHat = torch.empty(self.NOut, dtype=self.cdtype, device=self.device)
        return self.forward_(fHat, f)

    def adjoint(self):
        return AdjointPlan(self)

    @property
    def H(self):
        return AdjointPlan(self)

    def __repr__(self):
        return (f"GB300NFFTPlan with {self.J} sampling points for an input array of size{self.N} and an output "
                f"array of size{self.NOut} with dims {self.dims}")

    # ------------------------------------------------------ optional interface
    def convolve_(self, g, fHat):
        """convolve!(p, g, fHat) (src/convolution.jl:20-53)."""
        g_real = not g.is_complex()
        f_real = not fHat.is_complex()
        if not g_real and f_real:
            raise ArgumentError("Complex input g requires Complex output fHat")
        if tuple(g.shape) != self.Ñ:
            raise DimensionMismatch(f"size(g)={tuple(g.shape)} ≠ Ñ = {self.Ñ}")
        if tuple(fHat.shape) != (self.J,):
            raise DimensionMismatch(f"size(fHat)={tuple(fHat.shape)} ≠ J = {self.J}")
        gd = self.dtype if g_real else self.cdtype
        fd = self.dtype if f_real else self.cdtype
        if g.dtype != gd or not _is_colmajor(g) or fHat.dtype != fd or not fHat.is_contiguous():
            raise ArgumentError("convolve! needs column-major arrays of the plan's element type")
        self._sync_stream()
        _check(L.load().nfft_convolve(self._handle, _ptr(g), int(g_real), _ptr(fHat), int(f_real)))
        return fHat

    def convolve_transpose_(self, fHat, g):
        """convolve_transpose!(p, fHat, g) (src/convolution.jl:115-149)."""
        f_real = not fHat.is_complex()
        g_real = not g.is_complex()
        if not f_real and g_real:
            raise ArgumentError("Complex input fHat requires Complex output g")
        if tuple(g.shape) != self.Ñ:
            raise DimensionMismatch(f"size(g)={tuple(g.shape)} ≠ Ñ = {self.Ñ}")
        if tuple(fHat.shape) != (self.J,):
            raise DimensionMismatch(f"size(fHat)={tuple(fHat.shape)} ≠ J = {self.J}")
        gd = self.dtype if g_real else self.cdtype
        fd = self.dtype if f_real else self.cdtype
        if g.dtype != gd or not _is_colmajor(g) or fHat.dtype != fd or not fHat.is_contiguous():
            raise ArgumentError("convolve_transpose! needs column-major arrays of the plan's element type")
        self._sync_stream()
        _check(L.load().nfft_convolve_transpose(self._handle, _ptr(fHat), int(f_real), _ptr(g), int(g_real)))
        return g

    def deconvolve_(self, f, g):
        """deconvolve!(p, f, g) (src/deconvolution.jl:2-45)."""
        f = self._image(f)
        if tuple(g.shape) != self.Ñ or g.dtype != self.cdtype or not _is_colmajor(g):
            raise DimensionMismatch("g must be a column-major complex array of size Ñ")
        self._sync_stream()
        _check(L.load().nfft_deconvolve(self._handle, _ptr(f), _ptr(g)))
        return g

    def deconvolve_transpose_(self, g, f):
        """deconvolve_transpose!(p, g, f) (src/deconvolution.jl:49-92)."""
        f = self._image(f)
        if tuple(g.shape) != self.Ñ or g.dtype != self.cdtype or not _is_colmajor(g):
            raise DimensionMismatch("g must be a column-major complex array of size Ñ")
        self._sync_stream()
        _check(L.load().nfft_deconvolve_transpose(self._handle, _ptr(g), _ptr(f)))
        return f

    def grad_nodes_(self, dk, v, w):
        """dk[d, j] = Re(conj(w_j) * d(A v)_j / dk[d, j]) (dk: real (D, M)
        column-major, i.e. a (M, D) contiguous buffer viewed transposed)."""
        v = self._image(v)
        w = self._nodevec(w)
        if tuple(dk.shape) != (len(self.N), self.J) or dk.dtype != self.dtype or dk.stride()[0] != 1:
            raise ArgumentError("dk must be a column-major real (D, M) tensor")
        self._sync_stream()
        _check(L.load().nfft_grad_nodes(self._handle, _ptr(v), _ptr(w), _ptr(dk)))
        return dk

    def autotune(self, use_cache=True):
        """Pick the fastest spreading tile shape for these nodes (re-bins)."""
        self._sync_stream()
        _check(L.load().nfft_autotune(self._handle, int(bool(use_cache))))
        self._refresh_info()
        return self.params.blockSize

    def set_block_size(self, bs, row_parity_warps=None):
        """Re-tile the plan (blockSize) and re-bin its nodes; for D = 3,
        row_parity_warps = 2 spreads with 16 warps per tile (nfft_set_tiling)."""
        arr = (ctypes.c_int64 * 3)(*(list(bs) + [1] * (3 - len(bs))))
        self._sync_stream()
        if row_parity_warps is None:
            _check(L.load().nfft_set_block_size(self._handle, arr))
        else:
            _check(L.load().nfft_set_tiling(self._handle, arr, int(row_parity_warps)))
        self._refresh_info()
        return self.params.blockSize

    def _refresh_info(self):
        info = L.nfft_info()
        _check(L.load().nfft_get_info(self._handle, ctypes.byref(info)))
        self._info = info
        self.params.blockSize = tuple(int(info.block_size[d]) for d in range(len(self.N)))

    # -------------------------------------------------------------- diagnostics
    def binning(self):
        """Integer outputs of the device binning (host numpy arrays)."""
        M = self.J
        perm = np.zeros(max(M, 1), np.int32)
        ts = np.zeros(int(self._info.num_tiles) + 1, np.int32)
        gi = np.zeros(max(M * len(self.N), 1), np.int32)
        P32 = ctypes.POINTER(ctypes.c_int32)
        _check(L.load().nfft_get_binning(self._handle, perm.ctypes.data_as(P32), ts.ctypes.data_as(P32),
                                         gi.ctypes.data_as(P32)))
        return dict(perm=perm[:M], tile_start=ts, grid_index=gi[:M * len(self.N)].reshape(M, len(self.N)).T.copy())

    def deconv_factors(self):
        n = sum(self.N)
        out = np.zeros(n, np.float32 if self.precision == 32 else np.float64)
        _check(L.load().nfft_get_deconv_factors(self._handle, ctypes.c_void_p(out.ctypes.data)))
        res, o = [], 0
        for nd in self.N:
            res.append(out[o:o + nd].copy())
            o += nd
        return res

    def info(self):
        i = L.nfft_info()
        _check(L.load().nfft_get_info(self._handle, ctypes.byref(i)))
        return {f: (tuple(getattr(i, f)) if hasattr(getattr(i, f), "__len__") else getattr(i, f))
                for f, _ in i._fields_}

    def synchronize(self):
        _check(L.load().nfft_sync(self._handle))


class AdjointPlan:
    """adjoint(p) (AbstractNFFTs/src/interface.jl:122-123)."""

    def __init__(self, parent):
        self.parent = parent

    def size_in(self):
        return self.parent.NOut

    def size_out(self):
        return self.parent.N

    def __mul__(self, fHat):
        p = self.parent
        if not isinstance(fHat, torch.Tensor):
            fHat = torch.as_tensor(np.asarray(fHat))
        if tuple(fHat.shape) != p.NOut:
            raise DimensionMismatch("Data is not consistent with NFFTPlan")
        if len(p.NOut) > 1:  # directional plans: column-major node-value arrays
            fHat = as_colmajor(fHat, p.NOut, p.cdtype, p.device)
        else:
            fHat = fHat.to(device=p.device, dtype=p.cdtype).contiguous()
        f = empty_image(p.N, p.cdtype, p.device)
        return p.adjoint_(f, fHat)

    def adjoint(self):
        return self.parent

    def copy(self):
        return AdjointPlan(self.parent.copy())

    def __repr__(self):
        return "Adjoint " + repr(self.parent)


def adjoint(p):
    return p.adjoint()


def plan_nfft(*args, **kwargs):
    """plan_nfft([CuArray,] k, N; m, σ, reltol, window, precompute, blocking, ...).

    The optional leading array type mirrors ``plan_nfft(CuArray, k, N)``; any
    value there is accepted and ignored (plans always live on the GPU).
    ``σ`` may be passed as ``sigma`` or ``σ``.
    """
    if args and (isinstance(args[0], type) or args[0] is None):
        args = args[1:]
    k, N = args[0], args[1]
    if "σ" in kwargs:
        kwargs["sigma"] = kwargs.pop("σ")
    timing = kwargs.get("timing")
    if isinstance(N, int):
        N = (N,)
    dims = kwargs.pop("dims", None)
    if dims is not None:
        r = _dims_range(dims, len(N))
        if r != (1, len(N)):
            return GB300DirectionalPlan(k, N, dims=r, **kwargs)
    p = GB300NFFTPlan(k, N, **kwargs)
    if timing is not None:
        timing.pre = p._timing.pre if p._timing is not None else 0.0
    return p


def mul_(out, p, x):
    """mul!(out, p, x) for a plan or an adjoint plan."""
    if isinstance(p, AdjointPlan):
        return p.parent.adjoint_(out, x)
    return p.forward_(out, x)


def nodes_(p, k):
    return p.nodes_(k)


def size_in(p):
    return p.size_in()


def size_out(p):
    return p.size_out()


def convolve_(p, g, fHat):
    return p.convolve_(g, fHat)


def convolve_transpose_(p, fHat, g):
    return p.convolve_transpose_(fHat, g)


def deconvolve_(p, f, g):
    return p.deconvolve_(f, g)


def deconvolve_transpose_(p, g, f):
    return p.deconvolve_transpose_(g, f)


def nfft(k, f, **kw):
    """nfft(k, f) = plan_nfft(k, size(f)) * f (AbstractNFFTs/src/derived.jl:134-150)."""
    return plan_nfft(k, tuple(f.shape), **kw) * f


def nfft_adjoint(k, N, fHat, **kw):
    """nfft_adjoint(k, N, fHat) = adjoint(plan_nfft(k, N)) * fHat (:152-166)."""
    return adjoint(plan_nfft(k, N, **kw)) * fHat


def kernel_launch_count():
    return int(L.load().nfft_kernel_launch_count())


class NFFTBatch:
    """Many plans transformed together (nfft_batch_* of include/nfft_gb300.h).

    No reference counterpart: NFFT.jl runs one plan per ``mul!``.  Members
    need nodes, ``blocking=True``, ``compensated=False``, D = 2 or 3 and the
    same precision, D, ``m`` and window-evaluation mode; each stage runs as
    one launch over all plans, the whole direction replayed as a CUDA graph.
    The batch runs on the stream current at creation; calls must be made
    with that stream current.  After ``nodes_`` on a member, build the batch
    again.
    """

    def __init__(self, plans):
        plans = list(plans)
        if not plans:
            raise ArgumentError("need at least one plan")
        dev = plans[0].device
        if any(p.device != dev for p in plans):
            raise ArgumentError("plans of a batch must live on one device")
        self.plans = plans
        self.device = dev
        lib = L.load()
        arr = (ctypes.c_void_p * len(plans))(*[p._handle.value for p in plans])
        h = ctypes.c_void_p()
        with torch.cuda.device(dev):
            self._stream = torch.cuda.current_stream(dev).cuda_stream
            _check(lib.nfft_batch_create(ctypes.byref(h), arr, len(plans), ctypes.c_void_p(self._stream)))
        self._handle = h
        for p in plans:
            p._stream = None  # the batch re-bound the plan's stream; the next plan call re-binds it
        self._keep = plans

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                L.load().nfft_batch_destroy(h)
            except Exception:
                pass
            self._handle = None

    def __len__(self):
        return len(self.plans)

    def _call(self, fn, ins, outs):
        if len(ins) != len(self.plans) or len(outs) != len(self.plans):
            raise DimensionMismatch(f"need {len(self.plans)} inputs and outputs")
        if torch.cuda.current_stream(self.device).cuda_stream != self._stream:
            raise ArgumentError("call the batch with the stream current at its creation")
        n = len(self.plans)
        a = (ctypes.c_void_p * n)(*[t.data_ptr() for t in ins])
        b = (ctypes.c_void_p * n)(*[t.data_ptr() for t in outs])
        _check(fn(self._handle, a, b))

    def _lengths(self, *lists):
        for x in lists:
            if len(x) != len(self.plans):
                raise DimensionMismatch(f"need {len(self.plans)} inputs and outputs, got {len(x)}")

    def forward_(self, fHats, fs):
        """mul!(fHats[i], plans[i], fs[i]) for every i."""
        self._lengths(fHats, fs)
        fs = [p._image(f) for p, f in zip(self.plans, fs)]
        fHats = [p._nodevec(v) for p, v in zip(self.plans, fHats)]
        self._call(L.load().nfft_batch_forward, fs, fHats)
        return fHats

    def adjoint_(self, fs, fHats):
        """mul!(fs[i], adjoint(plans[i]), fHats[i]) for every i."""
        self._lengths(fHats, fs)
        fs = [p._image(f) for p, f in zip(self.plans, fs)]
        fHats = [p._nodevec(v) for p, v in zip(self.plans, fHats)]
        self._call(L.load().nfft_batch_adjoint, fHats, fs)
        return fs

    def forward(self, fs):
        self._lengths(fs)
        outs = [torch.empty(p.NOut, dtype=p.cdtype, device=p.device) for p in self.plans]
        return self.forward_(outs, [as_colmajor(f, p.N, p.cdtype, p.device) for p, f in zip(self.plans, fs)])

    def adjoint(self, fHats):
        self._lengths(fHats)
        outs = [empty_image(p.N, p.cdtype, p.device) for p in self.plans]
        return self.adjoint_(outs, [v.to(device=p.device, dtype=p.cdtype).contiguous()
                                    for p, v in zip(self.plans, fHats)])


def _dims_range(dims, D):
    """dims as an Integer or a UnitRange (1-based, inclusive) -> (lo, hi)."""
    if isinstance(dims, (int, np.integer)):
        lo = hi = int(dims)
    elif isinstance(dims, range):
        if dims.step != 1 or len(dims) == 0:
            raise ArgumentError("dims must be a contiguous range")
        lo, hi = dims.start, dims.stop - 1
    else:
        d = [int(x) for x in np.atleast_1d(dims)]
        if d != list(range(d[0], d[0] + len(d))):
            raise ArgumentError("dims must be a contiguous range")
        lo, hi = d[0], d[-1]
    if lo < 1 or hi > D:
        raise ArgumentError(f"dims {lo}:{hi} do not fit a {D}-dimensional array")
    return lo, hi


class GB300DirectionalPlan:
    """NFFTPlan with ``dims`` (src/directional.jl, src/implementation.jl:73-104):
    the NFFT along the contiguous dimensions ``dims`` of an array of size N,
    every other index a batch column.  ``k`` is len(dims) x J; NOut is N with
    the dims range replaced by J.  precompute is LINEAR, as in the reference.
    Node-value arrays (fHat) are column-major of shape NOut."""

    def __init__(self, k, N, *, dims, m=None, sigma=None, reltol=None, window="kaiser_bessel",
                 precompute=None, blocking=None, sortNodes=False, storeDeconvolutionIdx=False, blockSize=None,
                 compensated=False, timing=None, fftflags=None, device="cuda"):
        kk = GB300NFFTPlan._nodes_array(k)
        N = tuple(int(n) for n in N)
        lo, hi = dims
        R = hi - lo + 1
        if kk.shape[0] != R:
            raise ArgumentError(f"Nodes x have dimension {kk.shape[0]} != {R}")
        if len(N) > 3:
            raise NotImplementedError("directional plans support arrays of up to 3 dimensions")
        if window not in WINDOWS:
            raise NotImplementedError(f"Window {window} not yet implemented!")
        m_, s_, r_ = accuracy_params(m, sigma, reltol)
        dt = kk.dtype if isinstance(kk, np.ndarray) else {torch.float32: np.float32,
                                                          torch.float64: np.float64}[kk.dtype]
        self.precision = 32 if dt == np.float32 else 64
        self.dtype = torch.float32 if self.precision == 32 else torch.float64
        self.cdtype = torch.complex64 if self.precision == 32 else torch.complex128
        dev = torch.device(device)
        if dev.type == "cuda" and dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        self.N = N
        self.dims = tuple(range(lo, hi + 1))
        self.J = int(kk.shape[1])
        self.NOut = N[:lo - 1] + (self.J,) + N[hi:]
        self.params = NFFTParams(m=m_, sigma=s_, reltol=r_, window=window, precompute=PrecomputeFlags.LINEAR,
                                 sortNodes=bool(sortNodes), storeDeconvolutionIdx=bool(storeDeconvolutionIdx),
                                 blocking=False, blockSize=tuple(blockSize or ()), compensated=False)
        lib = L.load()
        prm = L.nfft_params()
        lib.nfft_params_default(ctypes.byref(prm))
        prm.m = m_
        prm.sigma = s_
        prm.window = WINDOWS[window]
        prm.precompute = int(PrecomputeFlags.LINEAR)
        prm.blocking = 0
        Narr = (ctypes.c_int64 * 3)(*(list(N) + [1] * (3 - len(N))))
        h = ctypes.c_void_p()
        with torch.cuda.device(dev):
            stream = torch.cuda.current_stream(dev)
            _check(lib.nfft_dplan_create(ctypes.byref(h), self.precision, len(N), Narr, lo - 1, hi - 1, self.J,
                                         ctypes.byref(prm), ctypes.c_void_p(stream.cuda_stream)))
        self._handle = h
        self._stream = stream.cuda_stream
        sig = 2.0 * ((int(np.ceil(s_ * N[lo - 1])) // 2)) / N[lo - 1]
        self.params.sigma = sig
        self.Ñ = tuple(2 * (int(np.ceil(s_ * n)) // 2) if lo - 1 <= d <= hi - 1 else n for d, n in enumerate(N))
        self.Ntilde = self.Ñ
        self.nodes_(kk)

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                L.load().nfft_dplan_destroy(h)
            except Exception:
                pass
            self._handle = None

    def _sync_stream(self):
        s = torch.cuda.current_stream(self.device).cuda_stream
        if s != self._stream:
            _check(L.load().nfft_dplan_set_stream(self._handle, ctypes.c_void_p(s)))
            self._stream = s

    def nodes_(self, k):
        kk = GB300NFFTPlan._nodes_array(k)
        if kk.shape[0] != len(self.dims):
            raise ArgumentError(f"Nodes x have dimension {kk.shape[0]} != {len(self.dims)}")
        if kk.shape[1] != self.J:
            raise DimensionMismatch("nodes! on a directional plan keeps the node count")
        self._sync_stream()
        lib = L.load()
        if isinstance(kk, torch.Tensor):
            kt = kk.to(device=self.device, dtype=self.dtype).t().contiguous()
            rc = lib.nfft_dplan_set_nodes(self._handle, _ptr(kt), 1)
        else:
            kc = np.ascontiguousarray(kk.T.astype(np.float32 if self.precision == 32 else np.float64))
            rc = lib.nfft_dplan_set_nodes(self._handle, ctypes.c_void_p(kc.ctypes.data), 0)
        _check(rc)
        self.k = kk
        return self

    def size_in(self):
        return self.N

    def size_out(self):
        return self.NOut

    def _arr(self, x, shape):
        if not isinstance(x, torch.Tensor) or tuple(x.shape) != shape:
            raise DimensionMismatch("Data is not consistent with NFFTPlan")
        if x.dtype != self.cdtype or x.device != self.device or not _is_colmajor(x):
            raise ArgumentError(f"arrays must be column-major {self.cdtype} tensors on {self.device}")
        return x

    def forward_(self, fHat, f):
        f = self._arr(f, self.N)
        fHat = self._arr(fHat, self.NOut)
        self._sync_stream()
        _check(L.load().nfft_dplan_forward(self._handle, _ptr(f), _ptr(fHat)))
        return fHat

    def adjoint_(self, f, fHat):
        f = self._arr(f, self.N)
        fHat = self._arr(fHat, self.NOut)
        self._sync_stream()
        _check(L.load().nfft_dplan_adjoint(self._handle, _ptr(fHat), _ptr(f)))
        return f

    def __mul__(self, f):
        f = as_colmajor(f, self.N, self.cdtype, self.device)
        return self.forward_(empty_image(self.NOut, self.cdtype, self.device), f)

    def adjoint(self):
        return AdjointPlan(self)

    @property
    def H(self):
        return AdjointPlan(self)

    def copy(self):
        return GB300DirectionalPlan(self.k, self.N, dims=(self.dims[0], self.dims[-1]), m=self.params.m,
                                    sigma=self.params.sigma, window=self.params.window, device=self.device)

    def __repr__(self):
        return (f"GB300DirectionalPlan with {self.J} sampling points for an input array of size{self.N} and an "
                f"output array of size{self.NOut} with dims {self.dims}")
