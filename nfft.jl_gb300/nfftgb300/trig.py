"""Direct transforms and NFCT / NFST plans on the GPU.

Also a fast NNFFT plan (``plan_nnfft`` / ``GB300NNFFTPlan``: the transform of
``NNDFTPlan`` computed with two NFFT plans, ``nfft_nnplan_*``).

Mirrors NFFT.jl's direct plans (src/direct.jl: ``NDFTPlan``, ``NDCTPlan``,
``NDSTPlan``, ``NNDFTPlan`` with ``ndft``, ``ndft_adjoint``, ``ndct``,
``ndct_transposed``) and AbstractNFFTs' NFCT / NFST interface
(``plan_nfct``, ``plan_nfst``, ``nfct``, ``nfct_transpose``, ``nfst``,
``nfst_transpose``; AbstractNFFTs/src/interface.jl:73-90, derived.jl:134-160)
on the library's ``nfft_direct`` and ``nfft_tplan_*`` entry points.

Layouts follow Julia: images are column-major tensors of logical shape N
(``empty_image``), node vectors contiguous, nodes D x J.  NFCT / NFST data is
real; NDFT / NNDFT data complex.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib as L
from . import plan as P

NDFT, NDCT, NDST, NNDFT = 0, 1, 2, 3


def _device(device):
    dev = torch.device(device)
    if dev.type == "cuda" and dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    return dev


def _nodes_tensor(k, device, dtype=None):
    """k (D x J, numpy or torch; a vector is 1 x J) -> (D, J) and a contiguous
    device tensor in column-major D x J order (coordinate fastest)."""
    kk = P.GB300NFFTPlan._nodes_array(k)
    if dtype is None:
        dtype = torch.float32 if kk.dtype in (np.float32, torch.float32) else torch.float64
    if isinstance(kk, torch.Tensor):
        kt = kk.to(device=device, dtype=dtype).t().contiguous()
    else:
        kt = torch.from_numpy(np.ascontiguousarray(kk.T)).to(device=device, dtype=dtype)
    return tuple(kk.shape), kt, dtype


class _DirectPlan:
    """Shared part of the direct plans: nodes on the device, one
    ``nfft_direct`` call per product."""

    kind = NDFT
    complex_data = True

    def __init__(self, k, N, device="cuda"):
        self.device = _device(device)
        (D, J), self._k, self.dtype = _nodes_tensor(k, self.device)
        if isinstance(N, int):
            N = (N,)
        self.N = tuple(int(n) for n in N)
        if D != len(self.N):
            raise P.ArgumentError(f"Nodes x have dimension {D} != {len(self.N)}")
        if D > 4:
            raise NotImplementedError("direct transforms support D <= 4")
        self.D, self.J = D, J
        self.k = k
        self.cdtype = torch.complex64 if self.dtype == torch.float32 else torch.complex128
        self.precision = 32 if self.dtype == torch.float32 else 64

    def size_in(self):
        return self.N

    def size_out(self):
        return (self.J,)

    def _data_dtype(self, cplx):
        return self.cdtype if cplx else self.dtype

    def _run(self, adjoint, x, out, cplx):
        lib = L.load()
        Narr = (ctypes.c_int64 * 4)(*(list(self._Narg()) + [1] * (4 - len(self._Narg()))))
        y = self._y if self.kind == NNDFT else None
        stream = torch.cuda.current_stream(self.device).cuda_stream
        P._check(lib.nfft_direct(self.kind, self.precision, self.D, Narr, self.J, P._ptr(self._k),
                                 P._ptr(y) if y is not None else None, int(adjoint), int(cplx), P._ptr(x),
                                 P._ptr(out), ctypes.c_void_p(stream)))
        return out

    def _Narg(self):
        return self.N

    def _check_image(self, f, cplx):
        if not isinstance(f, torch.Tensor) or tuple(f.shape) != self.size_in():
            raise P.DimensionMismatch(f"Data f is not consistent with {type(self).__name__}")
        if f.dtype != self._data_dtype(cplx) or f.device != self.device or not P._is_colmajor(f):
            raise P.ArgumentError(f"image must be a column-major {self._data_dtype(cplx)} tensor on {self.device}")
        return f

    def _check_nodevec(self, v, cplx):
        if not isinstance(v, torch.Tensor) or tuple(v.shape) != (self.J,):
            raise P.DimensionMismatch(f"Data fHat is not consistent with {type(self).__name__}")
        if v.dtype != self._data_dtype(cplx) or v.device != self.device or not v.is_contiguous():
            raise P.ArgumentError(f"node vector must be a contiguous {self._data_dtype(cplx)} tensor")
        return v

    def _cplx_of(self, t):
        if self.complex_data:
            return True
        return t.is_complex() if isinstance(t, torch.Tensor) else bool(np.iscomplexobj(t))

    def forward_(self, fHat, f):
        """mul!(fHat, p, f)."""
        cplx = self.complex_data or f.is_complex()
        self._check_image(f, cplx)
        self._check_nodevec(fHat, cplx)
        return self._run(False, f, fHat, cplx)

    def _backward_(self, f, fHat):
        cplx = self.complex_data or fHat.is_complex()
        self._check_nodevec(fHat, cplx)
        self._check_image(f, cplx)
        return self._run(True, fHat, f, cplx)

    def __mul__(self, f):
        cplx = self._cplx_of(f)
        f = P.as_colmajor(f, self.size_in(), self._data_dtype(cplx), self.device)
        out = torch.empty(self.J, dtype=self._data_dtype(cplx), device=self.device)
        return self.forward_(out, f)

    def _backward_mul(self, fHat):
        cplx = self._cplx_of(fHat)
        if not isinstance(fHat, torch.Tensor):
            fHat = torch.as_tensor(np.asarray(fHat))
        fHat = fHat.to(device=self.device, dtype=self._data_dtype(cplx)).contiguous()
        f = P.empty_image(self.size_in(), self._data_dtype(cplx), self.device)
        return self._backward_(f, fHat)


class _AdjointOf:
    def __init__(self, parent):
        self.parent = parent

    def __mul__(self, fHat):
        return self.parent._backward_mul(fHat)

    def mul_(self, f, fHat):
        return self.parent._backward_(f, fHat)


class NDFTPlan(_DirectPlan):
    """NDFTPlan(k, N) (src/direct.jl:1-45, :99-151): exact NDFT on the GPU."""

    kind = NDFT

    def adjoint_(self, f, fHat):
        """mul!(f, adjoint(p), fHat)."""
        return self._backward_(f, fHat)

    def adjoint(self):
        return _AdjointOf(self)

    @property
    def H(self):
        return _AdjointOf(self)


class NDCTPlan(_DirectPlan):
    """NDCTPlan(k, N) (src/direct.jl:153-199): exact cosine transform, real
    (or complex) data."""

    kind = NDCT
    complex_data = False

    def transpose_(self, f, fHat):
        """mul!(f, transpose(p), fHat)."""
        return self._backward_(f, fHat)

    def transpose(self):
        return _AdjointOf(self)

    @property
    def T(self):
        return _AdjointOf(self)


class NDSTPlan(NDCTPlan):
    """NDSTPlan(k, N) (src/direct.jl:202-249): exact sine transform;
    size_in = N .- 1."""

    kind = NDST

    def size_in(self):
        return tuple(n - 1 for n in self.N)


class NNDFTPlan(NDFTPlan):
    """NNDFTPlan(k, y) (src/direct.jl:29-37, :252-287): exact transform
    between nodes k (D x J) and points y (D x N)."""

    kind = NNDFT

    def __init__(self, k, y, device="cuda"):
        dev = _device(device)
        (Dk, J), kt, dtype = _nodes_tensor(k, dev)
        (Dy, Ny), yt, _ = _nodes_tensor(y, dev, dtype)
        if Dk != Dy:
            raise P.ArgumentError(f"Nodes k have dimension {Dk} != {Dy} of the points y")
        if Dk > 4:
            raise NotImplementedError("direct transforms support D <= 4")
        self.device, self._k, self.dtype = dev, kt, dtype
        self._y = yt
        self.D, self.J = Dk, J
        self.N = Ny
        self.k, self.y = k, y
        self.cdtype = torch.complex64 if dtype == torch.float32 else torch.complex128
        self.precision = 32 if dtype == torch.float32 else 64

    def size_in(self):
        return (self.N,)

    def _Narg(self):
        return (self.N,)


def ndft(k, f, device="cuda"):
    """ndft(k, f) (src/direct.jl:81-82)."""
    f_shape = tuple(f.shape)
    return NDFTPlan(k, f_shape, device) * f


def ndft_adjoint(k, N, fHat, device="cuda"):
    """ndft_adjoint(k, N, fHat) (src/direct.jl:84-85)."""
    return NDFTPlan(k, N, device).adjoint() * fHat


def ndct(k, f, device="cuda"):
    """ndct(k, f) (src/direct.jl:87-88)."""
    return NDCTPlan(k, tuple(f.shape), device) * f


def ndct_transposed(k, N, fHat, device="cuda"):
    """ndct_transposed(k, N, fHat) (src/direct.jl:90-91)."""
    return NDCTPlan(k, N, device).transpose() * fHat


# AbstractNFFTs exports the name ndct_transpose (AbstractNFFTs/src/AbstractNFFTs.jl:25)
ndct_transpose = ndct_transposed


# ------------------------------------------------------------ NFCT / NFST
class _TrigPlan:
    """NFCT / NFST plan of size N on the GPU NFFT (size 2N) of the even / odd
    extension; real data of the nodes' type."""

    kind = NDCT

    def __init__(self, k, N, *, m=None, sigma=None, reltol=None, window="kaiser_bessel",
                 precompute=P.PrecomputeFlags.POLYNOMIAL, blocking=True, blockSize=None, device="cuda", **_):
        self.device = _device(device)
        if isinstance(N, int):
            N = (N,)
        self.N = tuple(int(n) for n in N)
        kk = P.GB300NFFTPlan._nodes_array(k)
        D, J = kk.shape
        if D != len(self.N):
            raise P.ArgumentError(f"Nodes x have dimension {D} != {len(self.N)}")
        if window not in P.WINDOWS:
            raise NotImplementedError(f"Window {window} not yet implemented!")
        m_, s_, r_ = P.accuracy_params(m, sigma, reltol)
        self.dtype = torch.float32 if kk.dtype in (np.float32, torch.float32) else torch.float64
        self.precision = 32 if self.dtype == torch.float32 else 64
        self.D, self.J = D, J
        self.params = P.NFFTParams(m=m_, sigma=s_, reltol=r_, window=window,
                                   precompute=P.PrecomputeFlags(precompute), blocking=bool(blocking),
                                   blockSize=tuple(blockSize or ()))
        lib = L.load()
        prm = L.nfft_params()
        lib.nfft_params_default(ctypes.byref(prm))
        prm.m = m_
        prm.sigma = s_
        prm.window = P.WINDOWS[window]
        prm.precompute = int(precompute)
        prm.blocking = int(bool(blocking))
        for d, b in enumerate(tuple(blockSize or ())[:3]):
            prm.block_size[d] = int(b)
        Narr = (ctypes.c_int64 * 3)(*(list(self.N) + [1] * (3 - D)))
        h = ctypes.c_void_p()
        self._handle = None
        with torch.cuda.device(self.device):
            stream = torch.cuda.current_stream(self.device).cuda_stream
            P._check(lib.nfft_tplan_create(ctypes.byref(h), self.kind, self.precision, D, Narr, int(J),
                                           ctypes.byref(prm), ctypes.c_void_p(stream)))
        self._handle = h
        self._stream = stream
        self.nodes_(kk)

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                L.load().nfft_tplan_destroy(h)
            except Exception:
                pass
            self._handle = None

    def _sync_stream(self):
        s = torch.cuda.current_stream(self.device).cuda_stream
        if s != self._stream:
            P._check(L.load().nfft_tplan_set_stream(self._handle, ctypes.c_void_p(s)))
            self._stream = s

    def size_in(self):
        return self.N

    def size_out(self):
        return (self.J,)

    def nodes_(self, k):
        """nodes!(p, k)."""
        kk = P.GB300NFFTPlan._nodes_array(k)
        if kk.shape != (self.D, self.J):
            raise P.DimensionMismatch(f"nodes must be {self.D} x {self.J}")
        self._sync_stream()
        if isinstance(kk, torch.Tensor):
            kt = kk.to(device=self.device, dtype=self.dtype).t().contiguous()
            P._check(L.load().nfft_tplan_set_nodes(self._handle, P._ptr(kt), 1))
        else:
            kc = np.ascontiguousarray(kk.T.astype(np.float32 if self.precision == 32 else np.float64))
            P._check(L.load().nfft_tplan_set_nodes(self._handle, ctypes.c_void_p(kc.ctypes.data), 0))
        self.k = kk
        return self

    def _image(self, f):
        if not isinstance(f, torch.Tensor) or tuple(f.shape) != self.size_in():
            raise P.DimensionMismatch(f"Data f is not consistent with {type(self).__name__}")
        if f.dtype != self.dtype or f.device != self.device or not P._is_colmajor(f):
            raise P.ArgumentError(f"image must be a column-major {self.dtype} tensor on {self.device}")
        return f

    def _nodevec(self, v):
        if not isinstance(v, torch.Tensor) or tuple(v.shape) != (self.J,):
            raise P.DimensionMismatch(f"Data fHat is not consistent with {type(self).__name__}")
        if v.dtype != self.dtype or v.device != self.device or not v.is_contiguous():
            raise P.ArgumentError(f"node vector must be a contiguous {self.dtype} tensor on {self.device}")
        return v

    def forward_(self, fHat, f):
        """mul!(fHat, p, f)."""
        f = self._image(f)
        fHat = self._nodevec(fHat)
        self._sync_stream()
        P._check(L.load().nfft_tplan_forward(self._handle, P._ptr(f), P._ptr(fHat)))
        return fHat

    def transpose_(self, f, fHat):
        """mul!(f, transpose(p), fHat)."""
        f = self._image(f)
        fHat = self._nodevec(fHat)
        self._sync_stream()
        P._check(L.load().nfft_tplan_transpose(self._handle, P._ptr(fHat), P._ptr(f)))
        return f

    def __mul__(self, f):
        f = P.as_colmajor(f, self.size_in(), self.dtype, self.device)
        fHat = torch.empty(self.J, dtype=self.dtype, device=self.device)
        return self.forward_(fHat, f)

    def _backward_mul(self, fHat):
        if not isinstance(fHat, torch.Tensor):
            fHat = torch.as_tensor(np.asarray(fHat))
        fHat = fHat.to(device=self.device, dtype=self.dtype).contiguous()
        f = P.empty_image(self.size_in(), self.dtype, self.device)
        return self.transpose_(f, fHat)

    def transpose(self):
        return _AdjointOf(self)

    @property
    def T(self):
        return _AdjointOf(self)


class GB300NFCTPlan(_TrigPlan):
    """NFCT plan (AbstractNFCTPlan): fHat_j = sum_{n in [0,N)} f_n prod_d cos(2 pi k_dj n_d)."""

    kind = NDCT


class GB300NFSTPlan(_TrigPlan):
    """NFST plan (AbstractNFSTPlan): fHat_j = sum_{n in [1,N-1]} f_n prod_d
    sin(2 pi k_dj n_d); size_in = N .- 1 (as NDSTPlan)."""

    kind = NDST

    def size_in(self):
        return tuple(n - 1 for n in self.N)


def plan_nfct(*args, **kwargs):
    """plan_nfct([CuArray,] k, N; m, σ, window, ...)."""
    if args and (isinstance(args[0], type) or args[0] is None):
        args = args[1:]
    if "σ" in kwargs:
        kwargs["sigma"] = kwargs.pop("σ")
    return GB300NFCTPlan(args[0], args[1], **kwargs)


def plan_nfst(*args, **kwargs):
    """plan_nfst([CuArray,] k, N; m, σ, window, ...); N is the plan size,
    the input has N .- 1 points."""
    if args and (isinstance(args[0], type) or args[0] is None):
        args = args[1:]
    if "σ" in kwargs:
        kwargs["sigma"] = kwargs.pop("σ")
    return GB300NFSTPlan(args[0], args[1], **kwargs)


def nfct(k, f, **kw):
    """nfct(k, f) (AbstractNFFTs/src/derived.jl:139-142)."""
    return plan_nfct(k, tuple(f.shape), **kw) * f


def nfct_transpose(k, N, fHat, **kw):
    """nfct_transpose(k, N, fHat) (derived.jl:146-149)."""
    return plan_nfct(k, N, **kw).transpose() * fHat


def nfst(k, f, **kw):
    """nfst(k, f): the plan has size size(f) .+ 1 so that f is its input
    (size_in = N .- 1)."""
    return plan_nfst(k, tuple(n + 1 for n in f.shape), **kw) * f


def nfst_transpose(k, N, fHat, **kw):
    """nfst_transpose(k, N, fHat) (derived.jl:146-149): N is the plan size."""
    return plan_nfst(k, N, **kw).transpose() * fHat


# ------------------------------------------------------------------ NNFFT
class GB300NNFFTPlan:
    """Fast NNFFT (AbstractNNFFTPlan; the transform of NNDFTPlan,
    src/direct.jl:252-287): fHat_j = sum_l c_l exp(-2 pi i k_j . y_l) with nodes
    k (D x J, |k| <= 1/2) and points y (D x N).  Computed by spreading c at
    y / N1, a forward NFFT of size sigma N1 at k / sigma1 and a division by the
    window transform (``nfft_nnplan_*``); accuracy as an NFFT with m, sigma."""

    def __init__(self, k, y, *, m=None, sigma=None, reltol=None, window="kaiser_bessel",
                 precompute=P.PrecomputeFlags.POLYNOMIAL, blocking=True, device="cuda", **_):
        self.device = _device(device)
        kk = P.GB300NFFTPlan._nodes_array(k)
        yy = P.GB300NFFTPlan._nodes_array(y)
        if kk.shape[0] != yy.shape[0]:
            raise P.ArgumentError(f"Nodes k have dimension {kk.shape[0]} != {yy.shape[0]} of the points y")
        if kk.shape[0] > 3:
            raise NotImplementedError("NNFFT plans support D <= 3")
        if window not in P.WINDOWS:
            raise NotImplementedError(f"Window {window} not yet implemented!")
        m_, s_, r_ = P.accuracy_params(m, sigma, reltol)
        self.dtype = torch.float32 if kk.dtype in (np.float32, torch.float32) else torch.float64
        self.cdtype = torch.complex64 if self.dtype == torch.float32 else torch.complex128
        self.precision = 32 if self.dtype == torch.float32 else 64
        self.D, self.J = kk.shape
        self.N = int(yy.shape[1])
        self.params = P.NFFTParams(m=m_, sigma=s_, reltol=r_, window=window,
                                   precompute=P.PrecomputeFlags(precompute), blocking=bool(blocking))
        lib = L.load()
        prm = L.nfft_params()
        lib.nfft_params_default(ctypes.byref(prm))
        prm.m = m_
        prm.sigma = s_
        prm.window = P.WINDOWS[window]
        prm.precompute = int(precompute)
        prm.blocking = int(bool(blocking))
        h = ctypes.c_void_p()
        self._handle = None
        with torch.cuda.device(self.device):
            stream = torch.cuda.current_stream(self.device).cuda_stream
            P._check(lib.nfft_nnplan_create(ctypes.byref(h), self.precision, self.D, int(self.J), self.N,
                                            ctypes.byref(prm), ctypes.c_void_p(stream)))
        self._handle = h
        self._stream = stream
        self.nodes_(kk, yy)

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                L.load().nfft_nnplan_destroy(h)
            except Exception:
                pass
            self._handle = None

    def _sync_stream(self):
        s = torch.cuda.current_stream(self.device).cuda_stream
        if s != self._stream:
            P._check(L.load().nfft_nnplan_set_stream(self._handle, ctypes.c_void_p(s)))
            self._stream = s

    def size_in(self):
        return (self.N,)

    def size_out(self):
        return (self.J,)

    def nodes_(self, k, y):
        """nodes!(p, k) with the points y."""
        kk = P.GB300NFFTPlan._nodes_array(k)
        yy = P.GB300NFFTPlan._nodes_array(y)
        if kk.shape != (self.D, self.J) or yy.shape != (self.D, self.N):
            raise P.DimensionMismatch(f"nodes must be {self.D} x {self.J} and points {self.D} x {self.N}")
        npdt = np.float32 if self.precision == 32 else np.float64
        kc = np.ascontiguousarray((kk.cpu().numpy() if isinstance(kk, torch.Tensor) else kk).T.astype(npdt))
        yc = np.ascontiguousarray((yy.cpu().numpy() if isinstance(yy, torch.Tensor) else yy).T.astype(npdt))
        self._sync_stream()
        P._check(L.load().nfft_nnplan_set_nodes(self._handle, ctypes.c_void_p(kc.ctypes.data),
                                                 ctypes.c_void_p(yc.ctypes.data), 0))
        self.k, self.y = kk, yy
        return self

    def _vec(self, v, n, what):
        if not isinstance(v, torch.Tensor) or tuple(v.shape) != (n,):
            raise P.DimensionMismatch(f"{what} is not consistent with the NNFFT plan")
        if v.dtype != self.cdtype or v.device != self.device or not v.is_contiguous():
            raise P.ArgumentError(f"{what} must be a contiguous {self.cdtype} tensor on {self.device}")
        return v

    def forward_(self, fHat, c):
        """mul!(fHat, p, c)."""
        c = self._vec(c, self.N, "input")
        fHat = self._vec(fHat, self.J, "output")
        self._sync_stream()
        P._check(L.load().nfft_nnplan_forward(self._handle, P._ptr(c), P._ptr(fHat)))
        return fHat

    def adjoint_(self, c, fHat):
        """mul!(c, adjoint(p), fHat)."""
        c = self._vec(c, self.N, "output")
        fHat = self._vec(fHat, self.J, "input")
        self._sync_stream()
        P._check(L.load().nfft_nnplan_adjoint(self._handle, P._ptr(fHat), P._ptr(c)))
        return c

    def _to_vec(self, v):
        if not isinstance(v, torch.Tensor):
            v = torch.as_tensor(np.asarray(v))
        return v.to(device=self.device, dtype=self.cdtype).contiguous()

    def __mul__(self, c):
        fHat = torch.empty(self.J, dtype=self.cdtype, device=self.device)
        return self.forward_(fHat, self._to_vec(c))

    def _backward_mul(self, fHat):
        c = torch.empty(self.N, dtype=self.cdtype, device=self.device)
        return self.adjoint_(c, self._to_vec(fHat))

    def adjoint(self):
        return _AdjointOf(self)

    @property
    def H(self):
        return _AdjointOf(self)


def plan_nnfft(*args, **kwargs):
    """plan_nnfft([CuArray,] k, y; m, σ, window, ...) (AbstractNFFTs/src/derived.jl:39-42)."""
    if args and (isinstance(args[0], type) or args[0] is None):
        args = args[1:]
    if "σ" in kwargs:
        kwargs["sigma"] = kwargs.pop("σ")
    return GB300NNFFTPlan(args[0], args[1], **kwargs)
