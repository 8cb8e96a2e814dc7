"""GPU tests of the plan interface: the reference's constructor, convolve,
chainrules, sampling-density and issue tests, restated for the GPU plan and
checked against the oracle (CPU restatement of NFFT.jl) or the NDFT."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import nfftgb300 as nf  # noqa: E402
from nfftgb300 import autodiff, tools  # noqa: E402
from oracle import oracle  # noqa: E402


def cflat(x):
    return np.asarray(x).ravel(order="F")


def rand_k(D, M, seed=0, dtype=np.float64):
    return (np.random.default_rng(seed).random((D, M)) - 0.5).astype(dtype)


def cnormal(shape, seed=1, dtype=np.complex128):
    rng = np.random.default_rng(seed)
    return ((rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)).astype(dtype)


# ------------------------------------------------------------ constructors

def test_node_range_and_nan_rejected():
    """test/constructors.jl:27-32."""
    with pytest.raises(nf.ArgumentError):
        nf.plan_nfft(np.array([[-0.6, 0.9], [0.5, -0.5]]), (2, 2))
    with pytest.raises(nf.ArgumentError):
        nf.plan_nfft(np.array([[-0.3, 0.3], [0.3, np.nan]]), (2, 2))
    with pytest.raises(nf.ArgumentError):
        nf.plan_nfft(np.zeros((1, 4)), (2, 2))  # dimension mismatch of nodes, :20


def test_tiny_plan_and_copy():
    """NFFTPlan(zeros(2,4), (2,2)) and copy(p) (test/constructors.jl:22-26):
    a grid smaller than the window wraps taps several times."""
    p = nf.plan_nfft(np.zeros((2, 4)), (2, 2))
    q = p.copy()
    assert q.N == p.N and q.Ñ == p.Ñ and q.J == p.J and q.params.m == p.params.m
    f = cnormal((2, 2))
    y1 = (p * nf.as_colmajor(f, (2, 2), torch.complex128)).cpu().numpy()
    y2 = (q * nf.as_colmajor(f, (2, 2), torch.complex128)).cpu().numpy()
    assert np.array_equal(y1, y2)
    op = oracle.OraclePlan(np.zeros((2, 4)), (2, 2))
    assert oracle.rel_l2(y1, op.forward(f)) < 1e-11
    x = (nf.adjoint(p) * torch.ones(4, dtype=torch.complex128)).cpu().numpy()
    assert oracle.rel_l2(cflat(x), cflat(op.adjoint(np.ones(4)))) < 1e-11


def test_nodes_bang_equivalent_to_new_plan():
    """nodes!(p2, trj1) gives the plan built from trj1 (test/constructors.jl:36-66)."""
    Nx = 32
    trj1, trj2 = rand_k(2, 1000, 1), rand_k(2, 1000, 2)
    p1 = nf.plan_nfft(trj1, (Nx, Nx))
    p2 = nf.plan_nfft(trj2, (Nx, Nx))
    nf.nodes_(p2, trj1)
    b1, b2 = p1.binning(), p2.binning()
    for key in b1:
        assert np.array_equal(b1[key], b2[key])
    f = cnormal((Nx, Nx))
    fd = nf.as_colmajor(f, (Nx, Nx), torch.complex128)
    assert torch.equal(p1 * fd, p2 * fd)
    assert p1.params.m == p2.params.m and p1.Ñ == p2.Ñ


def test_dimension_mismatch():
    p = nf.plan_nfft(rand_k(2, 50), (8, 8))
    with pytest.raises(nf.DimensionMismatch):
        p * torch.zeros((8, 9), dtype=torch.complex128, device="cuda")
    with pytest.raises(nf.DimensionMismatch):
        nf.adjoint(p) * torch.zeros(49, dtype=torch.complex128)
    with pytest.raises(nf.DimensionMismatch):
        nf.mul_(torch.zeros(3, dtype=torch.complex128, device="cuda"), p,
                nf.empty_image((8, 8), torch.complex128))


def test_convolve_throws():
    """test/convolve.jl:43-54."""
    N, J = (9, 8), 101
    k = rand_k(2, J, 3, np.float32)
    p = nf.plan_nfft(k, N, m=5, sigma=2.0, precompute=nf.LINEAR)
    Nt = p.Ñ
    C32 = torch.complex64
    with pytest.raises(nf.ArgumentError):
        p.convolve_(torch.ones(Nt, dtype=C32, device="cuda").permute(1, 0).contiguous().permute(1, 0),
                    torch.zeros(J, dtype=torch.float32, device="cuda"))
    with pytest.raises(nf.ArgumentError):
        p.convolve_transpose_(torch.ones(J, dtype=C32, device="cuda"), nf.empty_image(Nt, torch.float32))
    with pytest.raises(nf.DimensionMismatch):
        p.convolve_(nf.empty_image(Nt, C32), torch.zeros(2, dtype=C32, device="cuda"))
    with pytest.raises(nf.DimensionMismatch):
        p.convolve_(nf.empty_image(N, C32), torch.zeros(J, dtype=C32, device="cuda"))
    with pytest.raises(nf.DimensionMismatch):
        p.convolve_transpose_(torch.ones(2, dtype=C32, device="cuda"), nf.empty_image(Nt, C32))
    with pytest.raises(nf.DimensionMismatch):
        p.convolve_transpose_(torch.ones(J, dtype=C32, device="cuda"), nf.empty_image(N, C32))


@pytest.mark.parametrize("pre", [nf.LINEAR, nf.FULL, nf.TENSOR, nf.POLYNOMIAL])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_convolve_isolation(pre, dtype):
    """convolve! / convolve_transpose! against the oracle, complex and real
    (test/convolve.jl:57-146)."""
    N, J = (9, 8), 101
    k = rand_k(2, J, 4, dtype)
    p = nf.plan_nfft(k, N, m=5, sigma=2.0, precompute=pre)
    op = oracle.OraclePlan(k, N, m=5, sigma=2.0, precompute=int(pre), dtype=dtype)
    tol = 1e-11 if dtype == np.float64 else 1e-5
    rng = np.random.default_rng(5)
    g = rng.random(p.Ñ) + 1j * rng.random(p.Ñ)
    cd = p.cdtype
    gd = nf.as_colmajor(g, p.Ñ, cd)
    fh = torch.empty(J, dtype=cd, device="cuda")
    assert p.convolve_(gd, fh) is fh
    assert oracle.rel_l2(fh.cpu().numpy(), op.convolve(g)) < tol
    # real -> real
    gr = nf.as_colmajor(g.real, p.Ñ, p.dtype)
    fr = torch.empty(J, dtype=p.dtype, device="cuda")
    p.convolve_(gr, fr)
    assert oracle.rel_l2(fr.cpu().numpy(), op.convolve(g.real).real) < tol
    # real -> complex
    p.convolve_(gr, fh)
    assert oracle.rel_l2(fh.cpu().numpy(), op.convolve(g.real)) < tol
    fhat = rng.random(J) + 1j * rng.random(J)
    gout = nf.empty_image(p.Ñ, cd)
    assert p.convolve_transpose_(torch.as_tensor(fhat).to(cd).cuda(), gout) is gout
    assert oracle.rel_l2(cflat(gout.cpu().numpy()), cflat(op.convolve_transpose(fhat))) < tol
    goutr = nf.empty_image(p.Ñ, p.dtype)
    p.convolve_transpose_(torch.as_tensor(fhat.real).to(p.dtype).cuda(), goutr)
    assert oracle.rel_l2(cflat(goutr.cpu().numpy()), cflat(op.convolve_transpose(fhat.real).real)) < tol


@pytest.mark.parametrize("D,N", [(2, (20, 14)), (3, (10, 12, 8))])
def test_convolve_transpose_unaligned_grid(D, N):
    """A caller's grid that starts 8 bytes past a 16-byte boundary (a view
    with a storage offset) gets the same result as an aligned one (the FP32
    tile flush adds point pairs with 16-byte atomics only on aligned grids)."""
    J = 500
    k = rand_k(D, J, 11, np.float32)
    p = nf.plan_nfft(k, N, m=4, sigma=2.0)
    rng = np.random.default_rng(2)
    fh = torch.as_tensor(rng.standard_normal(J) + 1j * rng.standard_normal(J)).to(torch.complex64).cuda()
    ng = int(np.prod(p.Ñ))
    a = torch.empty(ng, dtype=torch.complex64, device="cuda")
    buf = torch.empty(ng + 1, dtype=torch.complex64, device="cuda")
    b = buf[1:]
    assert b.data_ptr() % 16 == 8
    ga = a.reshape(p.Ñ[::-1]).permute(*reversed(range(D)))
    gb = b.reshape(p.Ñ[::-1]).permute(*reversed(range(D)))
    p.convolve_transpose_(fh, ga)
    p.convolve_transpose_(fh, gb)
    op = oracle.OraclePlan(k, N, m=4, sigma=2.0, dtype=np.float32)
    ref = cflat(op.convolve_transpose(fh.cpu().numpy()))
    assert oracle.rel_l2(cflat(ga.cpu().numpy()), ref) < 1e-5
    assert oracle.rel_l2(cflat(gb.cpu().numpy()), ref) < 1e-5


def test_deconvolve_pair():
    N = (12, 10, 6)
    k = rand_k(3, 200, 6)
    p = nf.plan_nfft(k, N, m=4, sigma=2.0)
    op = oracle.OraclePlan(k, N, m=4, sigma=2.0)
    f = cnormal(N, 7)
    g = nf.empty_image(p.Ñ, torch.complex128)
    p.deconvolve_(nf.as_colmajor(f, N, torch.complex128), g)
    assert oracle.rel_l2(cflat(g.cpu().numpy()), cflat(op.deconvolve(f))) < 1e-13
    out = nf.empty_image(N, torch.complex128)
    p.deconvolve_transpose_(g, out)
    assert oracle.rel_l2(cflat(out.cpu().numpy()), cflat(op.deconvolve_transpose(op.deconvolve(f)))) < 1e-13


def test_issue_106():
    """test/issues.jl: node 0.008333333, N = 240, LINEAR, non-blocking."""
    trj = np.full((1, 2), 0.008333333, np.float32)
    for blocking in (False, True):
        p = nf.plan_nfft(trj, (240,), precompute=nf.LINEAR, blocking=blocking)
        lam = nf.empty_image((240,), torch.complex64)
        nf.mul_(lam, nf.adjoint(p), torch.ones(2, dtype=torch.complex64, device="cuda"))
        op = oracle.OraclePlan(trj, (240,), precompute=oracle.LINEAR, dtype=np.float32)
        assert oracle.rel_l2(lam.cpu().numpy(), op.adjoint(np.ones(2, np.complex64))) < 1e-5


def test_empty_node_set():
    p = nf.plan_nfft(np.zeros((2, 0)), (16, 16))
    y = p * nf.as_colmajor(cnormal((16, 16)), (16, 16), torch.complex128)
    assert y.shape == (0,)
    x = nf.adjoint(p) * torch.zeros(0, dtype=torch.complex128)
    assert float(x.abs().max()) == 0.0


def test_timing_stats_filled():
    t = nf.TimingStats()
    p = nf.plan_nfft(rand_k(3, 5000, 8, np.float32), (32, 32, 32), timing=t)
    f = nf.as_colmajor(cnormal((32, 32, 32), dtype=np.complex64), (32, 32, 32), torch.complex64)
    y = p * f
    nf.adjoint(p) * y
    p._timing_update()
    assert t.pre > 0 and t.fft > 0 and t.conv > 0 and t.deconv > 0
    assert t.conv_adjoint > 0 and t.fft_adjoint > 0 and t.deconv_adjoint > 0


def test_config1_plain_2d_fp64():
    """Plain 2-D NFFT, ComplexF64, N = (128,128), M = 16384, KB m=4, sigma=2,
    TENSOR: GPU against the oracle (<= 1e-11) and the NDFT."""
    N, M = (128, 128), 16384
    k = rand_k(2, M, 123)
    f = cnormal(N, 124)
    fhat = cnormal(M, 125)
    p = nf.plan_nfft(k, N, m=4, sigma=2.0, window="kaiser_bessel", precompute=nf.TENSOR)
    op = oracle.OraclePlan(k, N, m=4, sigma=2.0, precompute=oracle.TENSOR)
    y = (p * nf.as_colmajor(f, N, torch.complex128)).cpu().numpy()
    x = (nf.adjoint(p) * torch.as_tensor(fhat)).cpu().numpy()
    assert oracle.rel_l2(y, op.forward(f)) < 1e-11
    assert oracle.rel_l2(cflat(x), cflat(op.adjoint(fhat))) < 1e-11
    sub = np.random.default_rng(0).choice(M, 256, replace=False)
    assert oracle.rel_l2(y[sub], oracle.ndft_forward(k, f, subset=sub)) < 1e-7
    lin = np.random.default_rng(1).choice(int(np.prod(N)), 256, replace=False)
    assert oracle.rel_l2(cflat(x)[lin], oracle.ndft_adjoint(k, N, fhat, subset=lin)) < 1e-7


# -------------------------------------------------------------- chainrules

@pytest.mark.parametrize("N", [17, 33, 67])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_chainrules(N, dtype):
    """test/chainrules.jl: gradients of sum(abs2, p*v) and sum(abs2, p'*v)
    against an explicit dense Fourier matrix, rel 1e-4."""
    rng = np.random.default_rng(N)
    M = int(rng.integers(N // 2, 2 * N))
    k = (rng.random(M) - 0.5).astype(dtype)
    cdt = torch.complex64 if dtype == np.float32 else torch.complex128
    x = np.arange(-(N // 2), -(N // 2) + N)
    A = np.exp(-2j * np.pi * k[:, None].astype(np.float64) * x[None, :])
    p = nf.plan_nfft(k, (N,), m=4, sigma=2.0)
    v = torch.tensor(rng.random(N) + 1j * rng.random(N), dtype=cdt, device="cuda", requires_grad=True)
    loss = autodiff.plan_apply(p, v).abs().pow(2).sum()
    loss.backward()
    vv = v.detach().cpu().numpy().astype(np.complex128)
    ref = 2 * A.conj().T @ (A @ vv)
    assert abs(loss.item() - np.sum(np.abs(A @ vv) ** 2)) / loss.item() < 1e-4
    assert np.linalg.norm(v.grad.cpu().numpy() - ref) / np.linalg.norm(ref) < 1e-4
    w = torch.tensor(rng.random(M) + 1j * rng.random(M), dtype=cdt, device="cuda", requires_grad=True)
    loss2 = autodiff.plan_apply_adjoint(p, w).abs().pow(2).sum()
    loss2.backward()
    ww = w.detach().cpu().numpy().astype(np.complex128)
    ref2 = 2 * A @ (A.conj().T @ ww)
    assert np.linalg.norm(w.grad.cpu().numpy() - ref2) / np.linalg.norm(ref2) < 1e-4


def spiral_nodes(N, interleaves, samples):
    """Archimedean spiral reaching |k| = 0.5: r = 0.5 t, theta = 2 pi T t + 2 pi i / interleaves."""
    turns = N / (2 * interleaves)
    t = np.arange(samples) / samples
    th = 2 * np.pi * turns * t[None, :] + 2 * np.pi * np.arange(interleaves)[:, None] / interleaves
    r = 0.5 * t[None, :]
    return np.stack([(r * np.cos(th)).ravel(), (r * np.sin(th)).ravel()])


def test_node_gradient_vs_finite_differences():
    """Loss ||A(k) f - y||^2 on a small spiral (FP64): the node gradient
    against central finite differences with step 1e-6."""
    N = (32, 32)
    k = spiral_nodes(32, 4, 128)
    M = k.shape[1]
    f = cnormal(N, 3)
    yt = cnormal(M, 4)
    p = nf.plan_nfft(k, N, m=6, sigma=2.0)
    kt = torch.tensor(k, device="cuda", requires_grad=True)
    fd = nf.as_colmajor(f, N, torch.complex128).requires_grad_(True)
    ytd = torch.tensor(yt, device="cuda")
    loss = (autodiff.nfft_nodes(kt, fd, p) - ytd).abs().pow(2).sum()
    loss.backward()
    gk = kt.grad.cpu().numpy()
    q = nf.plan_nfft(k, N, m=6, sigma=2.0)
    fdd = nf.as_colmajor(f, N, torch.complex128)

    def L(kk):
        q.nodes_(kk)
        return float(((q * fdd) - ytd).abs().pow(2).sum())

    rng = np.random.default_rng(9)
    h = 1e-6
    for j in rng.choice(M, 12, replace=False):
        for d in range(2):
            kp, km = k.copy(), k.copy()
            kp[d, j] += h
            km[d, j] -= h
            fdiff = (L(kp) - L(km)) / (2 * h)
            assert abs(fdiff - gk[d, j]) <= 1e-4 * max(1.0, abs(fdiff)), (j, d, fdiff, gk[d, j])
    # gradient in f: 2 A^H (A f - y)
    gf = fd.grad.cpu().numpy()
    r = (p * fdd - ytd)
    ref = (2 * (nf.adjoint(p) * r)).cpu().numpy()
    assert oracle.rel_l2(gf, ref) < 1e-12


def test_node_gradient_matches_ndft_derivative():
    """dk against the analytic NDFT derivative sum_n f_n (-2 pi i n_d) e^{-2 pi i k.n}
    (m = 6: window error far below the tolerance)."""
    N = (24, 20)
    k = rand_k(2, 300, 10)
    f = cnormal(N, 11)
    w = cnormal(300, 12)
    p = nf.plan_nfft(k, N, m=6, sigma=2.0)
    dk = torch.empty((300, 2), dtype=torch.float64, device="cuda")
    p.grad_nodes_(dk.t(), nf.as_colmajor(f, N, torch.complex128), torch.as_tensor(w).cuda())
    grids = np.meshgrid(*[np.arange(n) - n // 2 for n in N], indexing="ij")
    ph = np.exp(-2j * np.pi * (k[0][:, None] * grids[0].ravel()[None] + k[1][:, None] * grids[1].ravel()[None]))
    fv = f.ravel()
    ref = np.zeros((2, 300))
    for d in range(2):
        dy = (ph * (-2j * np.pi * grids[d].ravel()[None])) @ fv
        ref[d] = np.real(np.conj(w) * dy)
    assert oracle.rel_l2(dk.t().cpu().numpy(), ref) < 1e-6


# ----------------------------------------------------------------- NFFTTools

@pytest.mark.parametrize("pre", [nf.LINEAR, nf.FULL, nf.TENSOR, nf.POLYNOMIAL])
def test_sdc_equispaced(pre):
    """test/gpu.jl:52-65 and test/samplingDensity.jl:10-27: weights 1/|N|."""
    N = (9, 8)
    xs = (np.arange(N[0]) / N[0] - 0.5).astype(np.float32)
    ys = (np.arange(N[1]) / N[1] - 0.5).astype(np.float32)
    nodes = np.array([[x, y] for y in ys for x in xs], dtype=np.float32).T
    p = nf.plan_nfft(nodes, N, m=5, sigma=2.0, precompute=pre)
    w = tools.sdc(p, iters=10)
    assert w.dtype == torch.float32
    wn = w.cpu().numpy()
    assert np.all(wn > 0)
    np.testing.assert_allclose(wn, 1 / 72, rtol=np.sqrt(np.finfo(np.float32).eps))
    op = oracle.OraclePlan(nodes, N, m=5, sigma=2.0, precompute=int(pre), dtype=np.float32)
    np.testing.assert_allclose(wn, oracle.sdc(op, iters=10), rtol=1e-5)


def test_config5_spiral_gradients_full_size():
    """Differentiated 2-D spiral NFFT: N = (256, 256), 32 interleaves x 2048
    samples of an Archimedean spiral reaching |k| = 0.5, loss ||A(k) f - y||^2
    in FP32 with gradients in f and k; the k-gradient is checked against FP64
    central finite differences (step 1e-6) of the same loss on an FP64 plan,
    and the f-gradient against 2 A^H (A f - y)."""
    N = (256, 256)
    k64 = spiral_nodes(256, 32, 2048)
    M = k64.shape[1]
    f = cnormal(N, 21)
    yt = cnormal(M, 22)
    k32 = k64.astype(np.float32)
    p32 = nf.plan_nfft(k32, N, m=4, sigma=2.0)
    kt = torch.tensor(k32, device="cuda", requires_grad=True)
    fd = nf.as_colmajor(f, N, torch.complex64).requires_grad_(True)
    ytd = torch.tensor(yt.astype(np.complex64), device="cuda")
    loss = (autodiff.nfft_nodes(kt, fd, p32) - ytd).abs().pow(2).sum()
    loss.backward()
    gk = kt.grad.cpu().numpy().astype(np.float64)
    # FP64 reference loss for finite differences (nodes as the FP32 plan saw them)
    kref = k32.astype(np.float64)
    q = nf.plan_nfft(kref, N, m=4, sigma=2.0)
    f64 = nf.as_colmajor(f.astype(np.complex64).astype(np.complex128), N, torch.complex128)
    y64 = torch.tensor(yt.astype(np.complex64).astype(np.complex128), device="cuda")

    def L(kk):
        q.nodes_(kk)
        return float(((q * f64) - y64).abs().pow(2).sum())

    rng = np.random.default_rng(5)
    h = 1e-6
    num, ana = [], []
    for j in rng.choice(M, 16, replace=False):
        for d in range(2):
            kp, km = kref.copy(), kref.copy()
            kp[d, j] += h
            km[d, j] -= h
            num.append((L(kp) - L(km)) / (2 * h))
            ana.append(gk[d, j])
    num, ana = np.array(num), np.array(ana)
    assert np.linalg.norm(num - ana) / np.linalg.norm(num) < 1e-3
    # gradient in f
    q.nodes_(kref)
    r = q * f64 - y64
    ref = (2 * (nf.adjoint(q) * r)).cpu().numpy()
    assert oracle.rel_l2(fd.grad.cpu().numpy().astype(np.complex128), ref) < 1e-4


# ------------------------------------------------------------ sortNodes

def lex_reference(k):
    """Column order of sortslices(k, dims=2) by a plain stable sort on
    per-column keys (value, then -0.0 before 0.0, per coordinate)."""
    M = k.shape[1]
    return sorted(range(M), key=lambda j: tuple(v for d in range(k.shape[0])
                                                 for v in (k[d, j], 0 if np.signbit(k[d, j]) else 1)))


@pytest.mark.parametrize("D", [1, 2, 3])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("on_device", [0, 1])
def test_sort_nodes_matches_sortslices(D, dtype, on_device):
    """nfft_sort_nodes (host and device arrays) equals sortslices(k, dims=2)
    bit for bit, ties and signed zeros included."""
    import ctypes
    rng = np.random.default_rng(D)
    M = 3000
    k = (rng.integers(-6, 6, size=(D, M)) / 12.0).astype(dtype)  # many ties per coordinate
    k[:, :40] = 0.0
    k[0, 5:25] = -0.0
    ref = k[:, lex_reference(k)]
    k2 = k.copy()
    assert np.array_equal(k2[:, oracle.sort_nodes_lex(k2.copy())], ref)
    oracle.sort_nodes_lex(k2)
    assert np.array_equal(k2, ref) and np.array_equal(np.signbit(k2), np.signbit(ref))
    lib = nf.load()
    prec = 32 if dtype == np.float32 else 64
    if on_device:
        kt = torch.as_tensor(k.T.copy()).cuda()  # column-major D x M
        rc = lib.nfft_sort_nodes(prec, D, M, ctypes.c_void_p(kt.data_ptr()), 1, None)
        out = kt.cpu().numpy().T
    else:
        kc = np.ascontiguousarray(k.T)
        rc = lib.nfft_sort_nodes(prec, D, M, ctypes.c_void_p(kc.ctypes.data), 1 if on_device else 0, None)
        out = kc.T
    assert rc == 0
    assert np.array_equal(out, ref) and np.array_equal(np.signbit(out), np.signbit(ref))


@pytest.mark.parametrize("as_tensor", [False, True])
def test_sort_nodes_plan_matches_oracle(as_tensor):
    """plan_nfft(k, N; sortNodes=true) sorts the caller's k in place
    (src/precomputation.jl:52-54) and every output follows that order: fHat
    equals the oracle's sortNodes plan at 1e-11 (FP64); nodes! sorts too
    (src/implementation.jl:112-114)."""
    N = (16, 12, 10)
    k0 = rand_k(3, 2500, seed=11)
    k0[:, 100:140] = k0[:, 0:1]  # duplicate nodes
    f = cnormal(N, 2)
    fh = cnormal(2500, 3)
    ref_k = k0[:, lex_reference(k0)]
    kc = k0.copy()
    op = oracle.OraclePlan(kc, N, m=4, sigma=2.0, precompute=oracle.TENSOR, sortNodes=True)
    assert np.array_equal(kc, ref_k)
    kin = torch.as_tensor(k0.copy()) if as_tensor else k0.copy()
    p = nf.plan_nfft(kin, N, m=4, sigma=2.0, precompute=nf.TENSOR, sortNodes=True)
    kin_np = kin.numpy() if as_tensor else kin
    assert np.array_equal(kin_np, ref_k)
    y = (p * nf.as_colmajor(f, N, torch.complex128)).cpu().numpy()
    assert oracle.rel_l2(y, op.forward(f)) < 1e-11
    x = (nf.adjoint(p) * torch.as_tensor(fh)).cpu().numpy()
    assert oracle.rel_l2(x, op.adjoint(fh)) < 1e-11
    # the outputs follow the sorted order: node i of the plan is column i of ref_k
    y_unsorted = (nf.plan_nfft(k0.copy(), N, m=4, sigma=2.0, precompute=nf.TENSOR) *
                  nf.as_colmajor(f, N, torch.complex128)).cpu().numpy()
    assert oracle.rel_l2(y, y_unsorted[lex_reference(k0)]) < 1e-13
    # nodes!(p, k2) sorts k2 in place as well
    k2 = rand_k(3, 2500, seed=12)
    ref2 = k2[:, lex_reference(k2)]
    p.nodes_(k2)
    assert np.array_equal(k2, ref2)
    # invalid nodes: rejected before anything is reordered
    bad = rand_k(3, 50, seed=13)
    bad[1, 7] = 0.75
    keep = bad.copy()
    with pytest.raises(nf.ArgumentError):
        nf.plan_nfft(bad, N, m=4, sigma=2.0, sortNodes=True)
    assert np.array_equal(bad, keep)
