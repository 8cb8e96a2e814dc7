"""Direct transforms (src/direct.jl: NDFT, NDCT, NDST, NNDFT) and the NFCT /
NFST plans on the GPU.  The direct kernels sum in FP64 and must equal the
FP64 oracle to 1e-12 (FP64 data) / 1e-6 (FP32 outputs).  The fast NFCT /
NFST follow the reference's wrapper tests (test/wrappers.jl:100-205: sizes
(256,), (30,32), (10,12,14); J = prod(N) nodes in [0, 1/2); m = 5, sigma = 2;
relative error < 1e-7 against the direct transform, forward and transpose),
plus FP32 at 1e-5."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import nfftgb300 as nf  # noqa: E402
from oracle import oracle  # noqa: E402


def host(t):
    return t.cpu().numpy()


def rel(a, b):
    return oracle.rel_l2(a, b)


@pytest.mark.parametrize("N", [(40,), (12, 10), (6, 8, 5), (4, 5, 3, 4), (33,)])
@pytest.mark.parametrize("prec", [64, 32])
def test_ndft_direct(N, prec):
    rng = np.random.default_rng(len(N))
    dt = np.float64 if prec == 64 else np.float32
    D, J = len(N), 70
    k = (rng.random((D, J)) - 0.5).astype(dt)
    f = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    v = rng.standard_normal(J) + 1j * rng.standard_normal(J)
    p = nf.NDFTPlan(k, N)
    tol = 1e-12 if prec == 64 else 1e-6
    ref = oracle.ndft_forward_sep(k.astype(np.float64), f.astype(np.complex64 if prec == 32 else np.complex128))
    assert rel(host(p * f), ref) < tol
    refa = oracle.ndft_adjoint_sep(k.astype(np.float64), N, v.astype(np.complex64 if prec == 32 else np.complex128))
    assert rel(host(p.adjoint() * v), refa) < tol
    if D <= 3 and prec == 64:
        assert rel(host(nf.ndft(k, f)), oracle.ndft_forward(k, f)) < 1e-12


@pytest.mark.parametrize("N", [(256,), (30, 32), (10, 12, 14), (6, 6, 6, 6)])
def test_ndct_ndst_direct(N):
    rng = np.random.default_rng(sum(N))
    D = len(N)
    J = min(int(np.prod(N)), 600)
    k = 0.5 * rng.random((D, J))
    f = rng.standard_normal(N)
    v = rng.standard_normal(J)
    pc = nf.NDCTPlan(k, N)
    assert rel(host(pc * f), oracle.ndct_forward(k, f)) < 1e-12
    assert rel(host(pc.transpose() * v), oracle.ndct_transpose(k, N, v)) < 1e-12
    # complex data through the same plan
    fc = f + 1j * rng.standard_normal(N)
    assert rel(host(pc * fc), oracle.ndct_forward(k, fc)) < 1e-12
    Np = tuple(n + 1 for n in N)
    ps = nf.NDSTPlan(k, Np)
    assert ps.size_in() == N
    assert rel(host(ps * f), oracle.ndst_forward(k, f)) < 1e-12
    assert rel(host(ps.transpose() * v), oracle.ndst_transpose(k, Np, v)) < 1e-12
    # FP32 nodes and data: FP64 sums stored in FP32
    p32 = nf.NDCTPlan(k.astype(np.float32), N)
    assert rel(host(p32 * f.astype(np.float32)), oracle.ndct_forward(k.astype(np.float32), f.astype(np.float32))) < 1e-6


@pytest.mark.parametrize("D", [1, 2, 3])
def test_nndft_direct(D):
    """test/wrappers.jl:70-96 shapes: J = N = 40, y in [-5, 5)^D."""
    rng = np.random.default_rng(D)
    J, Ny = 40, 40
    k = rng.random((D, J)) - 0.5
    y = (rng.random((D, Ny)) - 0.5) * 10
    p = nf.NNDFTPlan(k, y)
    fh = rng.standard_normal(J) + 1j * rng.standard_normal(J)
    f = host(p.adjoint() * fh)
    assert rel(f, oracle.nndft_adjoint(k, y, fh)) < 1e-12
    assert rel(host(p * f), oracle.nndft_forward(k, y, f)) < 1e-12


def test_direct_split_sums_many_inputs():
    """Few outputs, many inputs: the input range is split over CTAs and the
    FP64 partials added in a second pass (deterministic: two runs agree)."""
    rng = np.random.default_rng(5)
    N = (128, 96)
    k = rng.random((2, 3)) - 0.5
    f = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    p = nf.NDFTPlan(k, N)
    a, b = host(p * f), host(p * f)
    assert np.array_equal(a, b)
    assert rel(a, oracle.ndft_forward(k, f)) < 1e-12


@pytest.mark.parametrize("N", [(256,), (30, 32), (10, 12, 14)])
def test_nfct_vs_ndct(N):
    rng = np.random.default_rng(len(N) + 10)
    D = len(N)
    J = int(np.prod(N))
    k = 0.5 * rng.random((D, J))
    p = nf.plan_nfct(k, N, m=5, sigma=2.0)
    pd = nf.NDCTPlan(k, N)
    fHat = rng.random(J)
    f = host(p.transpose() * fHat)
    fd = host(pd.transpose() * fHat)
    assert rel(f, fd) < 1e-7
    g = host(p * f)
    gd = host(pd * f)
    assert rel(g, gd) < 1e-7
    assert rel(fd, oracle.ndct_transpose(k, N, fHat)) < 1e-12


@pytest.mark.parametrize("N", [(256,), (8, 8), (10, 12, 14)])
def test_nfst_vs_ndst(N):
    rng = np.random.default_rng(len(N) + 20)
    D = len(N)
    J = int(np.prod(N))
    k = 0.5 * rng.random((D, J))
    Np = tuple(n + 1 for n in N)
    p = nf.plan_nfst(k, Np, m=5, sigma=2.0)
    pd = nf.NDSTPlan(k, Np)
    assert p.size_in() == N
    fHat = rng.random(J)
    f = host(p.transpose() * fHat)
    fd = host(pd.transpose() * fHat)
    assert rel(f, fd) < 1e-7
    g = host(p * f)
    gd = host(pd * f)
    assert rel(g, gd) < 1e-7


@pytest.mark.parametrize("kind", ["nfct", "nfst"])
def test_trig_fp32_and_helpers(kind):
    rng = np.random.default_rng(3)
    N = (24, 20)
    k = (0.5 * rng.random((2, 500))).astype(np.float32)
    if kind == "nfct":
        f = rng.standard_normal(N).astype(np.float32)
        g = host(nf.nfct(k, f, m=4, sigma=2.0))
        assert rel(g, oracle.ndct_forward(k, f)) < 1e-5
        v = rng.standard_normal(500).astype(np.float32)
        assert rel(host(nf.nfct_transpose(k, N, v, m=4, sigma=2.0)), oracle.ndct_transpose(k, N, v)) < 1e-5
    else:
        f = rng.standard_normal(N).astype(np.float32)
        g = host(nf.nfst(k, f, m=4, sigma=2.0))
        assert rel(g, oracle.ndst_forward(k, f)) < 1e-5
        v = rng.standard_normal(500).astype(np.float32)
        Np = (25, 21)
        assert rel(host(nf.nfst_transpose(k, Np, v, m=4, sigma=2.0)), oracle.ndst_transpose(k, Np, v)) < 1e-5


def test_trig_nodes_and_errors():
    rng = np.random.default_rng(4)
    N = (16, 16)
    k1 = 0.5 * rng.random((2, 100))
    k2 = 0.5 * rng.random((2, 100))
    p = nf.plan_nfct(k1, N, m=5, sigma=2.0)
    p.nodes_(k2)
    f = rng.standard_normal(N)
    assert rel(host(p * f), oracle.ndct_forward(k2, f)) < 1e-7
    with pytest.raises(nf.DimensionMismatch):
        p * rng.standard_normal((16, 15))
    with pytest.raises(nf.ArgumentError):
        nf.plan_nfct(k1, (16, 16, 16))
    with pytest.raises(nf.ArgumentError):
        nf.NDFTPlan(k1, (8,))
    with pytest.raises(nf.ArgumentError):
        nf.plan_nfst(k1 + 1.0, N)                # nodes beyond 1/2


def test_empty_node_sets():
    """M = 0: forward outputs are empty, transposes / adjoints are zero images."""
    N = (8, 6)
    k0 = np.zeros((2, 0))
    p = nf.NDFTPlan(k0, N)
    assert host(p.adjoint() * np.zeros(0, complex)).shape == N
    assert np.all(host(p.adjoint() * np.zeros(0, complex)) == 0)
    assert host(p * np.ones(N, complex)).shape == (0,)
    c = nf.plan_nfct(k0, N)
    assert np.all(host(c.transpose() * np.zeros(0)) == 0)
    assert host(c * np.ones(N)).shape == (0,)
    s = nf.plan_nfst(k0, (8, 7))
    assert np.all(host(s.transpose() * np.zeros(0)) == 0)


def test_ndst_with_single_point_dimension():
    """N_d = 2 gives a single sine term n_d = 1 in that dimension."""
    rng = np.random.default_rng(8)
    k = 0.5 * rng.random((2, 50))
    N = (2, 9)
    f = rng.standard_normal((1, 8))
    p = nf.NDSTPlan(k, N)
    assert p.size_in() == (1, 8)
    assert rel(host(p * f), oracle.ndst_forward(k, f)) < 1e-12
    q = nf.plan_nfst(k, N, m=5, sigma=2.0)
    assert rel(host(q * f), oracle.ndst_forward(k, f)) < 1e-7


@pytest.mark.parametrize("D", [1, 2, 3])
@pytest.mark.parametrize("m,tol", [(4, 1e-6), (6, 1e-9)])
def test_nnfft_vs_nndft(D, m, tol):
    """Fast NNFFT against the NNDFT (test/wrappers.jl:70-96 shapes: J = N = 40,
    y in [-5, 5)^D); FP64, forward and adjoint."""
    rng = np.random.default_rng(10 * D + m)
    J, Ny = 40, 40
    k = rng.random((D, J)) - 0.5
    y = (rng.random((D, Ny)) - 0.5) * 10
    p = nf.plan_nnfft(k, y, m=m, sigma=2.0)
    c = rng.standard_normal(Ny) + 1j * rng.standard_normal(Ny)
    fh = rng.standard_normal(J) + 1j * rng.standard_normal(J)
    assert rel(host(p * c), oracle.nndft_forward(k, y, c)) < tol
    assert rel(host(p.adjoint() * fh), oracle.nndft_adjoint(k, y, fh)) < tol
    # larger point clouds and FP32
    k2 = (rng.random((D, 3000)) - 0.5).astype(np.float32)
    y2 = ((rng.random((D, 2000)) - 0.5) * 40).astype(np.float32)
    q = nf.plan_nnfft(k2, y2, m=4, sigma=2.0)
    c2 = (rng.standard_normal(2000) + 1j * rng.standard_normal(2000)).astype(np.complex64)
    ref = nf.NNDFTPlan(k2, y2) * c2
    assert rel(host(q * c2), host(ref)) < 1e-5
