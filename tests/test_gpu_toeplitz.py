"""Toeplitz tools on the GPU (NFFTTools/src/Toeplitz.jl) against the oracle:
the reference's own checks of test/testToeplitz.jl (kernel ≈ explicit kernel,
rtol 1e-6 Float64 / 1e-5 Float32; convolveToeplitzKernel! ≈
nfft_adjoint(nfft(x)), rtol 1e-5) plus parity of every path with the FP64
oracle: the kernel from the plan (same window tensor) to 1e-11 in FP64, the
explicit kernel to 1e-12, the convolution (fused pruned-FFT path and cuFFT
path, D = 1..3) to 1e-12 FP64 / 1e-5 FP32."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import nfftgb300 as nf  # noqa: E402
from nfftgb300 import tools  # noqa: E402
from oracle import oracle  # noqa: E402


def isapprox(a, b, rtol):
    """Julia's a ≈ b (rtol): norm(a - b) <= rtol * max(norm(a), norm(b))."""
    a = np.asarray(a, np.complex128).ravel()
    b = np.asarray(b, np.complex128).ravel()
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


def host(t):
    return t.cpu().numpy()


@pytest.mark.parametrize("Nx", [32, 33, 64])
def test_kernel_vs_explicit_fp64(Nx):
    rng = np.random.default_rng(Nx)
    tr = rng.random((2, 1000)) - 0.5
    ka = tools.calculate_toeplitz_kernel((Nx, Nx), tr, m=4, sigma=2.0, precompute=nf.TENSOR)
    assert tuple(ka.shape) == (2 * Nx, 2 * Nx) and ka.dtype == torch.complex128
    kx_ref = oracle.toeplitz_kernel_explicit((Nx, Nx), tr)
    assert isapprox(host(ka), kx_ref, 1e-6)                   # test/testToeplitz.jl:17
    ka_ref = oracle.toeplitz_kernel((Nx, Nx), tr, m=4, sigma=2.0)
    assert oracle.rel_l2(host(ka), ka_ref) < 1e-11            # same algorithm, FP64
    kx = tools.calculate_toeplitz_kernel_explicit((Nx, Nx), tr)
    assert oracle.rel_l2(host(kx), kx_ref) < 1e-12
    # the in-place form on a plan that held other nodes (test/testToeplitz.jl:20-31)
    p = nf.plan_nfft(rng.random((2, 1000)) - 0.5, (2 * Nx, 2 * Nx), m=4, sigma=2.0, precompute=nf.TENSOR)
    lam = nf.empty_image((2 * Nx, 2 * Nx), torch.complex128)
    tools.calculate_toeplitz_kernel_(lam, p, tr)
    assert oracle.rel_l2(host(lam), ka_ref) < 1e-11
    # with the plan's default accuracy parameters, as the reference's test does
    q = nf.plan_nfft(rng.random((2, 1000)) - 0.5, (2 * Nx, 2 * Nx))
    tools.calculate_toeplitz_kernel_(lam, q, tr)
    assert isapprox(host(lam), kx_ref, 1e-6)


def test_kernel_fp32_and_gram():
    """test/testToeplitz.jl:34-52."""
    rng = np.random.default_rng(7)
    Nx = 32
    tr = (rng.random((2, 10000)) - 0.5).astype(np.float32)
    ka = tools.calculate_toeplitz_kernel((Nx, Nx), tr, m=4, sigma=2.0)
    assert ka.dtype == torch.complex64
    assert isapprox(host(ka), oracle.toeplitz_kernel_explicit((Nx, Nx), tr), 1e-5)
    x = (rng.standard_normal((Nx, Nx)) + 1j * rng.standard_normal((Nx, Nx))).astype(np.complex64)
    p = nf.plan_nfft(tr, (Nx, Nx))
    xn = host(nf.adjoint(p) * (p * x))
    y = nf.as_colmajor(x, (Nx, Nx), torch.complex64)
    tools.convolve_toeplitz_kernel_(y, ka)
    assert isapprox(host(y), xn, 1e-5)


def test_kernel_rect_and_3d():
    """test/testToeplitz.jl:58-82 (Float32, rtol 1e-5)."""
    rng = np.random.default_rng(9)
    tr = (rng.random((2, 1000)) - 0.5).astype(np.float32)
    ka = tools.calculate_toeplitz_kernel((32, 33), tr)
    assert tuple(ka.shape) == (64, 66)
    assert isapprox(host(ka), oracle.toeplitz_kernel_explicit((32, 33), tr), 1e-5)
    tr3 = (rng.random((3, 1000)) - 0.5).astype(np.float32)
    ka3 = tools.calculate_toeplitz_kernel((32, 32, 32), tr3)
    kx3_ref = oracle.toeplitz_kernel_explicit((32, 32, 32), tr3)
    assert isapprox(host(ka3), kx3_ref, 1e-5)
    kx3 = tools.calculate_toeplitz_kernel_explicit((32, 32, 32), tr3)
    assert oracle.rel_l2(host(kx3), kx3_ref) < 1e-6          # FP32 storage of FP64 sums


CONV_CASES = [
    ((100,), False),
    ((32, 32), True),
    ((64, 48), False),
    ((256, 128), True),
    ((512, 32), True),      # x lines of 1024
    ((32, 512), True),      # fused last-axis lines of 1024
    ((32, 32, 32), True),
    ((64, 32, 128), True),
    ((32, 24, 16), False),
]


@pytest.mark.parametrize("shape,fused", CONV_CASES)
@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_convolve_parity(shape, fused, dtype):
    rng = np.random.default_rng(len(shape) * 1000 + shape[0])
    shape_os = tuple(2 * n for n in shape)
    lam = (rng.standard_normal(shape_os) + 1j * rng.standard_normal(shape_os)).astype(dtype)
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dtype)
    ref = oracle.convolve_toeplitz(x, lam)
    tol = 1e-12 if dtype == np.complex128 else 1e-5
    ct = torch.complex128 if dtype == np.complex128 else torch.complex64
    lam_d = nf.as_colmajor(lam, shape_os, ct)
    outs = {}
    for mode in ("auto", "cufft"):
        tz = tools.Toeplitz(shape, ct, fft=mode)
        assert tz.fused == (fused and mode == "auto")
        y = nf.as_colmajor(x, shape, ct)
        tz.convolve_(y, lam_d)
        outs[mode] = host(y)
        assert oracle.rel_l2(outs[mode], ref) < tol, mode
        # a second application reuses the workspace (no stale grid state)
        y2 = nf.as_colmajor(x, shape, ct)
        tz.convolve_(y2, lam_d)
        assert np.array_equal(host(y2), outs[mode])
    assert oracle.rel_l2(outs["auto"], outs["cufft"]) < tol


def test_convolve_noncolmajor_input_in_place():
    rng = np.random.default_rng(3)
    shape = (32, 64)
    lam = rng.standard_normal((64, 128)) + 1j * rng.standard_normal((64, 128))
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    y = torch.from_numpy(x).cuda()                              # row-major
    tools.convolve_toeplitz_kernel_(y, nf.as_colmajor(lam, (64, 128), torch.complex128))
    assert oracle.rel_l2(host(y), oracle.convolve_toeplitz(x, lam)) < 1e-12


def test_toeplitz_errors():
    rng = np.random.default_rng(0)
    tz = tools.Toeplitz((32, 32), torch.complex64)
    lam = tz.empty_kernel()
    with pytest.raises(nf.DimensionMismatch):
        tz.convolve_(nf.empty_image((32, 31), torch.complex64), lam)
    with pytest.raises(nf.DimensionMismatch):
        tz.convolve_(nf.empty_image((32, 32), torch.complex64), nf.empty_image((64, 62), torch.complex64))
    with pytest.raises(nf.ArgumentError):
        tz.convolve_(nf.empty_image((32, 32), torch.complex64), nf.empty_image((64, 64), torch.complex128))
    p = nf.plan_nfft((rng.random((2, 50)) - 0.5).astype(np.float32), (32, 32))
    with pytest.raises(nf.DimensionMismatch):
        tz.kernel_(lam, p)                                      # plan must have size 2N
    p64 = nf.plan_nfft(rng.random((2, 50)) - 0.5, (64, 64))
    with pytest.raises(nf.ArgumentError):
        tz.kernel_(lam, p64)                                    # precision mismatch
    with pytest.raises(nf.ArgumentError):
        tools.Toeplitz((32, 32), torch.complex64, fft="fftw")
    with pytest.raises(nf.ArgumentError):
        tz.kernel_explicit_(lam, rng.random((3, 10)) - 0.5)     # 3-D nodes for a 2-D image


def test_gram_large_3d_fused_vs_cufft():
    """Bench-size case (256^3 image, 512^3 kernel, FP32): the fused path equals
    the cuFFT path, and the operator with a Gram kernel is Hermitian,
    <x, T y> = <T x, y>, both size-independent properties."""
    rng = np.random.default_rng(11)
    shape = (256, 256, 256)
    M = 200_000
    tr = (rng.random((3, M)) - 0.5).astype(np.float32)
    tz = tools.Toeplitz(shape, torch.complex64)
    assert tz.fused
    lam = tools.calculate_toeplitz_kernel(shape, tr, toeplitz=tz)
    g = torch.Generator(device="cuda").manual_seed(5)
    x = nf.empty_image(shape, torch.complex64)
    x.copy_(torch.randn(shape, dtype=torch.complex64, device="cuda", generator=g))
    yv = nf.empty_image(shape, torch.complex64)
    yv.copy_(torch.randn(shape, dtype=torch.complex64, device="cuda", generator=g))
    tx = x.clone()
    tz.convolve_(tx, lam)
    ty = yv.clone()
    tz.convolve_(ty, lam)
    ref = tools.Toeplitz(shape, torch.complex64, fft="cufft")
    tx2 = x.clone()
    ref.convolve_(tx2, lam)
    d = (tx - tx2).abs().double().norm() / tx2.abs().double().norm()
    assert float(d) < 1e-5
    lhs = torch.vdot(x.flatten().to(torch.complex128), ty.flatten().to(torch.complex128))
    rhs = torch.vdot(tx.flatten().to(torch.complex128), yv.flatten().to(torch.complex128))
    assert abs(complex(lhs - rhs)) < 1e-4 * abs(complex(lhs))


def test_toeplitz_kernel_of_empty_node_set_is_zero():
    tz = tools.Toeplitz((32, 32), torch.complex64)
    lam = tools.calculate_toeplitz_kernel((32, 32), np.zeros((2, 0), np.float32), toeplitz=tz)
    assert float(lam.abs().max()) == 0.0
    y = nf.as_colmajor(np.ones((32, 32), np.complex64), (32, 32), torch.complex64)
    tz.convolve_(y, lam)
    assert float(y.abs().max()) == 0.0
