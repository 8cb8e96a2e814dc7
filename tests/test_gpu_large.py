"""Full-size GPU checks on the benchmark configurations, through
size-independent properties and FP64 NDFT subsets:

* 3-D radial koosh-ball, N = 256^3, 8192 x 512 nodes, FP32, m = 4:
  rel l2 error <= 1e-5 against the FP64 NDFT on node / frequency subsets,
  adjointness <A f, y> = <f, A^H y>, linearity, and FP32 vs the FP64 tiled
  plan and the FP64 plain path on the same nodes.
* 1-D large, N = 2^22, M = 2^24, m = 5, FP32: error vs the FP64 NDFT on a
  node subset and an output subset.
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import nfftgb300 as nf  # noqa: E402
from oracle import oracle  # noqa: E402
import bench  # noqa: E402


def cnormal(shape, seed, dtype=np.complex64):
    rng = np.random.default_rng(seed)
    return ((rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / math.sqrt(2)).astype(dtype)


@pytest.fixture(scope="module")
def radial():
    k = bench.radial_nodes(np.float32)
    f = cnormal(bench.N3, 123)
    fhat = cnormal(bench.M_NODES, 124)
    p = nf.plan_nfft(k, bench.N3, m=4, sigma=2.0)
    return k, f, fhat, p


def test_radial_accuracy_vs_ndft(radial):
    k, f, fhat, p = radial
    fd = nf.as_colmajor(f, bench.N3, torch.complex64)
    y = (p * fd).cpu().numpy()
    x = (nf.adjoint(p) * torch.as_tensor(fhat)).cpu().numpy()
    ef, ea = bench.rel_err_subset(k.astype(np.float64), f.astype(np.complex128), fhat.astype(np.complex128), y, x,
                                  n_fwd=48, n_adj=24)
    assert ef < 1e-5 and ea < 1e-5, (ef, ea)


def test_radial_adjointness_and_linearity(radial):
    k, f, fhat, p = radial
    fd = nf.as_colmajor(f, bench.N3, torch.complex64)
    y = p * fd
    x = nf.adjoint(p) * torch.as_tensor(fhat)
    fh = torch.as_tensor(fhat).cuda()
    lhs = torch.vdot(fh.to(torch.complex128), y.to(torch.complex128))
    rhs = torch.vdot(x.to(torch.complex128).reshape(-1), fd.to(torch.complex128).reshape(-1))
    assert abs(complex(lhs - rhs)) / abs(complex(lhs)) < 1e-5
    y2 = p * (2 * fd)
    assert float((y2 - 2 * y).abs().max() / y.abs().max()) < 1e-6


def test_radial_fp32_vs_fp64_paths(radial):
    k, f, fhat, p = radial
    fd = nf.as_colmajor(f, bench.N3, torch.complex64)
    y32 = (p * fd).to(torch.complex128)
    k64 = k.astype(np.float64)
    p64 = nf.plan_nfft(k64, bench.N3, m=4, sigma=2.0)
    f64 = fd.to(torch.complex128)
    y64 = p64 * f64
    assert float((y32 - y64).norm() / y64.norm()) < 1e-5
    del p64
    pp = nf.plan_nfft(k64, bench.N3, m=4, sigma=2.0, blocking=False)
    yp = pp * f64
    assert float((yp - y64).norm() / y64.norm()) < 1e-11
    xp = nf.adjoint(pp) * torch.as_tensor(fhat.astype(np.complex128))
    x32 = nf.adjoint(p) * torch.as_tensor(fhat)
    assert float((x32.to(torch.complex128) - xp).norm() / xp.norm()) < 1e-5


def test_1d_large_accuracy():
    N = (2 ** 22,)
    M = 2 ** 24
    rng = np.random.default_rng(3)
    k = (rng.random((1, M)) - 0.5).astype(np.float32)
    f = cnormal(N, 5)
    fhat = cnormal(M, 6)
    p = nf.plan_nfft(k, N, m=5, sigma=2.0)
    y = (p * nf.as_colmajor(f, N, torch.complex64)).cpu().numpy()
    sub = rng.choice(M, 32, replace=False)
    ref = oracle.ndft_forward(k.astype(np.float64), f.astype(np.complex128), subset=sub)
    assert oracle.rel_l2(y[sub], ref) < 1e-5
    x = (nf.adjoint(p) * torch.as_tensor(fhat)).cpu().numpy()
    lin = rng.choice(N[0], 8, replace=False)
    refx = oracle.ndft_adjoint(k.astype(np.float64), N, fhat.astype(np.complex128), subset=lin)
    assert oracle.rel_l2(x[lin], refx) < 1e-5
