"""Full-size GPU checks on the benchmark configurations, through
size-independent properties and FP64 NDFT subsets:

* 3-D radial koosh-ball, N = 256^3, 8192 x 512 nodes, FP32, m = 4:
  rel l2 error <= 1e-5 against the FP64 NDFT (the oracle's) on 4096 random
  nodes (forward) and 4096 random output frequencies (adjoint),
  adjointness <A f, y> = <f, A^H y>, linearity, and FP32 vs the FP64 tiled
  plan and the FP64 plain path on the same nodes.
* 1-D large, N = 2^22, M = 2^24, m = 5, FP32, compensated spreading (and the
  plain FP32 spreader): error vs the FP64 NDFT on 4096 random nodes and 4096
  random output frequencies.
* The library's exact GPU sums (NDFT / NNDFT plans), which bench.py uses to
  report these errors, agree with the oracle's NDFT on the same subsets.
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import nfftgb300 as nf  # noqa: E402
from oracle import oracle  # noqa: E402
import bench  # noqa: E402


N_FWD = 4096  # random nodes of the forward error subset
N_ADJ = 4096  # random output frequencies of the adjoint error subset


def subsets(M, n_img, seed):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(M, N_FWD, replace=False)), np.sort(rng.choice(n_img, N_ADJ, replace=False))


def frequencies(N, lin):
    """Integer frequencies n - N div 2 (D x len(lin)) of column-major linear indices."""
    idx = np.unravel_index(np.asarray(lin), N, order="F")
    return np.stack([i - n // 2 for i, n in zip(idx, N)]).astype(np.float64)


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


@pytest.fixture(scope="module")
def radial_ref(radial):
    """FP64 NDFT (oracle, OpenMP) of the radial inputs on 4096 random nodes and
    4096 random output frequencies."""
    k, f, fhat, p = radial
    k64 = k.astype(np.float64)
    sub, lin = subsets(k.shape[1], int(np.prod(bench.N3)), 7)
    ref_f = oracle.ndft_forward(k64, f.astype(np.complex128), subset=sub)
    ref_a = oracle.ndft_adjoint(k64, bench.N3, fhat.astype(np.complex128), subset=lin)
    return sub, lin, ref_f, ref_a


def test_radial_accuracy_vs_ndft(radial, radial_ref):
    k, f, fhat, p = radial
    sub, lin, ref_f, ref_a = radial_ref
    fd = nf.as_colmajor(f, bench.N3, torch.complex64)
    y = (p * fd).cpu().numpy()
    x = (nf.adjoint(p) * torch.as_tensor(fhat)).cpu().numpy()
    ef = oracle.rel_l2(y[sub], ref_f)
    ea = oracle.rel_l2(x.ravel(order="F")[lin], ref_a)
    assert ef <= 1e-5 and ea <= 1e-5, (ef, ea)


def test_bench_checker_matches_oracle_ndft(radial, radial_ref):
    """bench.py reports the errors against the library's exact FP64 GPU sums on
    the same 4096 / 4096 subsets; they must equal the oracle's NDFT."""
    k, f, fhat, p = radial
    sub, lin, ref_f, ref_a = radial_ref
    k64 = k.astype(np.float64)
    rf, ra = bench.ndft_reference_subsets(k64, f.astype(np.complex128), fhat.astype(np.complex128), sub, lin)
    assert oracle.rel_l2(rf, ref_f) < 1e-11
    assert oracle.rel_l2(ra, ref_a) < 1e-11


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


@pytest.fixture(scope="module")
def line1d():
    """Config 3 inputs and the oracle's FP64 NDFT on 4096 random nodes and 4096
    random output frequencies."""
    N = (2 ** 22,)
    M = 2 ** 24
    rng = np.random.default_rng(3)
    k = (rng.random((1, M)) - 0.5).astype(np.float32)
    f = cnormal(N, 5)
    fhat = cnormal(M, 6)
    sub, lin = subsets(M, N[0], 8)
    k64 = k.astype(np.float64)
    ref_f = oracle.ndft_forward(k64, f.astype(np.complex128), subset=sub)
    ref_a = oracle.ndft_adjoint(k64, N, fhat.astype(np.complex128), subset=lin)
    return N, k, f, fhat, sub, lin, ref_f, ref_a


@pytest.mark.parametrize("compensated", [True, False])
def test_1d_large_accuracy(line1d, compensated):
    N, k, f, fhat, sub, lin, ref_f, ref_a = line1d
    p = nf.plan_nfft(k, N, m=5, sigma=2.0, compensated=compensated)
    y = (p * nf.as_colmajor(f, N, torch.complex64)).cpu().numpy()
    x = (nf.adjoint(p) * torch.as_tensor(fhat)).cpu().numpy()
    ef = oracle.rel_l2(y[sub], ref_f)
    ea = oracle.rel_l2(x[lin], ref_a)
    assert ef <= 1e-5 and ea <= 1e-5, (ef, ea)
