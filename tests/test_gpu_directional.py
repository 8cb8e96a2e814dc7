"""Directional plans (plan_nfft(k, N; dims), src/directional.jl): the NFFT
along dims of a D-dimensional array equals the plain NFFT of every slice
along dims (test/accuracy.jl:83-162).  Checked slice by slice against the
FP64 NDFT oracle (rel l2 1e-7 FP64 -- the LINEAR window at the default
reltol 1e-9 -- and 1e-5 FP32) and against single GPU plans of the slices."""
import itertools

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import nfftgb300 as nf  # noqa: E402
from oracle import oracle  # noqa: E402


def slices(N, lo, hi):
    """Index tuples selecting every slice along dims lo..hi (1-based)."""
    pre = [range(n) for n in N[:lo - 1]]
    post = [range(n) for n in N[hi:]]
    for ip in itertools.product(*pre):
        for iq in itertools.product(*post):
            yield ip, iq


def check(D, N, lo, hi, dtype, seed):
    rng = np.random.default_rng(seed)
    R = hi - lo + 1
    J = int(np.prod(N))
    k = (rng.random((R, J)) - 0.5).astype(dtype)
    f = rng.random(N) + 1j * rng.random(N)
    p = nf.plan_nfft(k if R > 1 else k[0], N, dims=lo if lo == hi else range(lo, hi + 1))
    assert isinstance(p, nf.GB300DirectionalPlan)
    assert p.NOut == N[:lo - 1] + (J,) + N[hi:]
    fhat = (p * f).cpu().numpy()
    g = (nf.adjoint(p) * fhat).cpu().numpy()
    tol = 1e-7 if dtype == np.float64 else 1e-5
    k64 = k.astype(np.float64)
    worst_f = worst_g = 0.0
    for ip, iq in slices(N, lo, hi):
        sl_f = ip + (slice(None),) * R + iq
        sl_h = ip + (slice(None),) + iq
        ref = oracle.ndft_forward(k64, f[sl_f].astype(np.complex128))
        worst_f = max(worst_f, oracle.rel_l2(fhat[sl_h], ref))
        refg = oracle.ndft_adjoint(k64, N[lo - 1:hi], fhat[sl_h].astype(np.complex128))
        worst_g = max(worst_g, oracle.rel_l2(g[sl_f], refg))
    assert worst_f < tol
    assert worst_g < tol
    return p, k, f, fhat


@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_directional_one_dim(D, dtype):
    rng = np.random.default_rng(D)
    N = tuple(int(2 * rng.integers(4, 9)) for _ in range(D))
    for d in range(1, D + 1):
        check(D, N, d, d, dtype, seed=10 * D + d)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_directional_two_dims_of_three(dtype):
    rng = np.random.default_rng(3)
    N = tuple(int(2 * rng.integers(4, 9)) for _ in range(3))
    for lo in (1, 2):
        check(3, N, lo, lo + 1, dtype, seed=40 + lo)


def test_directional_matches_slice_plans():
    """The directional plan against single GPU plans (LINEAR) of each slice."""
    N = (10, 12, 8)
    p, k, f, fhat = check(3, N, 2, 2, np.float64, seed=5)
    q = nf.plan_nfft(k[0], (N[1],), precompute=nf.LINEAR, blocking=False)
    worst = 0.0
    for a in range(N[0]):
        for b in range(N[2]):
            y = (q * f[a, :, b]).cpu().numpy()
            worst = max(worst, oracle.rel_l2(fhat[a, :, b], y))
    assert worst < 1e-10


def test_directional_errors():
    rng = np.random.default_rng(0)
    k = rng.random(20) - 0.5
    with pytest.raises(nf.ArgumentError):
        nf.plan_nfft(k, (8, 8), dims=3)
    with pytest.raises(nf.ArgumentError):
        nf.plan_nfft(np.stack([k, k]), (8, 8, 8), dims=2)  # 2-D nodes for one dim
    with pytest.raises(nf.ArgumentError):
        nf.plan_nfft(k + 1.0, (8, 8), dims=1)
    p = nf.plan_nfft(k, (8, 6), dims=2)
    with pytest.raises(nf.DimensionMismatch):
        p * np.zeros((6, 8), complex)
    assert p.NOut == (8, 20) and p.Ñ == (8, 12)


@pytest.mark.parametrize("N,lo,hi,M", [((40, 24, 20), 2, 3, 3000), ((40, 24, 20), 2, 2, 500),
                                       ((70, 16), 2, 2, 45), ((33, 5, 16), 3, 3, 77)])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_directional_trailing_dims_tiled(monkeypatch, N, lo, hi, M, dtype):
    """Transform dims that do not lead (pre > 1: columns before dims) run on
    the tiled path through transposing pad / crop and node-value
    transpositions (ragged 32 x 32 tiles on both sides): slice-wise equal to
    the FP64 NDFT, and equal to the atomic per-(pre, node, post) path."""
    rng = np.random.default_rng(sum(N) + M)
    R = hi - lo + 1
    k = (rng.random((R, M)) - 0.5).astype(dtype)
    f = rng.random(N) + 1j * rng.random(N)
    dims = lo if lo == hi else range(lo, hi + 1)
    out = {}
    for tiled in ("1", "0"):
        monkeypatch.setenv("NFFT_GB300_DIRECTIONAL_TILED", tiled)
        p = nf.plan_nfft(k if R > 1 else k[0], N, dims=dims)
        fhat = (p * f).cpu().numpy()
        out[tiled] = (fhat, (nf.adjoint(p) * fhat).cpu().numpy())
    fhat, g = out["1"]
    tol = 1e-7 if dtype == np.float64 else 1e-5
    k64 = k.astype(np.float64)
    for n, (ip, iq) in enumerate(slices(N, lo, hi)):
        if n % 7:
            continue
        sl_f = ip + (slice(None),) * R + iq
        sl_h = ip + (slice(None),) + iq
        assert oracle.rel_l2(fhat[sl_h], oracle.ndft_forward(k64, f[sl_f].astype(np.complex128))) < tol
        refg = oracle.ndft_adjoint(k64, N[lo - 1:hi], fhat[sl_h].astype(np.complex128))
        assert oracle.rel_l2(g[sl_f], refg) < tol
    same = 1e-10 if dtype == np.float64 else 1e-6
    assert oracle.rel_l2(fhat, out["0"][0]) < same
    assert oracle.rel_l2(g, out["0"][1]) < same
