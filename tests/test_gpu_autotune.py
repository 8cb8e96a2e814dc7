"""The tile-shape autotuner (nfft_autotune), which replaces the fixed
_blockSize defaults of src/precomputation.jl:59-77: its choice is one of its
candidates, the re-tiled plan still matches the oracle, the choice round-trips
through the NFFT_GB300_TUNE_CACHE file, and a cached re-tune reproduces the
same tiles and results."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import nfftgb300 as nf  # noqa: E402
from oracle import oracle  # noqa: E402


def candidates(D, Nt, compensated=False):
    """The autotuner's candidate (tile shape, warp layout) set, clipped to the grid."""
    if D == 1:
        c = [(b, 1, 1, 1) for b in (256, 512, 1024, 2048, 4096)]
    elif D == 2:
        c = [(a, b, 1, 1) for a, b in ((8, 8), (16, 8), (16, 16), (32, 16), (32, 32), (64, 32), (64, 64),
                                       (128, 64), (128, 128))]
    else:
        c = []
        for s in ((8, 8, 8), (16, 16, 8), (16, 16, 16), (32, 16, 8), (32, 32, 8), (16, 8, 8)):
            c.append(s + (1,))
            if not compensated and s[1] >= 16:
                c.append(s + (2,))
    nt = list(Nt) + [1] * (3 - len(Nt))
    return {tuple(min(v, nt[d]) for d, v in enumerate(s[:3])) + (s[3],) for s in c}


def cache_entries(path):
    rows = {}
    for line in open(path):
        parts = line.split()
        rows[parts[0]] = tuple(int(v) for v in parts[1:5])
    return rows


CASES = [
    (3, (40, 36, 32), 30000, np.float32),
    (3, (24, 24, 24), 20000, np.float64),
    (2, (160, 128), 60000, np.float32),
    (2, (96, 96), 20000, np.float64),
]


@pytest.mark.parametrize("D,N,M,dtype", CASES)
def test_autotune_choice_parity_and_cache(tmp_path, monkeypatch, D, N, M, dtype):
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("NFFT_GB300_TUNE_CACHE", str(cache))
    rng = np.random.default_rng(D * 100 + M % 97)
    k = (rng.random((D, M)) - 0.5).astype(dtype)
    f = (rng.standard_normal(N) + 1j * rng.standard_normal(N)) / np.sqrt(2)
    fh = (rng.standard_normal(M) + 1j * rng.standard_normal(M)) / np.sqrt(2)
    cd = torch.complex64 if dtype == np.float32 else torch.complex128
    tol = 1e-5 if dtype == np.float32 else 1e-11
    p = nf.plan_nfft(k, N, m=4, sigma=2.0, precompute=nf.TENSOR)
    p.autotune(use_cache=False)
    rows = cache_entries(cache)
    assert len(rows) == 1
    choice = next(iter(rows.values()))
    assert tuple(p.params.blockSize) == choice[:D]
    assert choice in candidates(D, p.Ñ)
    op = oracle.OraclePlan(k.astype(np.float64), N, m=4, sigma=2.0, precompute=oracle.TENSOR)
    fd = nf.as_colmajor(f, N, cd)
    y = (p * fd).cpu().numpy()
    x = (nf.adjoint(p) * torch.as_tensor(fh).to(cd)).cpu().numpy()
    assert oracle.rel_l2(y, op.forward(f)) < tol
    assert oracle.rel_l2(x, op.adjoint(fh)) < tol
    # a fresh plan with the default tiles picks the cached choice
    p2 = nf.plan_nfft(k, N, m=4, sigma=2.0, precompute=nf.TENSOR)
    p2.autotune(use_cache=True)
    assert tuple(p2.params.blockSize) == choice[:D]
    assert cache_entries(cache) == rows
    y2 = (p2 * fd).cpu().numpy()
    x2 = (nf.adjoint(p2) * torch.as_tensor(fh).to(cd)).cpu().numpy()
    assert np.array_equal(y2, y)  # same tiles, same gather: bit-identical
    # the spreading flush adds tiles with atomics in no fixed order
    assert oracle.rel_l2(x2, x) < (1e-6 if dtype == np.float32 else 1e-13)


def test_autotune_cache_file_reloaded_when_the_variable_changes(tmp_path, monkeypatch):
    """Pointing NFFT_GB300_TUNE_CACHE at another file makes the library read
    that file: a hand-written entry for the plan's key is applied as is."""
    rng = np.random.default_rng(4)
    N, M = (64, 64), 20000
    k = (rng.random((2, M)) - 0.5).astype(np.float32)
    first = tmp_path / "a.txt"
    monkeypatch.setenv("NFFT_GB300_TUNE_CACHE", str(first))
    p = nf.plan_nfft(k, N, m=4, sigma=2.0, precompute=nf.TENSOR)
    p.autotune(use_cache=False)
    key, choice = next(iter(cache_entries(first).items()))
    forced = (16, 8, 1, 1) if choice[:2] != (16, 8) else (32, 16, 1, 1)
    second = tmp_path / "b.txt"
    second.write_text(f"{key} {forced[0]} {forced[1]} {forced[2]} {forced[3]}\n")
    monkeypatch.setenv("NFFT_GB300_TUNE_CACHE", str(second))
    p2 = nf.plan_nfft(k, N, m=4, sigma=2.0, precompute=nf.TENSOR)
    p2.autotune(use_cache=True)
    assert tuple(p2.params.blockSize) == forced[:2]
    f = (rng.standard_normal(N) + 1j * rng.standard_normal(N)) / np.sqrt(2)
    op = oracle.OraclePlan(k.astype(np.float64), N, m=4, sigma=2.0, precompute=oracle.TENSOR)
    y = (p2 * nf.as_colmajor(f, N, torch.complex64)).cpu().numpy()
    assert oracle.rel_l2(y, op.forward(f)) < 1e-5
