"""Host-side logic of the Python binding (no GPU)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import nfftgb300 as nf  # noqa: E402
from nfftgb300 import plan as P  # noqa: E402
from oracle import oracle  # noqa: E402


def test_accuracy_params_match_oracle():
    for kw in [{}, {"reltol": 1e-5}, {"reltol": 1e-12}, {"m": 3}, {"m": 3, "sigma": 1.5}, {"sigma": 2.0}]:
        assert nf.accuracy_params(**kw) == oracle.accuracy_params(**kw)


def test_colmajor_helpers():
    x = nf.empty_image((3, 4, 5), torch.float64, "cpu")
    assert tuple(x.shape) == (3, 4, 5) and x.stride() == (1, 3, 12)
    a = np.arange(60.0).reshape(3, 4, 5)
    y = nf.as_colmajor(a, (3, 4, 5), torch.float64, "cpu")
    assert P._is_colmajor(y)
    assert np.array_equal(y.numpy(), a)
    # memory order is Julia's: element (i0, i1, i2) at i0 + 3 i1 + 12 i2
    flat = y.permute(2, 1, 0).contiguous().reshape(-1).numpy()
    assert np.array_equal(flat, a.ravel(order="F"))
    with pytest.raises(nf.DimensionMismatch):
        nf.as_colmajor(a, (3, 4, 6), torch.float64, "cpu")


def test_exceptions_are_julia_named():
    assert issubclass(nf.DimensionMismatch, ValueError)
    assert issubclass(nf.ArgumentError, ValueError)
    assert int(nf.PrecomputeFlags.FULL) == 1 and int(nf.PrecomputeFlags.POLYNOMIAL) == 4


@pytest.mark.parametrize("N", [(16,), (12, 10), (8, 6, 10)])
def test_bench_sparse_b_comparator_matches_oracle(N):
    """bench.py's restatement of the reference's GPU algorithm (sparse B of
    exact window values + FFT) equals the oracle's FULL plan (on the CPU)."""
    torch = pytest.importorskip("torch")
    import bench
    from oracle import oracle
    rng = np.random.default_rng(len(N))
    D, M = len(N), 300
    k = rng.random((D, M)) - 0.5
    f = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    fh = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    inv = np.concatenate(oracle.deconv_factors("kaiser_bessel", N, tuple(2 * n for n in N), 4, 2.0))
    sb = bench.SparseBPath(k, N, 4, 2.0, inv, torch.float64, "cpu")
    y = sb.forward(torch.as_tensor(f.ravel(order="F"))).numpy()
    x = sb.adjoint(torch.as_tensor(fh)).numpy()
    op = oracle.OraclePlan(k, N, m=4, sigma=2.0, precompute=oracle.FULL)
    assert oracle.rel_l2(y, op.forward(f)) < 1e-13
    assert oracle.rel_l2(x, op.adjoint(fh).ravel(order="F")) < 1e-13


def test_bench_error_subsets_and_frequencies():
    """bench.py's error measurement: 4096 distinct sorted nodes / outputs, and
    the frequencies n - N div 2 of column-major output indices (the NNDFT
    points whose adjoint equals the NDFT adjoint there)."""
    import bench
    sub, lin = bench.error_subsets(10 ** 6, 256 ** 3)
    assert len(sub) == len(np.unique(sub)) == 4096 and np.all(np.diff(sub) > 0)
    assert len(lin) == 4096 and lin.max() < 256 ** 3
    N = (6, 8, 10)
    lin = np.arange(0, 480, 7)
    fr = bench.frequencies(N, lin)
    grids = np.meshgrid(*[np.arange(n) - n // 2 for n in N], indexing="ij")
    for d in range(3):
        assert np.array_equal(fr[d], grids[d].ravel(order="F")[lin])


def test_bench_clock_sampler_keeps_the_timed_region():
    """bench.py's clock record: nvidia-smi lines (timestamp first) are parsed,
    only samples inside the marked timed region count, throttle reasons are
    collected, and a region shorter than the interval takes the nearest
    sample."""
    import datetime
    import bench
    t0 = datetime.datetime(2026, 1, 2, 3, 4, 5, 0)

    def line(dt_ms, sm, reasons=("Not Active",) * 4):
        ts = (t0 + datetime.timedelta(milliseconds=dt_ms)).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
        return ", ".join([ts, "0", str(sm), "2070", "800.00 W", "0x0"] + list(reasons))

    cs = bench.ClockSampler()
    cs.out = [line(0, 1000), line(50, 2070), line(100, 2060, ("Not Active", "Not Active", "Not Active", "Active")),
              line(150, 2070), line(200, 900)]
    base = t0.timestamp()
    cs.t0, cs.t1 = base + 0.040, base + 0.160
    s = cs.summary()
    assert s["samples"] == 3 and s["sm_mhz"] == 2070 and s["sm_max_mhz"] == 2070
    assert s["reasons"] == ["sw_power_cap"] and s["window"] == "timed region"
    cs.t0, cs.t1 = base + 0.060, base + 0.070
    s = cs.summary()
    assert s["samples"] == 1 and s["sm_mhz"] == 2070 and s["window"].startswith("nearest")
    cs.out = ["garbage", ""]
    assert cs.summary() is None
