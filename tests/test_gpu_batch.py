"""Batched plans (nfft_batch_*): many plans of uneven N and M transformed as
one launch per stage, replayed as a CUDA graph.  Each member's result must
equal the member's own forward/adjoint (rel l2 <= 1e-12 FP64, 1e-6 FP32: only
the order of the grid flush's atomic additions differs) and the oracle
(1e-11 FP64 / 1e-5 FP32, as for single plans)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import nfftgb300 as nf  # noqa: E402
from oracle import oracle  # noqa: E402


def problems(D, shapes, Ms, seed, dtype):
    rng = np.random.default_rng(seed)
    out = []
    for N, M in zip(shapes, Ms):
        k = (rng.random((D, M)) - 0.5).astype(dtype)
        f = (rng.standard_normal(N) + 1j * rng.standard_normal(N)) / np.sqrt(2)
        fhat = (rng.standard_normal(M) + 1j * rng.standard_normal(M)) / np.sqrt(2)
        out.append((k, N, f, fhat))
    return out


SETS = {
    3: ([(16, 16, 16), (24, 20, 16), (32, 32, 8), (10, 12, 14)], [5000, 300, 12000, 1]),
    2: ([(64, 64), (100, 36), (33, 31), (128, 8)], [20000, 700, 1500, 0]),
}


@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("pre", [nf.POLYNOMIAL, nf.TENSOR])
def test_batch_matches_plans_and_oracle(D, prec, pre):
    dtype = np.float64 if prec == 64 else np.float32
    shapes, Ms = SETS[D]
    probs = problems(D, shapes, Ms, 50 + D, dtype)
    plans = [nf.plan_nfft(k, N, m=4, sigma=2.0, precompute=pre) for k, N, _, _ in probs]
    cd = plans[0].cdtype
    fs = [nf.as_colmajor(f, N, cd) for _, N, f, _ in probs]
    vs = [torch.as_tensor(fh).to(device="cuda", dtype=cd) for _, _, _, fh in probs]
    single_y = [(p * f).cpu().numpy() for p, f in zip(plans, fs)]
    single_x = [(nf.adjoint(p) * v).cpu().numpy() for p, v in zip(plans, vs)]
    batch = nf.NFFTBatch(plans)
    tol_self = 1e-12 if prec == 64 else 1e-6
    tol_or = 1e-11 if prec == 64 else 1e-5
    for rep in range(2):  # the second call replays the captured graphs
        ys = [y.cpu().numpy() for y in batch.forward(fs)]
        xs = [x.cpu().numpy() for x in batch.adjoint(vs)]
        for i, (k, N, f, fh) in enumerate(probs):
            if Ms[i] == 0:
                assert ys[i].shape == (0,)
                assert np.all(xs[i] == 0)
                continue
            assert oracle.rel_l2(ys[i], single_y[i]) <= tol_self, (rep, i)
            assert oracle.rel_l2(xs[i], single_x[i]) <= tol_self, (rep, i)
            if rep == 0:
                op = oracle.OraclePlan(k.astype(np.float64), N, m=4, sigma=2.0,
                                       precompute=oracle.TENSOR if pre == nf.TENSOR else oracle.POLYNOMIAL)
                assert oracle.rel_l2(ys[i], op.forward(f)) <= tol_or, i
                assert oracle.rel_l2(xs[i], op.adjoint(fh)) <= tol_or, i


def test_batch_new_inputs_each_call():
    probs = problems(3, *SETS[3], 7, np.float64)
    plans = [nf.plan_nfft(k, N, m=4, sigma=2.0) for k, N, _, _ in probs]
    batch = nf.NFFTBatch(plans)
    rng = np.random.default_rng(3)
    for _ in range(3):
        fs = [nf.as_colmajor(rng.standard_normal(p.N) + 1j * rng.standard_normal(p.N), p.N, p.cdtype)
              for p in plans]
        ys = batch.forward(fs)
        for p, f, y in zip(plans, fs, ys):
            if p.J:
                assert oracle.rel_l2(y.cpu().numpy(), (p * f).cpu().numpy()) <= 1e-12


def test_batch_rejects_mismatched_and_stale():
    rng = np.random.default_rng(0)
    k3 = rng.random((3, 100)) - 0.5
    a = nf.plan_nfft(k3, (8, 8, 8), m=4, sigma=2.0)
    with pytest.raises(nf.ArgumentError):
        nf.NFFTBatch([a, nf.plan_nfft(k3, (8, 8, 8), m=3, sigma=2.0)])
    with pytest.raises(nf.ArgumentError):
        nf.NFFTBatch([a, nf.plan_nfft(k3, (8, 8, 8), m=4, sigma=2.0, compensated=True)])
    with pytest.raises(nf.ArgumentError):
        nf.NFFTBatch([a, nf.plan_nfft(k3.astype(np.float32), (8, 8, 8), m=4, sigma=2.0)])
    with pytest.raises(nf.ArgumentError):
        nf.NFFTBatch([a, nf.plan_nfft(k3[:2], (8, 8), m=4, sigma=2.0)])
    with pytest.raises(NotImplementedError):
        nf.NFFTBatch([nf.plan_nfft(k3[:1], (64,), m=4, sigma=2.0)])
    b = nf.plan_nfft(k3, (12, 8, 10), m=4, sigma=2.0)
    batch = nf.NFFTBatch([a, b])
    fs = [nf.as_colmajor(np.ones(p.N, complex), p.N, p.cdtype) for p in (a, b)]
    batch.forward(fs)
    b.nodes_(rng.random((3, 100)) - 0.5)
    with pytest.raises(nf.ArgumentError):
        batch.forward(fs)
    with pytest.raises(nf.DimensionMismatch):
        nf.NFFTBatch([a]).forward(fs)


def config4_plans(seed=4, nplans=64):
    """64 2-D FP32 plans: N_i from {64, 96, 128, 192, 256, 384, 512} (grids of
    2 N_i, radix-3 sizes included), M_i = floor(10^U(4, 6)), nodes U[-1/2, 1/2)^2,
    Kaiser-Bessel m = 4, sigma = 2."""
    rng = np.random.default_rng(seed)
    sizes = [64, 96, 128, 192, 256, 384, 512]
    out = []
    for _ in range(nplans):
        n = int(rng.choice(sizes))
        M = int(10 ** rng.uniform(4, 6))
        k = (rng.random((2, M)) - 0.5).astype(np.float32)
        out.append((k, (n, n)))
    return out


def test_batch_config4_64_plans():
    probs = config4_plans()
    plans = [nf.plan_nfft(k, N, m=4, sigma=2.0) for k, N in probs]
    batch = nf.NFFTBatch(plans)
    rng = np.random.default_rng(9)
    fs = [nf.as_colmajor((rng.standard_normal(N) + 1j * rng.standard_normal(N)).astype(np.complex64), N,
                         torch.complex64) for _, N in probs]
    vs = [torch.as_tensor((rng.standard_normal(k.shape[1]) + 1j * rng.standard_normal(k.shape[1]))
                          .astype(np.complex64)).cuda() for k, _ in probs]
    ys = batch.forward(fs)
    xs = batch.adjoint(vs)
    for i, (p, (k, N)) in enumerate(zip(plans, probs)):
        assert oracle.rel_l2(ys[i].cpu().numpy(), (p * fs[i]).cpu().numpy()) <= 1e-6, i
        assert oracle.rel_l2(xs[i].cpu().numpy(), (nf.adjoint(p) * vs[i]).cpu().numpy()) <= 1e-6, i
    # accuracy of every member against the FP64 NDFT (oracle) on 256 random
    # nodes (forward) and 256 random output frequencies (adjoint)
    for i, (k, N) in enumerate(probs):
        k64 = k.astype(np.float64)
        f = fs[i].cpu().numpy().astype(np.complex128)
        rs = np.random.default_rng(100 + i)
        sub = rs.choice(k.shape[1], 256, replace=False)
        lin = rs.choice(N[0] * N[1], 256, replace=False)
        ref = oracle.ndft_forward(k64, f, subset=sub)
        assert oracle.rel_l2(ys[i].cpu().numpy()[sub], ref) <= 1e-5, i
        refx = oracle.ndft_adjoint(k64, N, vs[i].cpu().numpy().astype(np.complex128), subset=lin)
        assert oracle.rel_l2(xs[i].cpu().numpy().ravel(order="F")[lin], refx) <= 1e-5, i
