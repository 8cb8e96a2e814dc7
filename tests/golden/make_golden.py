"""Generate the golden fixtures of tests/golden/*.npz.

The reference (a Julia package) cannot run in this environment, so its own
outputs cannot be captured.  The fixtures hold seeded inputs together with
(a) the direct NDFT in FP64 (src/direct.jl:99-151), the exact ground truth the
reference's tests compare against, and (b) the oracle's NFFT outputs and
integer binning for the same inputs, as regression anchors.

Run from the repository root:  python tests/golden/make_golden.py [d1 d2 d3 tools]

tools.npz adds NFFTTools' Toeplitz kernel and product and the direct NDCT,
NDST and NNDFT on seeded 2-D inputs.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle  # noqa: E402

CASES = {
    "d1": dict(N=(32,), M=40, seed=123),
    "d2": dict(N=(12, 10), M=100, seed=124),
    "d3": dict(N=(6, 8, 6), M=150, seed=125),
}


def make(name, N, M, seed):
    rng = np.random.default_rng(seed)
    D = len(N)
    k = rng.random((D, M)) - 0.5
    f = (rng.standard_normal(N) + 1j * rng.standard_normal(N)) / np.sqrt(2)
    fhat = (rng.standard_normal(M) + 1j * rng.standard_normal(M)) / np.sqrt(2)
    out = dict(k=k, f=f, fhat=fhat, N=np.array(N))
    out["ndft_forward"] = oracle.ndft_forward(k, f)
    out["ndft_adjoint"] = oracle.ndft_adjoint(k, N, fhat)
    op = oracle.OraclePlan(k, N, m=4, sigma=2.0, precompute=oracle.TENSOR)
    out["nfft_forward_m4"] = op.forward(f)
    out["nfft_adjoint_m4"] = op.adjoint(fhat)
    b = op.blocks()
    out["block_start"] = b["block_start"]
    out["block_nodes"] = b["nodes"]
    out["trunc"] = b["trunc"]
    out["deconv_factors"] = np.concatenate(op.inv)
    out["poly_coeffs_m4"] = op.coeffs
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), f"{name}.npz"), **out)


def make_tools(seed=126):
    """NFFTTools' Toeplitz kernel / product and the direct NDCT / NDST / NNDFT
    of src/direct.jl on seeded 2-D inputs (oracle, FP64)."""
    rng = np.random.default_rng(seed)
    N = (12, 10)
    tr = rng.random((2, 200)) - 0.5
    x = (rng.standard_normal(N) + 1j * rng.standard_normal(N)) / np.sqrt(2)
    lam = oracle.toeplitz_kernel(N, tr, m=4, sigma=2.0)
    out = dict(N=np.array(N), tr=tr, x=x, toeplitz_kernel_m4=lam,
               toeplitz_kernel_explicit=oracle.toeplitz_kernel_explicit(N, tr),
               toeplitz_product_m4=oracle.convolve_toeplitz(x, lam))
    kc = 0.5 * rng.random((2, 60))
    fr = rng.standard_normal(N)
    v = rng.standard_normal(60)
    out.update(kc=kc, fr=fr, v=v, ndct_forward=oracle.ndct_forward(kc, fr),
               ndct_transpose=oracle.ndct_transpose(kc, N, v),
               ndst_forward=oracle.ndst_forward(kc, fr),
               ndst_transpose=oracle.ndst_transpose(kc, tuple(n + 1 for n in N), v))
    y = (rng.random((2, 30)) - 0.5) * 10
    fy = (rng.standard_normal(30) + 1j * rng.standard_normal(30)) / np.sqrt(2)
    out.update(y=y, fy=fy, nndft_forward=oracle.nndft_forward(tr[:, :60], y, fy),
               nndft_adjoint=oracle.nndft_adjoint(tr[:, :60], y, out["ndct_forward"].astype(np.complex128)))
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tools.npz"), **out)


if __name__ == "__main__":
    which = sys.argv[1:] or list(CASES) + ["tools"]
    for name in which:
        if name == "tools":
            make_tools()
        else:
            make(name, **CASES[name])
        print("wrote", name)
