"""nfft_bin_nodes_noalloc: node binning for callers that cannot call
cudaMalloc (for example a host framework whose caching allocator owns the
device memory, or a pipeline that must not take cudaMalloc's implicit device
synchronisation).  Its scratch is a static device array inside the library.

The test calls it through the C ABI twice in a row, with two different node
sets so that the second call starts from the first call's leftover scratch,
and requires bit-identical results to the binning of the existing entry
point (nfft_set_nodes, read back with nfft_get_binning).  This file is
collected last so that a run stopping at the first failure has run every
other test before it.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import nfftgb300 as nf  # noqa: E402


def _bin_noalloc(k, Nt, bs):
    lib = nf.load()
    D, M = k.shape
    prec = 32 if k.dtype == np.float32 else 64
    kd = torch.from_numpy(np.ascontiguousarray(k.T)).cuda()  # column-major D x M
    ntiles = int(np.prod([-(-n // b) for n, b in zip(Nt, bs)]))
    perm = torch.full((max(M, 1),), -1, dtype=torch.int32, device="cuda")
    tstart = torch.full((ntiles + 1,), -1, dtype=torch.int32, device="cuda")
    Nt_a = (ctypes.c_int64 * 3)(*(list(Nt) + [1] * (3 - D)))
    bs_a = (ctypes.c_int64 * 3)(*(list(bs) + [1] * (3 - D)))
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.nfft_bin_nodes_noalloc(prec, D, Nt_a, bs_a, M, ctypes.c_void_p(kd.data_ptr()),
                                    ctypes.c_void_p(perm.data_ptr()), ctypes.c_void_p(tstart.data_ptr()),
                                    ctypes.c_void_p(stream))
    assert rc == 0, lib.nfft_last_error()
    torch.cuda.synchronize()
    return perm.cpu().numpy()[:M], tstart.cpu().numpy()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_noalloc_binning_matches_set_nodes_twice(dtype):
    rng = np.random.default_rng(2024)
    cases = [((40, 36, 30), 60000), ((40, 36, 30), 25000)]
    for N, M in cases:  # two calls in a row, different node sets
        k = (rng.random((3, M)) - 0.5).astype(dtype)
        k[:, :6] = np.array([-0.5, 0.5, 0.0, -0.25, 0.25, -np.finfo(dtype).tiny], dtype)
        p = nf.plan_nfft(k, N, m=4, sigma=2.0, blockSize=(16, 16, 16))
        ref = p.binning()
        perm, tstart = _bin_noalloc(k, p.Ñ, p.params.blockSize)
        assert np.array_equal(perm, ref["perm"])
        assert np.array_equal(tstart, ref["tile_start"])


@pytest.mark.parametrize("D,N,bs,M,dtype", [
    # the static scratch at its limits: 2^18 FP64 nodes in 3-D and exactly 2^18 tiles
    (3, (64, 64, 64), (2, 2, 2), 1 << 18, np.float64),
    (1, (1 << 15,), (64,), 50000, np.float32),
    (2, (128, 100), (16, 8), 70000, np.float64),
])
def test_noalloc_binning_at_the_limits_and_in_1d_2d(D, N, bs, M, dtype):
    rng = np.random.default_rng(D)
    k = (rng.random((D, M)) - 0.5).astype(dtype)
    k[:, :3] = np.array([-0.5, 0.5, 0.0], dtype)  # boundary nodes in every dimension
    p = nf.plan_nfft(k, N, m=4, sigma=2.0, blockSize=bs)
    ref = p.binning()
    if D == 3:
        assert len(ref["tile_start"]) == (1 << 18) + 1
    perm, tstart = _bin_noalloc(k, p.Ñ, p.params.blockSize)
    assert np.array_equal(perm, ref["perm"])
    assert np.array_equal(tstart, ref["tile_start"])


def test_noalloc_rejects_oversized_request():
    lib = nf.load()
    Nt = (ctypes.c_int64 * 3)(64, 64, 64)
    bs = (ctypes.c_int64 * 3)(16, 16, 16)
    rc = lib.nfft_bin_nodes_noalloc(32, 3, Nt, bs, (1 << 18) + 1, ctypes.c_void_p(1), ctypes.c_void_p(1),
                                    ctypes.c_void_p(1), None)
    assert rc == nf._lib.NFFT_ERR_UNSUPPORTED
    assert b"at most" in lib.nfft_last_error()
