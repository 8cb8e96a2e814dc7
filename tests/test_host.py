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
