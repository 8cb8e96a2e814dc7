"""nfftgb300: GPU (GB300, sm_103a) NFFT plans behind the AbstractNFFTs interface.

The compute path is libnfftgb300.so (hand-written CUDA kernels + cuFFT behind
the C ABI of include/nfft_gb300.h); this package is the Python host binding.
"""
from .plan import (  # noqa: F401
    FULL, LINEAR, POLYNOMIAL, TENSOR, WINDOWS, AdjointPlan, ArgumentError, DimensionMismatch, GB300NFFTPlan,
    NFFTError, NFFTParams, PrecomputeFlags, TimingStats, accuracy_params, adjoint, as_colmajor, convolve_,
    convolve_transpose_, deconvolve_, deconvolve_transpose_, empty_image, kernel_launch_count, mul_, nfft,
    nfft_adjoint, GB300DirectionalPlan, NFFTBatch, nodes_, params_to_reltol, plan_nfft, reltol_to_params, size_in,
    size_out)
from .trig import (  # noqa: F401
    GB300NFCTPlan, GB300NFSTPlan, NDCTPlan, NDFTPlan, NDSTPlan, NNDFTPlan, ndct, ndct_transpose, ndct_transposed,
    ndft, ndft_adjoint, nfct, nfct_transpose, nfst, nfst_transpose, plan_nfct, plan_nfst, GB300NNFFTPlan,
    plan_nnfft)
from ._lib import LIB_PATH, exported_symbols, load  # noqa: F401
