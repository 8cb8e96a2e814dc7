"""NFFTTools clients on the GPU plan.

``sdc`` restates NFFTTools' sampling density compensation
(NFFTTools/src/samplingDensity.jl:59-155) on top of the plan's real-valued
``convolve!`` / ``convolve_transpose!`` and ``mul!``, the way NFFTTools uses the
reference's GPU plan (test/gpu.jl:52-65).
"""
from __future__ import annotations

import torch

from . import plan as P


def sdc(p, iters=20, weights=None, weights_tmp=None, workg=None, workf=None, workv=None):
    """Density compensation weights (real, length J) with the final scaling
    c = real(sum(v)) / ||v||^2 of sdc! (:138-155).  The work buffers may be
    passed in to avoid allocation, as in the reference."""
    T = p.dtype
    dev = p.device
    if weights is None:
        weights = torch.ones(p.J, dtype=T, device=dev)
    if weights_tmp is None:
        weights_tmp = torch.empty_like(weights)
    if workg is None:
        workg = P.empty_image(p.Ñ, T, dev)
    if workf is None:
        workf = torch.empty(p.J, dtype=p.cdtype, device=dev)
    if workv is None:
        workv = P.empty_image(p.N, p.cdtype, dev)
    scaling = None
    for i in range(iters):
        p.convolve_transpose_(weights, workg)
        if i == 0:
            scaling = workg.max()
        workg.div_(scaling)
        p.convolve_(workg, weights_tmp)
        weights_tmp.div_(scaling)
        if bool((weights_tmp <= 0).any()):
            raise ValueError("non-positive weights")
        weights.div_(weights_tmp)
    u = workv
    u.fill_(1)
    p.forward_(workf, u)
    workf.mul_(weights)
    p.adjoint_(workv, workf)
    c = workv.sum().real / (workv.abs() ** 2).sum()
    weights.mul_(c)
    return weights
