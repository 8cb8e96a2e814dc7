"""Differentiation rules of the NFFT plan for torch.autograd.

Mirrors AbstractNFFTs' ChainRulesCore extension
(AbstractNFFTs/ext/AbstractNFFTsChainRulesCoreExt.jl:14-64):

* ``plan_apply(p, f)`` = ``p * f``; pullback ``adjoint(p) * ȳ`` (:14-22).
* ``plan_apply_adjoint(p, fHat)`` = ``adjoint(p) * fHat``; pullback ``p * x̄``.
* ``nfft_nodes(k, f, p)`` = ``A(k) f`` with gradients for BOTH ``f`` and the node
  coordinates ``k``.  The reference returns NoTangent for ``k`` (:45, :61);
  here the node gradient comes from the library's ∂k kernel, which recomputes
  the window and its derivative per tap instead of storing a sparse matrix.

Complex gradients follow torch's convention (conjugate Wirtinger): for a
real loss L and y = A f, grad_f = A^H grad_y and
grad_k[d, j] = Re(conj(grad_y[j]) * dy_j/dk[d, j]).
"""
from __future__ import annotations

import torch

from . import plan as P


def _colmajor_from(x, p):
    return P.as_colmajor(x, p.N, p.cdtype, p.device)


class _Apply(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f, p):
        ctx.p = p
        fhat = torch.empty(p.NOut, dtype=p.cdtype, device=p.device)
        return p.forward_(fhat, _colmajor_from(f.detach(), p))

    @staticmethod
    def backward(ctx, gy):
        p = ctx.p
        out = P.empty_image(p.N, p.cdtype, p.device)
        return p.adjoint_(out, gy.detach().to(p.cdtype).contiguous()), None


class _ApplyAdjoint(torch.autograd.Function):
    @staticmethod
    def forward(ctx, fhat, p):
        ctx.p = p
        out = P.empty_image(p.N, p.cdtype, p.device)
        return p.adjoint_(out, fhat.detach().to(p.cdtype).contiguous())

    @staticmethod
    def backward(ctx, gx):
        p = ctx.p
        fhat = torch.empty(p.NOut, dtype=p.cdtype, device=p.device)
        return p.forward_(fhat, _colmajor_from(gx.detach(), p)), None


class _NodesApply(torch.autograd.Function):
    @staticmethod
    def forward(ctx, k, f, p):
        p.nodes_(k.detach())
        ctx.p = p
        fd = _colmajor_from(f.detach(), p)
        ctx.save_for_backward(fd)
        fhat = torch.empty(p.NOut, dtype=p.cdtype, device=p.device)
        return p.forward_(fhat, fd)

    @staticmethod
    def backward(ctx, gy):
        p = ctx.p
        (fd,) = ctx.saved_tensors
        gy = gy.detach().to(p.cdtype).contiguous()
        gk = gf = None
        if ctx.needs_input_grad[0]:
            D = len(p.N)
            buf = torch.empty((p.J, D), dtype=p.dtype, device=p.device)  # column-major (D, M)
            p.grad_nodes_(buf.t(), fd, gy)
            gk = buf.t()
        if ctx.needs_input_grad[1]:
            gf = P.empty_image(p.N, p.cdtype, p.device)
            p.adjoint_(gf, gy)
        return gk, gf, None


def plan_apply(p, f):
    """y = p * f, differentiable in f (rrule of *, :14-22)."""
    return _Apply.apply(f, p)


def plan_apply_adjoint(p, fhat):
    """x = adjoint(p) * fHat, differentiable in fHat."""
    return _ApplyAdjoint.apply(fhat, p)


def nfft_nodes(k, f, p):
    """y = A(k) f, differentiable in the nodes k (shape (D, M), real) and in f.
    The plan ``p`` is re-noded with ``k`` (nodes!) on every call."""
    return _NodesApply.apply(k, f, p)
