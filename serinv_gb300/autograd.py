"""Differentiable ``logdet(A) + y^T A^{-1} y`` for SPD BTA matrices.

``bta_logdet_quad(D, Lo, Ar, T, y, precision="fp64")`` returns the scalar
loss for the matrix whose lower stacks are ``D (n,b,b)``, ``Lo (n-1,b,b)``,
``Ar (n,a,b)``, ``T (a,a)`` (only the lower triangles of ``D`` and ``T`` are
read, as by ``pobtaf``) and a right-hand side ``y (n*b+a,)`` or
``(n*b+a, k)`` (then the loss sums the k quadratic forms).

Forward: ``pobtaf`` on a copy of the stacks, ``logdet = 2 sum log diag L``,
``x = A^{-1} y`` by ``pobtas`` (N then T).
Backward: ``dL/dA = A^{-1} - x x^T`` restricted to the BTA pattern — the
selected inverse from ``pobtasi`` minus the pattern blocks of ``x x^T`` —
mapped to the parameterisation: an entry of a stored lower block stands for
two entries of the symmetric matrix, so strictly-lower entries of ``D`` and
``T`` and every entry of ``Lo`` and ``Ar`` get twice the symmetric-matrix
gradient; strictly-upper entries of ``D`` and ``T`` (never read) get zero.
``dL/dy = 2 x``.
"""

from __future__ import annotations

import torch

from .algs import pobtaf, pobtas, pobtasi


def _pattern_outer(x: torch.Tensor, n: int, b: int, a: int):
    """Blocks of x x^T on the BTA pattern (x: (N, k); sums over the k columns)."""
    xb = x[: n * b].reshape(n, b, -1)
    xt = x[n * b:]
    oD = torch.bmm(xb, xb.transpose(1, 2))
    oLo = torch.bmm(xb[1:], xb[:-1].transpose(1, 2)) if n > 1 else xb.new_zeros((0, b, b))
    oAr = torch.matmul(xt.unsqueeze(0), xb.transpose(1, 2)) if a else xb.new_zeros((n, 0, b))
    oT = xt @ xt.T if a else xb.new_zeros((0, 0))
    return oD, oLo, oAr, oT


def _sym_param(G: torch.Tensor) -> torch.Tensor:
    """Gradient w.r.t. a stored lower triangle: 2 G below, G on, 0 above the diagonal."""
    return torch.tril(G, -1) * 2.0 + torch.diag_embed(torch.diagonal(G, dim1=-2, dim2=-1))


class BTALogdetQuad(torch.autograd.Function):
    @staticmethod
    def forward(ctx, D, Lo, Ar, T, y, precision):
        L = [t.detach().clone().contiguous() for t in (D, Lo, Ar, T)]
        pobtaf(*L, precision=precision)
        n, b, a = D.shape[0], D.shape[1], Ar.shape[1]
        logdet = 2.0 * torch.log(torch.diagonal(L[0], dim1=1, dim2=2)).sum()
        if a:
            logdet = logdet + 2.0 * torch.log(torch.diagonal(L[3])).sum()
        yy = y.detach().reshape(n * b + a, -1).contiguous()
        x = yy.clone()
        pobtas(*L, x, trans="N")
        pobtas(*L, x, trans="T")
        quad = (yy * x).sum()
        ctx.save_for_backward(*L, x)
        ctx.precision = precision
        ctx.yshape = y.shape
        return logdet + quad

    @staticmethod
    def backward(ctx, g):
        L0, L1, L2, L3, x = ctx.saved_tensors
        n, b, a = L0.shape[0], L0.shape[1], L2.shape[1]
        X = [t.clone() for t in (L0, L1, L2, L3)]
        pobtasi(*X, precision=ctx.precision)  # A^{-1} on the pattern
        oD, oLo, oAr, oT = _pattern_outer(x, n, b, a)
        GD = X[0] - oD
        GLo = X[1] - oLo
        GAr = X[2] - oAr
        GT = X[3] - oT
        dD = _sym_param(GD) * g
        dLo = 2.0 * GLo * g
        dAr = 2.0 * GAr * g
        dT = (_sym_param(GT) if a else GT) * g
        dy = (2.0 * x * g).reshape(ctx.yshape)
        return dD, dLo, dAr, dT, dy, None


def bta_logdet_quad(D, Lo, Ar, T, y, precision: str = "fp64") -> torch.Tensor:
    """Differentiable logdet(A) + y^T A^{-1} y (see the module docstring)."""
    return BTALogdetQuad.apply(D, Lo, Ar, T, y, precision)
