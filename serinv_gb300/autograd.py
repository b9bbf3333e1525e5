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
That mapping, the pattern blocks of ``x x^T`` and the scaling by the
upstream gradient run as one in-place pass over the selected inverse
(``sgb_bta_logdet_quad_grad``).  ``dL/dy = 2 x``.
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib
from .algs import _bta_struct, pobtaf, pobtas, pobtasi


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
        X = [t.clone() for t in (L0, L1, L2, L3)]
        pobtasi(*X, precision=ctx.precision)  # A^{-1} on the pattern
        # in place: X <- g * (A^{-1} - x x^T) on the pattern, mapped to the stored lower stacks
        gs = g.detach().to(device=x.device, dtype=x.dtype).reshape(1).contiguous()
        m = _bta_struct(*X)
        with torch.cuda.device(x.device):
            rc = _lib.load().sgb_bta_logdet_quad_grad(ctypes.byref(m), x.data_ptr(), x.shape[1], x.shape[1],
                                                       gs.data_ptr(), torch.cuda.current_stream(x.device).cuda_stream)
        _lib.raise_for(rc, "logdet/quadratic-form backward")
        dy = (2.0 * x * g).reshape(ctx.yshape)
        return X[0], X[1], X[2], X[3], dy, None


def bta_logdet_quad(D, Lo, Ar, T, y, precision: str = "fp64") -> torch.Tensor:
    """Differentiable logdet(A) + y^T A^{-1} y (see the module docstring)."""
    return BTALogdetQuad.apply(D, Lo, Ar, T, y, precision)
