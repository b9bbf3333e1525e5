"""Iteratively refined solve and the symmetric BTA product.

``pobtas_refine`` solves ``A x = B`` with a Cholesky factor ``L`` of ``A``
(from ``pobtaf``, FP64 or mixed precision) and refines the solution against
the original matrix: ``x <- L^{-T} L^{-1} B``, then ``iters`` times
``r = B - A x`` (in the storage precision, from A's lower stacks) and
``x += L^{-T} L^{-1} r``.  With a mixed-precision factor (relative error
~1e-11 at moderate conditioning) one or two steps bring the solution to the
FP64 solve's accuracy.  The reference has no such call: its ``pobtas``
(src/serinv/algs/pobtas.py:10-62) is the unrefined solve, which is what
``pobtas_refine(..., iters=0)`` computes.

``bta_matvec`` is the product ``y = A x`` used for the residual.
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib
from .algs import _bta_struct, _finish, _prepare, _ptr, _stream, _workspace


def bta_matvec(A_diagonal_blocks, A_lower_diagonal_blocks, A_lower_arrow_blocks, A_arrow_tip_block, x,
               alpha: float = 1.0, beta: float = 0.0, y=None):
    """``y = alpha * A x + beta * y`` for the symmetric BTA matrix of the lower
    stacks (only the lower triangles of the diagonal blocks and of the tip are
    read).  ``x``: (n*b + a,) or (n*b + a, nrhs).  Returns ``y`` (a new device
    tensor unless given)."""
    lib = _lib.load()
    arrays = [A_diagonal_blocks, A_lower_diagonal_blocks, A_lower_arrow_blocks, A_arrow_tip_block, x]
    names = ["A_diagonal_blocks", "A_lower_diagonal_blocks", "A_lower_arrow_blocks", "A_arrow_tip_block", "x"]
    if y is not None:
        arrays.append(y)
        names.append("y")
    device, w = _prepare(arrays, names)
    m = _bta_struct(*(t.t for t in w[:4]))
    N = m.n * m.b + m.a
    xt = w[4].t
    squeeze = xt.dim() == 1
    xt = xt.view(-1, 1) if squeeze else xt
    if xt.dim() != 2 or xt.shape[0] != N:
        raise ValueError(f"x must have shape ({N}, nrhs), got {tuple(w[4].t.shape)}")
    if xt.dtype != w[0].t.dtype:
        raise TypeError(f"x has dtype {xt.dtype}, the blocks have {w[0].t.dtype}")
    if y is None:
        yt = torch.zeros_like(xt)
        beta = 0.0
    else:
        yt = w[5].t.view(-1, 1) if w[5].t.dim() == 1 else w[5].t
        if tuple(yt.shape) != tuple(xt.shape) or yt.dtype != xt.dtype:
            raise ValueError("y must match x in shape and dtype")
    nrhs = xt.shape[1]
    with torch.cuda.device(device):
        rc = lib.sgb_bta_symv(ctypes.byref(m), _ptr(xt), max(nrhs, 1), _ptr(yt), max(nrhs, 1), nrhs, float(alpha),
                              float(beta), _stream(device))
        _lib.raise_for(rc, "bta_matvec")
        if y is not None:
            _finish(w)
            return y
    return yt.view(-1) if squeeze else yt


def pobtas_refine(A_diagonal_blocks, A_lower_diagonal_blocks, A_lower_arrow_blocks, A_arrow_tip_block,
                  L_diagonal_blocks, L_lower_diagonal_blocks, L_lower_arrow_blocks, L_arrow_tip_block, B,
                  iters: int = 2):
    """``B <- A^{-1} B`` in place: the solve with the factor ``L`` of ``A``
    followed by ``iters`` steps of iterative refinement against ``A`` (the
    original matrix, before ``pobtaf`` overwrote its copy).  Real dtypes."""
    if not 0 <= int(iters) <= 100:
        raise ValueError(f"iters must be in 0..100, got {iters}")
    lib = _lib.load()
    device, w = _prepare(
        (A_diagonal_blocks, A_lower_diagonal_blocks, A_lower_arrow_blocks, A_arrow_tip_block,
         L_diagonal_blocks, L_lower_diagonal_blocks, L_lower_arrow_blocks, L_arrow_tip_block, B),
        ("A_diagonal_blocks", "A_lower_diagonal_blocks", "A_lower_arrow_blocks", "A_arrow_tip_block",
         "L_diagonal_blocks", "L_lower_diagonal_blocks", "L_lower_arrow_blocks", "L_arrow_tip_block", "B"))
    mA = _bta_struct(*(t.t for t in w[:4]))
    mL = _bta_struct(*(t.t for t in w[4:8]))
    if (mA.n, mA.b, mA.a, mA.dtype) != (mL.n, mL.b, mL.a, mL.dtype):
        raise ValueError("A and L must have the same block structure and dtype")
    Bt = w[8].t
    Bt = Bt.view(-1, 1) if Bt.dim() == 1 else Bt
    N = mL.n * mL.b + mL.a
    if Bt.dim() != 2 or Bt.shape[0] != N:
        raise ValueError(f"B must have shape ({N}, nrhs), got {tuple(w[8].t.shape)}")
    if Bt.dtype != w[0].t.dtype:
        raise TypeError(f"B has dtype {Bt.dtype}, the blocks have {w[0].t.dtype}")
    nrhs = Bt.shape[1]
    with torch.cuda.device(device):
        nbytes = ctypes.c_size_t(0)
        _lib.raise_for(lib.sgb_pobtas_refine_workspace_size(ctypes.byref(mL), nrhs, ctypes.byref(nbytes)),
                       "pobtas_refine")
        ws = _workspace(nbytes.value, device)
        rc = lib.sgb_pobtas_refine(ctypes.byref(mA), ctypes.byref(mL), _ptr(Bt), nrhs, max(nrhs, 1), int(iters),
                                   ws.data_ptr(), nbytes.value, _stream(device))
        _lib.raise_for(rc, "pobtas_refine")
        _finish(w)
