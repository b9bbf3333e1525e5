"""Dense FP64 product through the library's engines (``sgb_dgemm``).

``dgemm(A, B, C=None, alpha=1, beta=0, transA=False, transB=False,
precision="fp64")`` computes ``C <- alpha op(A) op(B) + beta C`` on torch
CUDA float64 tensors (row-major, contiguous) with the FP64 pipe
(``"fp64"``) or the tensor-core slice products (``"mixed"`` / ``"mixed:S"``).
It is the block product every step of the BTA sweeps is built from, exposed
for testing and for callers that want the tensor-core FP64 product alone.
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib


def dgemm(A: torch.Tensor, B: torch.Tensor, C: torch.Tensor | None = None, alpha: float = 1.0,
          beta: float = 0.0, transA: bool = False, transB: bool = False, precision="fp64") -> torch.Tensor:
    lib = _lib.load()
    for t in (A, B) + ((C,) if C is not None else ()):
        if not (t.is_cuda and t.dtype == torch.float64 and t.dim() == 2 and t.is_contiguous()):
            raise TypeError("dgemm takes contiguous 2-D float64 CUDA tensors")
    M, K = (A.shape[1], A.shape[0]) if transA else (A.shape[0], A.shape[1])
    K2, N = (B.shape[1], B.shape[0]) if transB else (B.shape[0], B.shape[1])
    if K != K2:
        raise ValueError(f"inner dimensions differ: {K} vs {K2}")
    if C is None:
        C = torch.zeros((M, N), dtype=torch.float64, device=A.device)
        beta = 0.0
    if tuple(C.shape) != (M, N):
        raise ValueError(f"C must be {M}x{N}")
    prec = _lib.precision_code(precision)
    nbytes = ctypes.c_size_t(0)
    _lib.raise_for(lib.sgb_dgemm_workspace_size(prec, M, N, K, ctypes.byref(nbytes)), "dgemm")
    ws = torch.empty(nbytes.value, dtype=torch.uint8, device=A.device)
    with torch.cuda.device(A.device):
        rc = lib.sgb_dgemm(prec, b"T" if transA else b"N", b"T" if transB else b"N", M, N, K, float(alpha),
                           A.data_ptr() if A.numel() else None, A.shape[1] if A.shape[1] else 1,
                           B.data_ptr() if B.numel() else None, B.shape[1] if B.shape[1] else 1,
                           float(beta), C.data_ptr(), max(N, 1), ws.data_ptr(), nbytes.value,
                           torch.cuda.current_stream(A.device).cuda_stream)
        _lib.raise_for(rc, "dgemm")
        if (prec & 0xFF) == _lib.SGB_PREC_MIXED:
            _lib.raise_for(int(ws[:4].view(torch.int32).item()), "dgemm")
    return C
