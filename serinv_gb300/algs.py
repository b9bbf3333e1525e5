"""Drop-in ``pobtaf`` / ``pobtasi`` / ``pobtas`` running on the GB300 kernels.

Same names, positional arguments, keyword arguments, in-place semantics and
exception types as the reference's sequential functions:

* ``pobtaf``  — src/serinv/algs/pobtaf.py:11-94
* ``pobtasi`` — src/serinv/algs/pobtasi.py:10-89
* ``pobtas``  — src/serinv/algs/pobtas.py:10-62
* ``pobtf`` / ``pobtsi`` / ``pobts`` — src/serinv/algs/pobtf.py, pobtsi.py,
  pobts.py (the same calls with an empty arrow stack)

``buffer=`` selects the permuted middle-partition forms (either precision).
float64, float32, complex128 and complex64 stacks are accepted; complex
matrices are Hermitian and run through their real embedding.

Arrays may be torch tensors (CUDA or CPU), NumPy arrays, or any CUDA array
exporting ``__dlpack__`` (CuPy).  Device arrays are used in place on the
current torch stream; host arrays are copied to the GPU, processed, and
copied back in place.  Pinned host stacks (pobtaf, pobtasi) stream: the
blocks travel up in sweep order and back as soon as they are final,
overlapped with the computation, with a device copy of the whole matrix as
the working set.  ``device_streaming=True`` on host arrays (the reference's
streaming mode) instead keeps only a ring of blocks on the device, so the
matrix may exceed device memory; on device arrays it raises
NotImplementedError, as the reference does.  All arithmetic runs in
``libserinv_gb300.so``; if it cannot be loaded or no GPU is present, the
call raises — there is no CPU fallback.

Extensions (keyword-only, absent from the reference): ``precision`` —
``"fp64"`` (default, arithmetic in the storage type), ``"mixed"`` (FP64
storage, block products as exact bf16 slice products on the tensor cores,
6 slices), ``"mixed:S"`` (S slices, 3..7; S=7 is FP64-accurate) or
``"mixed:S:Si"`` (Si slices for the products with an explicit triangular
inverse, whose error grows with the conditioning); ``check_spd`` (pobtaf,
default True) — synchronise and raise ``numpy.linalg.LinAlgError`` on a
non-positive pivot, like SciPy's ``cholesky`` in the reference, and raise
on a device wait that timed out (with False neither is checked and the call
does not synchronise); ``ring_blocks`` (with ``device_streaming``) — blocks
held on the device (default 4 for pobtaf, 32 for pobtasi).
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib

_POBTAF_KW = {"device_streaming", "buffer", "factorize_last_block"}   # pobtaf.py:50
_POBTASI_KW = {"device_streaming", "buffer", "invert_last_block"}     # pobtasi.py:45
_EXTENSION_KW = {"precision", "check_spd", "ring_blocks"}
_STREAM_HOST_ONLY = "Host<->Device streaming only works when host-arrays are given."  # pobtaf.py:293-296


# --------------------------------------------------------------------------
# array plumbing


class _Arr:
    """A CUDA, C-contiguous torch view of a user array plus its write-back."""

    __slots__ = ("t", "src", "kind")

    def __init__(self, t: torch.Tensor, src, kind: str):
        self.t = t
        self.src = src
        self.kind = kind  # "dev" (shared storage), "devcopy", "torch_host", "numpy"

    def writeback(self) -> None:
        if self.kind == "devcopy":
            self.src.copy_(self.t)
        elif self.kind == "torch_host":
            # straight into the caller's memory (one DMA when it is pinned);
            # the caller's stream is synchronized before returning
            self.src.copy_(self.t, non_blocking=True)
        elif self.kind == "numpy":
            if self.src.flags.c_contiguous:
                torch.from_numpy(self.src).copy_(self.t.view(self.src.shape), non_blocking=True)
            else:
                host = self.t.to("cpu").numpy()
                np.copyto(self.src, host.reshape(self.src.shape), casting="no")


def _device_of(arrs) -> torch.device:
    for x in arrs:
        if isinstance(x, torch.Tensor) and x.is_cuda:
            return x.device
    if not torch.cuda.is_available():
        raise RuntimeError("serinv_gb300 needs a CUDA GPU; none is available (no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def _wrap(x, device: torch.device, name: str) -> _Arr:
    if isinstance(x, torch.Tensor):
        if x.is_cuda:
            if x.device != device:
                raise ValueError(f"{name} is on {x.device}, expected {device}")
            if x.is_conj() or x.is_neg():
                # lazily conjugated / negated views: materialise, write back through the view
                return _Arr(x.resolve_conj().resolve_neg().contiguous(), x, "devcopy")
            if x.is_contiguous():
                return _Arr(x, x, "dev")
            return _Arr(x.contiguous(), x, "devcopy")
        # asynchronous from pinned memory, ordered before the library's
        # kernels on the same stream
        return _Arr(x.resolve_conj().resolve_neg().to(device, non_blocking=True).contiguous(), x, "torch_host")
    if isinstance(x, np.ndarray):
        if not x.flags.writeable:
            raise ValueError(f"{name} is read-only; the computation is in place")
        return _Arr(torch.from_numpy(np.ascontiguousarray(x)).to(device, non_blocking=True), x, "numpy")
    if hasattr(x, "__dlpack__"):
        t = torch.from_dlpack(x)
        if not t.is_cuda:
            return _Arr(t.to(device).contiguous(), t, "torch_host")
        if t.device != device:
            raise ValueError(f"{name} is on {t.device}, expected {device}")
        if t.is_contiguous():
            return _Arr(t, t, "dev")
        return _Arr(t.contiguous(), t, "devcopy")
    raise TypeError(f"{name}: unsupported array type {type(x).__name__}")


def _dtype_code(dt: torch.dtype) -> int:
    if dt == torch.float64:
        return _lib.SGB_F64
    if dt == torch.float32:
        return _lib.SGB_F32
    if dt == torch.complex128:
        return _lib.SGB_C128
    if dt == torch.complex64:
        return _lib.SGB_C64
    raise TypeError(f"unsupported dtype {dt}")


def _ptr(t: torch.Tensor):
    return t.data_ptr() if t.numel() > 0 else None


def _bta_struct(D, Lo, Ar, T):
    """Validate the four stacks and build the C descriptor."""
    if D.dim() != 3 or D.shape[1] != D.shape[2]:
        raise ValueError(f"diagonal blocks must have shape (n, b, b), got {tuple(D.shape)}")
    n, b = D.shape[0], D.shape[1]
    if Ar.dim() != 3 or Ar.shape[0] != n or Ar.shape[2] != b:
        raise ValueError(f"arrow blocks must have shape (n, a, b) = ({n}, a, {b}), got {tuple(Ar.shape)}")
    a = Ar.shape[1]
    if Lo.dim() != 3 or tuple(Lo.shape) != (n - 1, b, b):
        raise ValueError(f"lower blocks must have shape ({n - 1}, {b}, {b}), got {tuple(Lo.shape)}")
    if tuple(T.shape) != (a, a):
        raise ValueError(f"arrow tip must have shape ({a}, {a}), got {tuple(T.shape)}")
    if n < 1 or b < 1:
        raise ValueError("need at least one diagonal block of size >= 1")
    dts = {D.dtype, Lo.dtype, Ar.dtype, T.dtype}
    if len(dts) != 1:
        raise TypeError(f"all blocks must share one dtype, got {sorted(map(str, dts))}")
    m = _lib.SgbBta()
    m.dtype = _dtype_code(D.dtype)
    m.n, m.b, m.a = n, b, a
    m.diag, m.lower, m.arrow, m.tip = _ptr(D), _ptr(Lo), _ptr(Ar), _ptr(T)
    return m


def _precision(kwargs) -> int:
    return _lib.precision_code(kwargs.get("precision", "fp64"))


def _workspace(nbytes: int, device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device)


def _check_status(ws: torch.Tensor, precision: int, what: str, always: bool = False) -> None:
    """The workspace's first int32 is the device status word (bounded waits)."""
    if not always and (precision & 0xFF) != _lib.SGB_PREC_MIXED:
        return
    code = int(ws[:4].view(torch.int32).item())
    _lib.raise_for(code, what)


def _copy_back(t: torch.Tensor, x) -> None:
    """Write a contiguous host copy back into the caller's array or tensor."""
    if isinstance(x, np.ndarray):
        np.copyto(x, t.numpy(), casting="no")
    else:
        x.copy_(t)


def _stream(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _prepare(arrays, names):
    device = _device_of(arrays)
    wrapped = [_wrap(x, device, nm) for x, nm in zip(arrays, names)]
    return device, wrapped


def _finish(wrapped) -> None:
    host = any(w.kind in ("numpy", "torch_host") for w in wrapped)
    for w in wrapped:
        w.writeback()
    if host:
        torch.cuda.current_stream(wrapped[0].t.device).synchronize()


def _pinned_host_stacks(arrays):
    """The stacks as C-contiguous pinned host tensors sharing the callers'
    memory (real dtype), or None when any of them is not one."""
    out = []
    for x in arrays:
        if isinstance(x, np.ndarray):
            if not (x.flags.c_contiguous and x.flags.writeable):
                return None
            t = torch.from_numpy(x)
        elif isinstance(x, torch.Tensor) and not x.is_cuda:
            if not x.is_contiguous() or x.is_conj() or x.is_neg():
                return None
            t = x
        else:
            return None
        if t.numel() and not t.is_pinned():
            return None
        out.append(t)
    if len({t.dtype for t in out}) != 1 or out[0].dtype not in (torch.float64, torch.float32):
        return None
    return out


def _streamed_host_stacks(arrays):
    """The stacks as C-contiguous real host tensors for the streamed ring
    (sharing the caller's memory where the layout allows, else copies to
    write back), or raise like the reference when any is a device array.
    Returns (tensors, writebacks) or None for complex stacks."""
    out, back = [], []
    for x in arrays:
        if isinstance(x, np.ndarray):
            if not x.flags.writeable:
                raise ValueError("the stacks are read-only; the computation is in place")
            t = torch.from_numpy(x) if x.flags.c_contiguous else torch.from_numpy(np.ascontiguousarray(x))
            if not x.flags.c_contiguous:
                back.append((t, x))
        elif isinstance(x, torch.Tensor) and not x.is_cuda:
            t = x.resolve_conj().resolve_neg()
            if not t.is_contiguous() or t is not x:
                t = t.contiguous()
                back.append((t, x))
        else:
            raise NotImplementedError(_STREAM_HOST_ONLY)
        out.append(t)
    if len({t.dtype for t in out}) != 1:
        raise TypeError(f"all blocks must share one dtype, got {sorted(str(t.dtype) for t in out)}")
    if out[0].dtype not in (torch.float64, torch.float32):
        return None
    return out, back


def _stream_call(entry, size_query, host, what, precision, flag, ring, with_info):
    """Streamed ring over host stacks (the C entry `entry`): only `ring`
    blocks and the tip are on the device; returns once the host arrays hold
    the result."""
    lib = _lib.load()
    device = torch.device("cuda", torch.cuda.current_device())
    mh = _bta_struct(*host)
    with torch.cuda.device(device):
        nbytes = ctypes.c_size_t(0)
        _lib.raise_for(size_query(ctypes.byref(mh), precision, int(ring), ctypes.byref(nbytes)), what)
        ws = _workspace(nbytes.value, device)
        args = [ctypes.byref(mh), int(flag), precision, int(ring), ws.data_ptr(), nbytes.value]
        info = torch.zeros(1, dtype=torch.int32, device=device) if with_info else None
        if with_info:
            args.append(info.data_ptr())
        args.append(_stream(device))
        _lib.raise_for(entry(*args), what)
        torch.cuda.current_stream(device).synchronize()
    return ws, info


def _host_call(entry, size_query, host, what, precision, flag, with_info):
    """Pinned host stacks: a device copy of the same shape is the working
    set, blocks travel up and back overlapped with the sweep (the C entry
    `entry`), and the call returns once the host arrays hold the result."""
    lib = _lib.load()
    device = torch.device("cuda", torch.cuda.current_device())
    dev = [torch.empty(t.shape, dtype=t.dtype, device=device) for t in host]
    mh = _bta_struct(*host)
    md = _bta_struct(*dev)
    with torch.cuda.device(device):
        nbytes = ctypes.c_size_t(0)
        _lib.raise_for(size_query(ctypes.byref(md), precision, ctypes.byref(nbytes)), what)
        ws = _workspace(nbytes.value, device)
        args = [ctypes.byref(mh), ctypes.byref(md), int(flag), precision, ws.data_ptr(), nbytes.value]
        info = torch.zeros(1, dtype=torch.int32, device=device) if with_info else None
        if with_info:
            args.append(info.data_ptr())
        args.append(_stream(device))
        _lib.raise_for(entry(*args), what)
        torch.cuda.current_stream(device).synchronize()
    return ws, info


# --------------------------------------------------------------------------
# public API


def pobtaf(A_diagonal_blocks, A_lower_diagonal_blocks, A_lower_arrow_blocks, A_arrow_tip_block, **kwargs):
    """Cholesky factorization of a block tridiagonal with arrowhead SPD matrix, in place.

    Mirrors src/serinv/algs/pobtaf.py:11-94.  Keyword arguments:
    ``device_streaming`` (host arrays stream through a ring of device
    blocks, pobtaf.py:284-524, so matrices larger than device memory work;
    device arrays raise NotImplementedError, pobtaf.py:293-296),
    ``buffer`` (an (n, b, b) array: the permuted middle-partition
    elimination of pobtaf.py:186-281),
    ``factorize_last_block`` (default True).  Unknown keywords raise
    TypeError (pobtaf.py:50-53).
    """
    unexpected = set(kwargs) - _POBTAF_KW - _EXTENSION_KW
    if unexpected:
        raise TypeError(f"Unexpected keyword arguments: {unexpected}")
    if kwargs.get("buffer", None) is not None:
        return _pobtaf_permuted(A_diagonal_blocks, A_lower_diagonal_blocks, A_lower_arrow_blocks,
                                A_arrow_tip_block, kwargs["buffer"], kwargs)
    factorize_last_block = bool(kwargs.get("factorize_last_block", True))
    precision = _precision(kwargs)
    check = bool(kwargs.get("check_spd", True))

    arrays = (A_diagonal_blocks, A_lower_diagonal_blocks, A_lower_arrow_blocks, A_arrow_tip_block)
    _device_of(arrays)  # no GPU: fail loudly before touching the arrays
    if kwargs.get("device_streaming", False):
        st = _streamed_host_stacks(arrays)
        if st is not None:
            lib = _lib.load()
            hs, back = st
            ws, info = _stream_call(lib.sgb_pobtaf_stream, lib.sgb_pobtaf_stream_workspace_size, hs, "pobtaf",
                                    precision, factorize_last_block, kwargs.get("ring_blocks", 0), True)
            for t, x in back:
                _copy_back(t, x)
            _check_status(ws, precision, "pobtaf", always=check)
            if check:
                k = int(info.item())
                if k > 0:
                    raise np.linalg.LinAlgError(f"{k}-th leading minor of the array is not positive definite")
            return
    host = _pinned_host_stacks(arrays)
    if host is not None:
        lib = _lib.load()
        ws, info = _host_call(lib.sgb_pobtaf_host, lib.sgb_pobtaf_workspace_size, host, "pobtaf", precision,
                              factorize_last_block, True)
        _check_status(ws, precision, "pobtaf", always=check)
        if check:
            k = int(info.item())
            if k > 0:
                raise np.linalg.LinAlgError(f"{k}-th leading minor of the array is not positive definite")
        return

    lib = _lib.load()
    device, w = _prepare(
        (A_diagonal_blocks, A_lower_diagonal_blocks, A_lower_arrow_blocks, A_arrow_tip_block),
        ("A_diagonal_blocks", "A_lower_diagonal_blocks", "A_lower_arrow_blocks", "A_arrow_tip_block"))
    m = _bta_struct(*(x.t for x in w))
    with torch.cuda.device(device):
        nbytes = ctypes.c_size_t(0)
        _lib.raise_for(lib.sgb_pobtaf_workspace_size(ctypes.byref(m), precision, ctypes.byref(nbytes)),
                       "pobtaf")
        ws = _workspace(nbytes.value, device)
        info = torch.zeros(1, dtype=torch.int32, device=device)
        rc = lib.sgb_pobtaf(ctypes.byref(m), int(factorize_last_block), precision, ws.data_ptr(),
                            nbytes.value, info.data_ptr(), _stream(device))
        _lib.raise_for(rc, "pobtaf")
        _finish(w)
        _check_status(ws, precision, "pobtaf", always=check)
        if check:
            k = int(info.item())
            if k > 0:
                raise np.linalg.LinAlgError(f"{k}-th leading minor of the array is not positive definite")


def pobtasi(L_diagonal_blocks, L_lower_diagonal_blocks, L_lower_arrow_blocks, L_arrow_tip_block, **kwargs):
    """Selected inversion of a block tridiagonal with arrowhead matrix from its Cholesky factor, in place.

    Mirrors src/serinv/algs/pobtasi.py:10-89.  Keyword arguments:
    ``device_streaming`` (host arrays stream through a ring of device blocks,
    pobtasi.py:247-496; device arrays raise NotImplementedError), ``buffer``
    (the permuted variant of
    pobtasi.py:175-244), ``invert_last_block``
    (default True).  Unknown keywords raise TypeError (pobtasi.py:45-48).
    """
    unexpected = set(kwargs) - _POBTASI_KW - _EXTENSION_KW
    if unexpected:
        raise TypeError(f"Unexpected keyword arguments: {unexpected}")
    if kwargs.get("buffer", None) is not None:
        return _pobtasi_permuted(L_diagonal_blocks, L_lower_diagonal_blocks, L_lower_arrow_blocks,
                                 L_arrow_tip_block, kwargs["buffer"], kwargs)
    invert_last_block = bool(kwargs.get("invert_last_block", True))
    precision = _precision(kwargs)

    arrays = (L_diagonal_blocks, L_lower_diagonal_blocks, L_lower_arrow_blocks, L_arrow_tip_block)
    _device_of(arrays)
    if kwargs.get("device_streaming", False):
        st = _streamed_host_stacks(arrays)
        if st is not None:
            lib = _lib.load()
            hs, back = st
            ws, _ = _stream_call(lib.sgb_pobtasi_stream, lib.sgb_pobtasi_stream_workspace_size, hs, "pobtasi",
                                 precision, invert_last_block, kwargs.get("ring_blocks", 0), False)
            for t, x in back:
                _copy_back(t, x)
            _check_status(ws, precision, "pobtasi")
            return
    host = _pinned_host_stacks(arrays)
    if host is not None:
        lib = _lib.load()
        ws, _ = _host_call(lib.sgb_pobtasi_host, lib.sgb_pobtasi_workspace_size, host, "pobtasi", precision,
                           invert_last_block, False)
        _check_status(ws, precision, "pobtasi")
        return

    lib = _lib.load()
    device, w = _prepare(
        (L_diagonal_blocks, L_lower_diagonal_blocks, L_lower_arrow_blocks, L_arrow_tip_block),
        ("L_diagonal_blocks", "L_lower_diagonal_blocks", "L_lower_arrow_blocks", "L_arrow_tip_block"))
    m = _bta_struct(*(x.t for x in w))
    with torch.cuda.device(device):
        nbytes = ctypes.c_size_t(0)
        _lib.raise_for(lib.sgb_pobtasi_workspace_size(ctypes.byref(m), precision, ctypes.byref(nbytes)),
                       "pobtasi")
        ws = _workspace(nbytes.value, device)
        rc = lib.sgb_pobtasi(ctypes.byref(m), int(invert_last_block), precision, ws.data_ptr(), nbytes.value,
                             _stream(device))
        _lib.raise_for(rc, "pobtasi")
        _finish(w)
        _check_status(ws, precision, "pobtasi")


def pobtas(L_diagonal_blocks, L_lower_diagonal_blocks, L_lower_arrow_blocks, L_arrow_tip_block, B, trans="N",
           **kwargs):
    """Triangular solve with the Cholesky factor of a BTA matrix, in place on ``B``.

    Mirrors src/serinv/algs/pobtas.py:10-62: ``trans="N"`` computes
    ``B <- L^{-1} B``, ``"T"``/``"C"`` computes ``B <- L^{-T} B``, anything
    else raises ValueError (pobtas.py:160-161).  ``partial=True`` skips the
    last diagonal block and the tip.  ``buffer`` selects the permuted solve
    of pobtas.py:164-218 (storage precision).  ``device_streaming``
    raises NotImplementedError (pobtas.py:33-36,49-52).  Like the reference,
    unknown keywords are ignored.  For arrow width 0 the call is the
    arrow-free solve of src/serinv/algs/pobts.py:57-118 (the reference's
    pobtas fails there).
    """
    buffer = kwargs.get("buffer", None)
    if kwargs.get("device_streaming", False):
        what = "natural" if buffer is None else "permuted"
        raise NotImplementedError(f"Streaming is not implemented for the {what} arrowhead.")
    if trans not in ("N", "T", "C"):
        raise ValueError(f"Invalid transpose argument: {trans}.")
    if buffer is not None:
        return _pobtas_permuted(L_diagonal_blocks, L_lower_diagonal_blocks, L_lower_arrow_blocks,
                                L_arrow_tip_block, B, buffer, trans, kwargs)
    partial = bool(kwargs.get("partial", False))
    precision = _precision(kwargs)

    lib = _lib.load()
    device, w = _prepare(
        (L_diagonal_blocks, L_lower_diagonal_blocks, L_lower_arrow_blocks, L_arrow_tip_block, B),
        ("L_diagonal_blocks", "L_lower_diagonal_blocks", "L_lower_arrow_blocks", "L_arrow_tip_block", "B"))
    m = _bta_struct(*(x.t for x in w[:4]))
    Bt = w[4].t
    squeeze = Bt.dim() == 1
    if squeeze:
        Bt = Bt.view(-1, 1)
    N = m.n * m.b + m.a
    if Bt.dim() != 2 or Bt.shape[0] != N:
        raise ValueError(f"B must have shape ({N}, nrhs), got {tuple(w[4].t.shape)}")
    if Bt.dtype != w[0].t.dtype:
        raise TypeError(f"B has dtype {Bt.dtype}, the factor has {w[0].t.dtype}")
    nrhs = Bt.shape[1]
    with torch.cuda.device(device):
        nbytes = ctypes.c_size_t(0)
        _lib.raise_for(lib.sgb_pobtas_workspace_size(ctypes.byref(m), nrhs, precision, ctypes.byref(nbytes)),
                       "pobtas")
        ws = _workspace(nbytes.value, device)
        rc = lib.sgb_pobtas(ctypes.byref(m), _ptr(Bt), nrhs, max(nrhs, 1), trans.encode(), int(partial),
                            precision, ws.data_ptr(), nbytes.value, _stream(device))
        _lib.raise_for(rc, "pobtas")
        _finish(w)


# --------------------------------------------------------------------------
# permuted (middle-partition) forms: the ``buffer=`` keyword


def _check_buffer(buf: torch.Tensor, D: torch.Tensor) -> None:
    n, b = D.shape[0], D.shape[1]
    if tuple(buf.shape) != (n, b, b):
        raise ValueError(f"buffer must have shape {(n, b, b)}, got {tuple(buf.shape)}")
    if buf.dtype != D.dtype:
        raise TypeError(f"buffer has dtype {buf.dtype}, the blocks have {D.dtype}")


def _pobtaf_permuted(D, Lo, Ar, T, buffer, kwargs):
    """pobtaf(..., buffer=): src/serinv/algs/pobtaf.py:186-281."""
    precision = _precision(kwargs)
    check = bool(kwargs.get("check_spd", True))
    lib = _lib.load()
    device, w = _prepare((D, Lo, Ar, T, buffer),
                         ("A_diagonal_blocks", "A_lower_diagonal_blocks", "A_lower_arrow_blocks",
                          "A_arrow_tip_block", "buffer"))
    _check_buffer(w[4].t, w[0].t)
    m = _bta_struct(*(x.t for x in w[:4]))
    with torch.cuda.device(device):
        nbytes = ctypes.c_size_t(0)
        _lib.raise_for(lib.sgb_pobtaf_permuted_workspace_size(ctypes.byref(m), precision, ctypes.byref(nbytes)),
                       "pobtaf")
        ws = _workspace(nbytes.value, device)
        info = torch.zeros(1, dtype=torch.int32, device=device)
        rc = lib.sgb_pobtaf_permuted(ctypes.byref(m), _ptr(w[4].t), precision, ws.data_ptr(), nbytes.value,
                                     info.data_ptr(), _stream(device))
        _lib.raise_for(rc, "pobtaf")
        _finish(w)
        _check_status(ws, precision, "pobtaf", always=check)
        if check:
            k = int(info.item())
            if k > 0:
                raise np.linalg.LinAlgError(f"{k}-th leading minor of the array is not positive definite")


def _pobtasi_permuted(D, Lo, Ar, T, buffer, kwargs):
    """pobtasi(..., buffer=): src/serinv/algs/pobtasi.py:175-244."""
    precision = _precision(kwargs)
    lib = _lib.load()
    device, w = _prepare((D, Lo, Ar, T, buffer),
                         ("L_diagonal_blocks", "L_lower_diagonal_blocks", "L_lower_arrow_blocks",
                          "L_arrow_tip_block", "buffer"))
    _check_buffer(w[4].t, w[0].t)
    m = _bta_struct(*(x.t for x in w[:4]))
    with torch.cuda.device(device):
        nbytes = ctypes.c_size_t(0)
        _lib.raise_for(lib.sgb_pobtasi_permuted_workspace_size(ctypes.byref(m), precision, ctypes.byref(nbytes)),
                       "pobtasi")
        ws = _workspace(nbytes.value, device)
        rc = lib.sgb_pobtasi_permuted(ctypes.byref(m), _ptr(w[4].t), precision, ws.data_ptr(), nbytes.value,
                                      _stream(device))
        _lib.raise_for(rc, "pobtasi")
        _finish(w)
        _check_status(ws, precision, "pobtasi")


def _pobtas_permuted(D, Lo, Ar, T, B, buffer, trans, kwargs):
    """pobtas(..., buffer=): src/serinv/algs/pobtas.py:164-218 (storage precision in either mode)."""
    precision = _precision(kwargs)
    lib = _lib.load()
    device, w = _prepare((D, Lo, Ar, T, B, buffer),
                         ("L_diagonal_blocks", "L_lower_diagonal_blocks", "L_lower_arrow_blocks",
                          "L_arrow_tip_block", "B", "buffer"))
    _check_buffer(w[5].t, w[0].t)
    m = _bta_struct(*(x.t for x in w[:4]))
    Bt = w[4].t
    if Bt.dim() == 1:
        Bt = Bt.view(-1, 1)
    N = m.n * m.b + m.a
    if Bt.dim() != 2 or Bt.shape[0] != N:
        raise ValueError(f"B must have shape ({N}, nrhs), got {tuple(w[4].t.shape)}")
    if Bt.dtype != w[0].t.dtype:
        raise TypeError(f"B has dtype {Bt.dtype}, the factor has {w[0].t.dtype}")
    nrhs = Bt.shape[1]
    with torch.cuda.device(device):
        nbytes = ctypes.c_size_t(0)
        _lib.raise_for(lib.sgb_pobtas_permuted_workspace_size(ctypes.byref(m), nrhs, precision,
                                                              ctypes.byref(nbytes)), "pobtas")
        ws = _workspace(nbytes.value, device)
        rc = lib.sgb_pobtas_permuted(ctypes.byref(m), _ptr(w[5].t), _ptr(Bt), nrhs, max(nrhs, 1), trans.encode(),
                                     precision, ws.data_ptr(), nbytes.value, _stream(device))
        _lib.raise_for(rc, "pobtas")
        _finish(w)


# --------------------------------------------------------------------------
# block tridiagonal (no arrowhead) family: the same kernels with a = 0


def _empty_arrow(D):
    """Arrow stack (n, 0, b) and tip (0, 0) of D's kind, dtype and device."""
    if isinstance(D, np.ndarray):
        return (np.empty((D.shape[0], 0, D.shape[2]), dtype=D.dtype), np.empty((0, 0), dtype=D.dtype))
    t = D if isinstance(D, torch.Tensor) else torch.from_dlpack(D)
    return (torch.empty((t.shape[0], 0, t.shape[2]), dtype=t.dtype, device=t.device),
            torch.empty((0, 0), dtype=t.dtype, device=t.device))


def pobtf(A_diagonal_blocks, A_lower_diagonal_blocks, **kwargs):
    """Cholesky factorization of a block tridiagonal SPD matrix, in place.

    Mirrors src/serinv/algs/pobtf.py:11-80 (kwargs ``device_streaming``,
    ``buffer`` -- the permuted form, _pobtf_permuted pobtf.py:125-185 --,
    ``factorize_last_block``; unknown keywords raise TypeError, pobtf.py:
    44-47).  Computes what pobtaf computes with an empty arrowhead.
    """
    unexpected = set(kwargs) - _POBTAF_KW - _EXTENSION_KW
    if unexpected:
        raise TypeError(f"Unexpected keyword arguments: {unexpected}")
    Ar, T = _empty_arrow(A_diagonal_blocks)
    pobtaf(A_diagonal_blocks, A_lower_diagonal_blocks, Ar, T, **kwargs)


def pobtsi(L_diagonal_blocks, L_lower_diagonal_blocks, **kwargs):
    """Selected inversion of a block tridiagonal matrix from its Cholesky factor, in place.

    Mirrors src/serinv/algs/pobtsi.py:10-75 (kwargs ``device_streaming``,
    ``buffer`` -- _pobtsi_permuted, pobtsi.py:128-179 --,
    ``invert_last_block``; unknown keywords raise TypeError, pobtsi.py:
    39-42).
    """
    unexpected = set(kwargs) - _POBTASI_KW - _EXTENSION_KW
    if unexpected:
        raise TypeError(f"Unexpected keyword arguments: {unexpected}")
    Ar, T = _empty_arrow(L_diagonal_blocks)
    pobtasi(L_diagonal_blocks, L_lower_diagonal_blocks, Ar, T, **kwargs)


def pobts(L_diagonal_blocks, L_lower_diagonal_blocks, B, trans="N", **kwargs):
    """Triangular solve with the Cholesky factor of a block tridiagonal matrix, in place on ``B``.

    Mirrors src/serinv/algs/pobts.py:10-55 (``trans`` "N", "T" or "C";
    ``partial``; ``buffer`` -- _pobts_permuted, pobts.py:121-165 --;
    ``device_streaming`` raises NotImplementedError; unknown keywords are
    ignored, as there).
    """
    if kwargs.get("device_streaming", False):
        what = "Permuted arrowhead is not implemented." if kwargs.get("buffer", None) is not None else \
            "Streaming is not implemented for the natural arrowhead."
        raise NotImplementedError(what)
    Ar, T = _empty_arrow(L_diagonal_blocks)
    pobtas(L_diagonal_blocks, L_lower_diagonal_blocks, Ar, T, B, trans=trans, **kwargs)
