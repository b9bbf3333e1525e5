"""ctypes binding of ``libserinv_gb300.so`` (the C ABI in include/serinv_gb300.h).

The library is built in-tree by ``serinv_gb300.build``.  Loading fails loudly
when it is missing: there is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import build as _build

SGB_OK = 0
SGB_ERR_SHAPE = 1
SGB_ERR_DTYPE = 2
SGB_ERR_NOT_SPD = 3
SGB_ERR_TIMEOUT = 4
SGB_ERR_CUDA = 5
SGB_ERR_WORKSPACE = 6
SGB_ERR_ARG = 7
SGB_ERR_UNSUPPORTED = 8

SGB_F32 = 0
SGB_F64 = 1
SGB_C64 = 2
SGB_C128 = 3

SGB_BATCH_TC_KSPLIT = 1

SGB_PREC_NATIVE = 0
SGB_PREC_MIXED = 1

PRECISIONS = {"native": SGB_PREC_NATIVE, "fp64": SGB_PREC_NATIVE, "mixed": SGB_PREC_MIXED}


def precision_code(precision) -> int:
    """'fp64' / 'native' -> native; 'mixed' -> 6 slices; 'mixed:S' -> S slices
    (3..7); 'mixed:S:Si' -> S slices, and Si for the products with an
    explicit triangular inverse (the accuracy lever at ill conditioning)."""
    if isinstance(precision, str) and precision.startswith("mixed:"):
        parts = precision.split(":")[1:]
        if not 1 <= len(parts) <= 2:
            raise ValueError(f"precision must be 'mixed:S' or 'mixed:S:Si', got {precision!r}")
        counts = [int(x) for x in parts]
        for c in counts:
            if not 3 <= c <= 7:
                raise ValueError(f"slice count must be in 3..7, got {c}")
        code = SGB_PREC_MIXED | (counts[0] << 8)
        if len(counts) == 2:
            code |= counts[1] << 16
        return code
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be 'fp64', 'mixed' or 'mixed:S', got {precision!r}")
    return PRECISIONS[precision]


class SgbBta(ctypes.Structure):
    _fields_ = [
        ("dtype", ctypes.c_int32),
        ("_pad", ctypes.c_int32),
        ("n", ctypes.c_int64),
        ("b", ctypes.c_int64),
        ("a", ctypes.c_int64),
        ("diag", ctypes.c_void_p),
        ("lower", ctypes.c_void_p),
        ("arrow", ctypes.c_void_p),
        ("tip", ctypes.c_void_p),
    ]


# name -> (restype, argtypes)
_SIGNATURES = {
    "sgb_version": (ctypes.c_int, []),
    "sgb_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "sgb_last_cuda_error": (ctypes.c_int, []),
    "sgb_pobtaf_workspace_size": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_int,
                                                 ctypes.POINTER(ctypes.c_size_t)]),
    "sgb_pobtasi_workspace_size": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_int,
                                                  ctypes.POINTER(ctypes.c_size_t)]),
    "sgb_pobtas_workspace_size": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_int64, ctypes.c_int,
                                                 ctypes.POINTER(ctypes.c_size_t)]),
    "sgb_pobtaf": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                  ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]),
    "sgb_pobtasi": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                   ctypes.c_size_t, ctypes.c_void_p]),
    "sgb_pobtas": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                  ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                  ctypes.c_size_t, ctypes.c_void_p]),
    "sgb_pobtaf_host": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.POINTER(SgbBta), ctypes.c_int, ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]),
    "sgb_pobtasi_host": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.POINTER(SgbBta), ctypes.c_int, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "sgb_pobtaf_stream_workspace_size": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_int, ctypes.c_int64,
                                                        ctypes.POINTER(ctypes.c_size_t)]),
    "sgb_pobtaf_stream": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_int, ctypes.c_int, ctypes.c_int64,
                                         ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]),
    "sgb_pobtasi_stream_workspace_size": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_int, ctypes.c_int64,
                                                         ctypes.POINTER(ctypes.c_size_t)]),
    "sgb_pobtasi_stream": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_int, ctypes.c_int, ctypes.c_int64,
                                          ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "sgb_pobtaf_permuted": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]),
    "sgb_pobtaf_permuted_workspace_size": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_int,
                                                          ctypes.POINTER(ctypes.c_size_t)]),
    "sgb_pobtasi_permuted_workspace_size": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_int,
                                                           ctypes.POINTER(ctypes.c_size_t)]),
    "sgb_pobtas_permuted_workspace_size": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_int64, ctypes.c_int,
                                                          ctypes.POINTER(ctypes.c_size_t)]),
    "sgb_pobtasi_permuted": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_void_p, ctypes.c_int,
                                            ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "sgb_pobtas_permuted": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_int64, ctypes.c_int64, ctypes.c_char, ctypes.c_int,
                                           ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "sgb_bta_symv": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                    ctypes.c_int64, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_void_p]),
    "sgb_pobtas_refine_workspace_size": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_int64,
                                                        ctypes.POINTER(ctypes.c_size_t)]),
    "sgb_pobtas_refine": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.POINTER(SgbBta), ctypes.c_void_p,
                                         ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p,
                                         ctypes.c_size_t, ctypes.c_void_p]),
    "sgb_bta_logdet_quad_grad": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_void_p, ctypes.c_int64,
                                                ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]),
    "sgb_dgemm_workspace_size": (ctypes.c_int, [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                                ctypes.POINTER(ctypes.c_size_t)]),
    "sgb_dgemm": (ctypes.c_int, [ctypes.c_int, ctypes.c_char, ctypes.c_char, ctypes.c_int64, ctypes.c_int64,
                                 ctypes.c_int64, ctypes.c_double, ctypes.c_void_p, ctypes.c_int64,
                                 ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p,
                                 ctypes.c_int64, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "sgb_pobtaf_noalloc": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.c_int, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    "sgb_pobtaf_noalloc_scratch_bytes": (ctypes.c_size_t, []),
    "sgb_batch_workspace_size": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.POINTER(ctypes.c_void_p),
                                                ctypes.POINTER(ctypes.c_int64), ctypes.c_int, ctypes.c_int,
                                                ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                                ctypes.POINTER(ctypes.c_size_t)]),
    "sgb_batch_plan_create": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.POINTER(ctypes.c_void_p),
                                             ctypes.POINTER(ctypes.c_int64), ctypes.c_int, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_void_p,
                                             ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]),
    "sgb_batch_plan_create_ex": (ctypes.c_int, [ctypes.POINTER(SgbBta), ctypes.POINTER(ctypes.c_void_p),
                                                ctypes.POINTER(ctypes.c_int64), ctypes.c_int, ctypes.c_int,
                                                ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t,
                                                ctypes.POINTER(ctypes.c_void_p)]),
    "sgb_batch_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "sgb_batch_info": (ctypes.c_void_p, [ctypes.c_void_p]),
    "sgb_batch_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "sgb_launch_count": (ctypes.c_longlong, []),
    "sgb_debug_spin_limit": (ctypes.c_longlong, [ctypes.c_longlong]),
    "sgb_profile_enable": (ctypes.c_int, [ctypes.c_int]),
    "sgb_profile_enable_classes": (ctypes.c_int, [ctypes.c_uint]),
    "sgb_profile_read": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_longlong),
                                        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "sgb_profile_read_issued": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
}

KCLASS = {"gemm": 0, "potrf_tile": 1, "trtri_tile": 2, "gemm_tc": 3, "split": 4, "panel": 5, "embed": 6}

_lock = threading.Lock()
_lib = None


def lib_path() -> str:
    return _build.LIBPATH


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load the shared library (building it first if it is absent)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"serinv_gb300: {path} is not built")
            _build.build()
        lib = ctypes.CDLL(path)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def exported_symbols():
    return list(_SIGNATURES)


def spin_limit(polls: int = -1) -> int:
    """Poll limit of the bounded device waits; sets it when polls >= 0 and
    returns the previous value (a test hook for the timeout path)."""
    return int(load().sgb_debug_spin_limit(int(polls)))


def launch_count() -> int:
    """Kernels launched by the library since it was loaded."""
    return int(load().sgb_launch_count())


def profile_enable(on: bool, classes=None) -> None:
    """Per-launch event timing: off, all kernel classes, or only `classes` (names of KCLASS)."""
    if classes is None or not on:
        load().sgb_profile_enable(1 if on else 0)
    else:
        load().sgb_profile_enable_classes(sum(1 << KCLASS[c] for c in classes))


def profile_read() -> dict:
    """Per kernel class: launches, device ms, algorithmic flops (synchronises)."""
    lib = load()
    out = {}
    for name, k in KCLASS.items():
        n = ctypes.c_longlong(0)
        ms = ctypes.c_double(0)
        fl = ctypes.c_double(0)
        raise_for(lib.sgb_profile_read(k, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(fl)), "profile")
        if n.value:
            iss = ctypes.c_double(0)
            raise_for(lib.sgb_profile_read_issued(k, ctypes.byref(iss)), "profile")
            out[name] = {"launches": n.value, "ms": ms.value, "flops": fl.value}
            if iss.value:
                out[name]["issued"] = iss.value
    return out


class SgbError(RuntimeError):
    pass


def raise_for(code: int, what: str) -> None:
    """Map a C return code to the exception type the reference would raise."""
    if code == SGB_OK:
        return
    lib = load()
    msg = f"{what}: {lib.sgb_strerror(code).decode()}"
    if code == SGB_ERR_CUDA:
        msg += f" (cudaError {lib.sgb_last_cuda_error()})"
        raise SgbError(msg)
    if code in (SGB_ERR_SHAPE, SGB_ERR_ARG):
        raise ValueError(msg)
    if code == SGB_ERR_DTYPE:
        raise TypeError(msg)
    if code == SGB_ERR_NOT_SPD:
        raise np.linalg.LinAlgError(msg)
    if code == SGB_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise SgbError(msg)
