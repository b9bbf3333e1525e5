"""Batches of independent BTA matrices in one graph launch.

``BatchPlan(mats, rhs=None, ops=("pobtaf", "pobtasi", "pobtas"),
precisions=None, nstreams=None)`` takes a list of ``(D, Lo, Ar, T)`` torch
CUDA stacks (float32, float64, complex64 or complex128; uneven n, b, a) and optional right-hand
sides ``(n*b+a, nrhs)``, and builds the C-level plan
(``sgb_batch_plan_create``): the matrices are spread over ``nstreams``
concurrent streams and their sweeps captured into one CUDA graph.
``plan.run()`` replays it on the current stream — every array is updated in
place exactly as by the single-matrix calls (factor, then the solve with the
factor, then the selected inversion).

``nstreams=None`` asks the autotuner (``autotune``): it times candidate
schedules on scratch copies of the same shapes -- the worker-stream count,
then the CTA count of the captured column-block launches, then whether the
tensor-core products split K over clusters -- and caches the winner in a
JSON file keyed by the batch signature, the device and the hardware-queue
count (``CUDA_DEVICE_MAX_CONNECTIONS``), so the user's data is never
touched while tuning.
"""

from __future__ import annotations

import ctypes
import hashlib
import json
import os

import torch

from . import _lib
from .algs import _bta_struct

_OPS = {"pobtaf": 1, "pobtasi": 2, "pobtas": 4}
CANDIDATES = (8, 16, 32, 64, 128)
PANEL_CANDIDATES = (18, 24, 32)
CACHE = os.environ.get("SGB_AUTOTUNE_CACHE",
                       os.path.join(os.path.expanduser("~"), ".cache", "serinv_gb300", "batch_autotune.json"))


def _signature(mats, rhs, ops, precisions) -> str:
    parts = []
    for i, (D, Lo, Ar, T) in enumerate(mats):
        nr = 0 if rhs is None or rhs[i] is None else rhs[i].shape[1]
        parts.append(f"{D.shape[0]}x{D.shape[1]}x{Ar.shape[1]}:{str(D.dtype)[6:]}:{nr}:{precisions[i]}")
    dev = torch.cuda.get_device_name(mats[0][0].device) if mats else ""
    conn = os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS", "8")
    key = ";".join(parts) + f"|ops={ops}|dev={dev}|conn={conn}"
    return hashlib.sha1(key.encode()).hexdigest()


class BatchPlan:
    def __init__(self, mats, rhs=None, ops=("pobtaf", "pobtasi", "pobtas"), precisions=None, nstreams=None,
                 panel_ctas=None, tc_ksplit=None):
        self.lib = _lib.load()
        self.mats = [tuple(x.contiguous() for x in m) for m in mats]
        for m in mats:
            for x in m:
                if not (x.is_cuda and x.is_contiguous()):
                    raise ValueError("batched stacks must be contiguous CUDA tensors (used in place)")
        self.rhs = rhs
        self.ops = sum(_OPS[o] for o in ops)
        if precisions is None:
            precisions = ["fp64"] * len(mats)
        self.precisions = [_lib.precision_code(p) if m[0].dtype in (torch.float64, torch.complex128)
                           else _lib.SGB_PREC_NATIVE
                           for p, m in zip(precisions, mats)]
        if nstreams is None:
            nstreams, tuned_panel, tuned_split = autotune(mats, rhs, ops, precisions)
            if panel_ctas is None:
                panel_ctas = tuned_panel
            if tc_ksplit is None:
                tc_ksplit = tuned_split
        self.nstreams = int(nstreams)
        self.panel_ctas = int(panel_ctas or 0)
        self.options = _lib.SGB_BATCH_TC_KSPLIT if tc_ksplit else 0
        n = len(mats)
        self._descs = (_lib.SgbBta * n)(*[_bta_struct(*m) for m in self.mats])
        self._rhs = (ctypes.c_void_p * n)(*[(r.data_ptr() if r is not None else None)
                                            for r in (rhs or [None] * n)])
        self._nrhs = (ctypes.c_int64 * n)(*[(r.shape[1] if r is not None else 0) for r in (rhs or [None] * n)])
        self._prec = (ctypes.c_int * n)(*self.precisions)
        nbytes = ctypes.c_size_t(0)
        _lib.raise_for(self.lib.sgb_batch_workspace_size(self._descs, self._rhs, self._nrhs, n, self.ops,
                                                         self._prec, self.nstreams, ctypes.byref(nbytes)),
                       "batch workspace")
        dev = mats[0][0].device
        self.ws = torch.empty(nbytes.value, dtype=torch.uint8, device=dev)
        plan = ctypes.c_void_p(0)
        with torch.cuda.device(dev):
            _lib.raise_for(self.lib.sgb_batch_plan_create_ex(self._descs, self._rhs, self._nrhs, n, self.ops,
                                                             self._prec, self.nstreams, self.panel_ctas,
                                                             self.options, self.ws.data_ptr(), nbytes.value,
                                                             ctypes.byref(plan)),
                           "batch plan")
        self.plan = plan
        self.device = dev

    def run(self) -> None:
        """Replay the whole batch on the current stream (asynchronous)."""
        with torch.cuda.device(self.device):
            _lib.raise_for(self.lib.sgb_batch_run(self.plan, torch.cuda.current_stream().cuda_stream), "batch run")

    def info(self) -> torch.Tensor:
        """Per-matrix pivot report of the last run (0 = SPD), as a host tensor (synchronises)."""
        ptr = self.lib.sgb_batch_info(self.plan)
        assert ptr == self.ws.data_ptr(), "the info words open the workspace"
        return self.ws[: 4 * len(self.mats)].view(torch.int32).cpu()

    def close(self) -> None:
        if getattr(self, "plan", None):
            self.lib.sgb_batch_plan_destroy(self.plan)
            self.plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _time_plan(mats, rhs, scratch, srhs, ops, precisions, ns, panel, reps, split=False):
    """Best of `reps` timed replays of one plan, after an untimed first replay
    (which also uploads the freshly instantiated graph)."""
    def restore():
        for dst, src in zip(scratch, mats):
            for d, s_ in zip(dst, src):
                d.copy_(s_)
        if srhs is not None:
            for d, s_ in zip(srhs, rhs):
                if d is not None:
                    d.copy_(s_)

    plan = BatchPlan(scratch, srhs, ops, precisions, nstreams=ns, panel_ctas=panel, tc_ksplit=split)
    times = []
    for k in range(reps + 1):
        restore()
        st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        st.record()
        plan.run()
        en.record()
        en.synchronize()
        if k > 0:
            times.append(st.elapsed_time(en))
    plan.close()
    return min(times)


def autotune(mats, rhs=None, ops=("pobtaf", "pobtasi", "pobtas"), precisions=None, candidates=CANDIDATES,
             panel_candidates=PANEL_CANDIDATES, reps: int = 2):
    """Pick (worker-stream count, column-block CTA count, tensor-core K
    split) by timing warm replays on scratch copies of the batch: the stream
    count first (CTA count 24, no K split), then the CTA count at that
    stream count, then the K split.  Cached by signature."""
    if precisions is None:
        precisions = ["fp64"] * len(mats)
    opcode = sum(_OPS[o] for o in ops)
    sig = _signature(mats, rhs, opcode, precisions)
    cache = {}
    try:
        with open(CACHE) as f:
            cache = json.load(f)
    except (OSError, ValueError):
        cache = {}
    hit = cache.get(sig)
    if isinstance(hit, list) and len(hit) == 3:
        return int(hit[0]), int(hit[1]), bool(hit[2])
    scratch = [tuple(x.clone() for x in m) for m in mats]
    srhs = None if rhs is None else [None if r is None else r.clone() for r in rhs]
    best_ns, best_t = None, float("inf")
    for ns in candidates:
        if ns > max(1, len(mats)) and best_ns is not None:
            break
        t = _time_plan(mats, rhs, scratch, srhs, ops, precisions, ns, 0, reps)
        if t < best_t:
            best_ns, best_t = ns, t
    best_panel = 0
    for pc in panel_candidates:
        if pc == 24:  # the stream search ran at 24
            continue
        t = _time_plan(mats, rhs, scratch, srhs, ops, precisions, best_ns, pc, reps)
        if t < best_t:
            best_panel, best_t = pc, t
    best_split = False
    t = _time_plan(mats, rhs, scratch, srhs, ops, precisions, best_ns, best_panel, reps, split=True)
    if t < best_t:
        best_split, best_t = True, t
    cache[sig] = [int(best_ns), int(best_panel), bool(best_split)]
    try:
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        with open(CACHE, "w") as f:
            json.dump(cache, f)
    except OSError:
        pass
    return int(best_ns), int(best_panel), bool(best_split)


def autotune_nstreams(mats, rhs=None, ops=("pobtaf", "pobtasi", "pobtas"), precisions=None,
                      candidates=CANDIDATES, reps: int = 2) -> int:
    """The stream count of ``autotune`` (kept for callers that choose only it)."""
    return autotune(mats, rhs, ops, precisions, candidates=candidates, reps=reps)[0]
