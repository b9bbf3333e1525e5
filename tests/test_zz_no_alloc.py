"""GPU: sgb_pobtaf_noalloc, the pobtaf entry point that allocates nothing.

It exists for callers that cannot allocate device memory (stream-capture
regions, allocator-free real-time loops, foreign-language hosts with only
device pointers); its scratch is a static device array.  Called through the
C ABI twice in a row, it must reproduce sgb_pobtaf (caller-provided
workspace) within the FP64 tolerance of the other parity tests (1e-12).
This file sorts last so that a failure here stops a -x run only after every
other test has run.
"""

import ctypes

import pytest
import torch

from serinv_gb300 import _lib
from serinv_gb300.synthetic import generate

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _desc(ts):
    D, Lo, Ar, T = ts
    m = _lib.SgbBta()
    m.dtype = _lib.SGB_F64
    m.n, m.b, m.a = D.shape[0], D.shape[1], Ar.shape[1]
    m.diag = D.data_ptr()
    m.lower = Lo.data_ptr() if Lo.numel() else None
    m.arrow = Ar.data_ptr() if Ar.numel() else None
    m.tip = T.data_ptr() if T.numel() else None
    return m


def _rel(x, y):
    return float(torch.linalg.norm(x - y) / torch.linalg.norm(y))


@pytest.mark.parametrize("shape", [(6, 100, 12), (3, 64, 0), (1, 33, 5)])
def test_noalloc_matches_pobtaf_twice(shape):
    lib = _lib.load()
    n, b, a = shape
    mat = generate(n, b, a, 0, seed=21 + n)
    A0 = [torch.from_numpy(x).cuda() for x in mat.arrays()]
    stream = torch.cuda.current_stream().cuda_stream

    # existing entry point, caller-provided workspace
    ref = [x.clone() for x in A0]
    mref = _desc(ref)
    need = ctypes.c_size_t(0)
    assert lib.sgb_pobtaf_workspace_size(ctypes.byref(mref), 0, ctypes.byref(need)) == 0
    assert need.value <= lib.sgb_pobtaf_noalloc_scratch_bytes()
    ws = torch.empty(need.value, dtype=torch.uint8, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert lib.sgb_pobtaf(ctypes.byref(mref), 1, 0, ws.data_ptr(), need.value, info.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    assert int(info.item()) == 0

    for _ in range(2):  # two calls in a row share the static scratch
        got = [x.clone() for x in A0]
        mg = _desc(got)
        info2 = torch.full((1,), -7, dtype=torch.int32, device="cuda")
        assert lib.sgb_pobtaf_noalloc(ctypes.byref(mg), 1, info2.data_ptr(), stream) == 0
        torch.cuda.synchronize()
        assert int(info2.item()) == 0
        for x, y in zip(got, ref):
            if y.numel():
                assert _rel(x, y) <= TOL


def test_noalloc_reports_not_spd():
    lib = _lib.load()
    mat = generate(3, 16, 2, 0, seed=5)
    mat.D[1][3, 3] = -1e6
    ts = [torch.from_numpy(x).cuda() for x in mat.arrays()]
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    m = _desc(ts)
    assert lib.sgb_pobtaf_noalloc(ctypes.byref(m), 1, info.data_ptr(), torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    assert int(info.item()) == 16 + 3 + 1


def test_noalloc_rejects_bad_descriptor():
    lib = _lib.load()
    assert lib.sgb_pobtaf_noalloc(None, 1, None, None) == _lib.SGB_ERR_ARG


def test_noalloc_reports_timeout_in_info():
    """A bounded device wait that gives up (poll limit 0, a test hook) is
    reported in the caller's info word as -SGB_ERR_TIMEOUT, since the status
    word sits in the private array; with the default limit the next call on
    the same array is clean and exact."""
    lib = _lib.load()
    mat = generate(3, 100, 12, 0, seed=29)
    A0 = [torch.from_numpy(x).cuda() for x in mat.arrays()]
    stream = torch.cuda.current_stream().cuda_stream
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    got = [x.clone() for x in A0]
    torch.cuda.synchronize()
    prev = _lib.spin_limit(0)
    try:
        assert lib.sgb_pobtaf_noalloc(ctypes.byref(_desc(got)), 1, info.data_ptr(), stream) == 0
        torch.cuda.synchronize()
    finally:
        _lib.spin_limit(prev)
    assert int(info.item()) == -_lib.SGB_ERR_TIMEOUT

    ref = [x.clone() for x in A0]
    mref = _desc(ref)
    need = ctypes.c_size_t(0)
    assert lib.sgb_pobtaf_workspace_size(ctypes.byref(mref), 0, ctypes.byref(need)) == 0
    ws = torch.empty(need.value, dtype=torch.uint8, device="cuda")
    assert lib.sgb_pobtaf(ctypes.byref(mref), 1, 0, ws.data_ptr(), need.value, None, stream) == 0
    got = [x.clone() for x in A0]
    assert lib.sgb_pobtaf_noalloc(ctypes.byref(_desc(got)), 1, info.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    assert int(info.item()) == 0
    for x, y in zip(got, ref):
        assert _rel(x, y) <= TOL
