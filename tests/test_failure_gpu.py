"""GPU: the failure surface, without any GPU fault.

* Non-finite input: a NaN on the diagonal of D_i, in a lower block or in an
  arrow block reaches a pivot, and pobtaf reports the 1-based global row of
  the first such pivot, as for a non-positive pivot (the reference raises
  from its per-block Cholesky: src/serinv/cupyfix/cholesky_lowerfill.py:
  79-81, src/serinv/__init__.py:150-151).  Both forms; in the mixed form the
  slice products carry a row or column holding a NaN through as NaN.
* Timeouts: with the poll limit of the bounded device waits set to 0
  (``sgb_debug_spin_limit``), every wait that does not find its condition
  already met gives up at once.  The column-block kernel and the
  tensor-core kernel then report SGB_ERR_TIMEOUT in their status word,
  every CTA leaves and the tensor memory is freed: the same calls with the
  default limit right after give correct results on the same context.
"""

import ctypes
import re

import numpy as np
import pytest
import torch

import oracle
import serinv_gb300 as sg
from serinv_gb300 import _lib
from serinv_gb300.synthetic import generate

from _golden import rel_err

pytestmark = pytest.mark.gpu


def _row_of(exc) -> int:
    m = re.match(r"(\d+)-th leading minor", str(exc))
    assert m, str(exc)
    return int(m.group(1))


CASES = [  # (n, b, a, dtype, precision): tile sweep, column-block kernel, mixed, float32
    (4, 64, 8, np.float64, "fp64"),
    (4, 128, 16, np.float64, "fp64"),
    (4, 128, 16, np.float64, "mixed"),
    (4, 96, 8, np.float32, "fp64"),
]


@pytest.mark.parametrize("case", CASES)
def test_nan_on_diagonal_reports_its_row(case):
    n, b, a, dt, prec = case
    m = generate(n, b, a, 1, seed=41, dtype=dt)
    i, r = 2, 37 % b
    m.D[i][r, r] = np.nan
    d = [torch.from_numpy(x).cuda() for x in m.arrays()]
    with pytest.raises(np.linalg.LinAlgError) as ei:
        sg.pobtaf(*d, precision=prec)
    assert _row_of(ei.value) == i * b + r + 1


@pytest.mark.parametrize("case", CASES)
def test_nan_in_lower_block_reaches_the_next_pivot(case):
    """Lo[i][r, c] = NaN makes row r of L_{i+1,i} NaN from column c on, so
    row and column r of the updated D_{i+1} are NaN: the first bad pivot is
    row r of block i+1."""
    n, b, a, dt, prec = case
    m = generate(n, b, a, 1, seed=43, dtype=dt)
    i, r, c = 1, 21 % b, 5
    m.Lo[i][r, c] = np.nan
    d = [torch.from_numpy(x).cuda() for x in m.arrays()]
    with pytest.raises(np.linalg.LinAlgError) as ei:
        sg.pobtaf(*d, precision=prec)
    assert _row_of(ei.value) == (i + 1) * b + r + 1


@pytest.mark.parametrize("case", [c for c in CASES if c[2] > 0])
def test_nan_in_arrow_block_reaches_the_tip(case):
    """Ar[0][r, c] = NaN: row r of every later arrow block and row and
    column r of the tip become NaN; the first bad pivot is tip row r."""
    n, b, a, dt, prec = case
    m = generate(n, b, a, 1, seed=47, dtype=dt)
    r = 3
    m.Ar[0][r, 2] = np.nan
    d = [torch.from_numpy(x).cuda() for x in m.arrays()]
    with pytest.raises(np.linalg.LinAlgError) as ei:
        sg.pobtaf(*d, precision=prec)
    assert _row_of(ei.value) == n * b + r + 1


class _SpinLimit:
    """Poll limit of the bounded device waits, restored on exit."""

    def __init__(self, polls):
        self.polls = polls

    def __enter__(self):
        torch.cuda.synchronize()
        self.prev = _lib.spin_limit(self.polls)
        return self

    def __exit__(self, *exc):
        torch.cuda.synchronize()
        _lib.spin_limit(self.prev)
        return False


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_column_block_kernel_timeout_is_reported(prec):
    """b = 128: the persistent column-block kernel.  Tile 1 arrives by value
    from the helper CTAs; with no polls allowed the factorizer's take of it
    gives up, so the timeout is certain."""
    m = generate(3, 128, 16, 1, seed=53)
    d = [torch.from_numpy(x).cuda() for x in m.arrays()]
    with _SpinLimit(0):
        with pytest.raises(_lib.SgbError, match="timed out"):
            sg.pobtaf(*d, precision=prec)
    # the context is intact: the same call with the default limit is right
    ref = m.copy()
    oracle.pobtaf(*ref.arrays())
    d = [torch.from_numpy(x).cuda() for x in m.arrays()]
    sg.pobtaf(*d, precision=prec)
    tol = 1e-12 if prec == "fp64" else 1e-9
    for g, r in zip(d, ref.arrays()):
        assert rel_err(g.cpu().numpy(), r) <= tol


def test_tensor_core_timeout_is_reported():
    """A 256 x 256 x 256 slice product (a K split over 4-CTA clusters): with
    no polls allowed the MMA warp's first stage wait gives up; the status
    word says so, and the next product on the same context is exact."""
    lib = _lib.load()
    M = N = K = 256
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.rand((M, K), generator=g, device="cuda", dtype=torch.float64) - 0.5
    B = torch.rand((K, N), generator=g, device="cuda", dtype=torch.float64) - 0.5
    prec = _lib.precision_code("mixed")
    need = ctypes.c_size_t(0)
    assert lib.sgb_dgemm_workspace_size(prec, M, N, K, ctypes.byref(need)) == 0
    ws = torch.zeros(need.value, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream

    def run():
        C = torch.zeros((M, N), dtype=torch.float64, device="cuda")
        rc = lib.sgb_dgemm(prec, b"N", b"N", M, N, K, 1.0, A.data_ptr(), K, B.data_ptr(), N, 0.0,
                           C.data_ptr(), N, ws.data_ptr(), need.value, stream)
        assert rc == 0
        torch.cuda.synchronize()
        return C, int(ws[:4].view(torch.int32).item())

    with _SpinLimit(0):
        _, status = run()
    assert status == _lib.SGB_ERR_TIMEOUT
    C, status = run()
    assert status == 0
    ref = A @ B
    assert float(torch.linalg.norm(C - ref) / torch.linalg.norm(ref)) <= 1e-12


def test_spin_limit_query_does_not_change_it():
    before = _lib.spin_limit()
    assert before == 1 << 22
    assert _lib.spin_limit() == before
