"""GPU: the uneven batch at its real sizes, against the oracle.

A slice of the actual 256-matrix batch (``batch_shapes``: n ~ U{16..256},
b in {32, 64, 128, 256}, a in {0, 4, 16}, half float32, half float64, values
from ``generate(..., seed=i)``) goes through one batch plan -- pobtaf, the
solve with 4 right-hand sides (N then T), pobtasi -- with the float64 items
in the FP64 form and in the mixed form.  At b = 256 the column blocks run as
cooperative launches side by side inside the plan's graph.

Every item is checked against the oracle (src/serinv/algs/pobtaf.py:97-183,
pobtasi.py:92-172, pobtas.py:65-161) computing in float64 on the item's
inputs (float32 items: the float32-rounded inputs), relative Frobenius error
per stack and for the solution: float64 1e-12, mixed 1e-9, float32 1e-5.
For a = 0 the oracle's solve is the arrow-free one (pobts.py:57-118), which
the reference's pobtas formulas reduce to.
"""

import numpy as np
import pytest
import torch

import oracle
from serinv_gb300.batched import BatchPlan
from serinv_gb300.synthetic import batch_shapes, generate

from _golden import rel_err

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "mixed": 1e-9, "f32": 1e-5}


def _select():
    """Items of the 256-matrix batch: four at b = 256 with n >= 128 covering
    a = 0, 4, 16 and both dtypes, and four smaller blocks."""
    sh = batch_shapes(256, 0)
    want = [
        lambda s: s[1] == 256 and s[0] >= 128 and s[2] == 0 and s[3] == np.float32,
        lambda s: s[1] == 256 and s[0] >= 128 and s[2] == 4 and s[3] == np.float64,
        lambda s: s[1] == 256 and s[0] >= 128 and s[2] == 16 and s[3] == np.float32,
        lambda s: s[1] == 256 and s[0] >= 128 and s[2] == 16 and s[3] == np.float64,
        lambda s: s[1] == 128 and s[3] == np.float64,
        lambda s: s[1] == 128 and s[3] == np.float32,
        lambda s: s[1] == 64 and s[2] == 0 and s[3] == np.float64,
        lambda s: s[1] == 32 and s[2] == 4 and s[3] == np.float32,
    ]
    picked = []
    for pred in want:
        # the smallest n that matches keeps the oracle's share of the test short
        cands = [i for i, s in enumerate(sh) if pred(s) and i not in picked]
        assert cands, "batch shape list lacks a wanted item"
        picked.append(min(cands, key=lambda i: sh[i][0]))
    return [(i, sh[i]) for i in picked]


def _oracle(m):
    """X stacks and the solution of one item, in float64."""
    D, Lo, Ar, T = (x.astype(np.float64) for x in m.arrays())
    B = m.B.astype(np.float64)
    oracle.pobtaf(D, Lo, Ar, T)
    L = (D.copy(), Lo.copy(), Ar.copy(), T.copy())
    oracle.pobtas(*L, B, trans="N")  # a = 0: the arrow-free solve of pobts.py:57-118
    oracle.pobtas(*L, B, trans="T")
    oracle.pobtasi(D, Lo, Ar, T)
    return (D, Lo, Ar, T), B


@pytest.fixture(scope="module")
def items():
    out = []
    for i, (n, b, a, dt) in _select():
        m = generate(n, b, a, 4, seed=i, dtype=dt)
        X, x = _oracle(m)
        out.append((i, m, X, x))
    return out


@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_config3_slice_against_oracle(items, form):
    mats = [tuple(torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in m.arrays()) for _, m, _, _ in items]
    rhs = [torch.from_numpy(m.B).cuda() for _, m, _, _ in items]
    prec = [form] * len(items)
    plan = BatchPlan(mats, rhs, precisions=prec, nstreams=8)
    plan.run()
    torch.cuda.synchronize()
    assert torch.all(plan.info() == 0)
    for (i, m, X, x), d, r in zip(items, mats, rhs):
        tol = TOL["f32"] if m.D.dtype == np.float32 else TOL[form]
        for name, got, ref in zip(("diag", "lower", "arrow", "tip"), d, X):
            if ref.size:
                e = rel_err(got.cpu().numpy(), ref)
                assert e <= tol, (i, m.n, m.b, m.a, str(m.D.dtype), form, name, e)
        e = rel_err(r.cpu().numpy(), x)
        assert e <= tol, (i, "solution", form, e)
    plan.close()
