"""GPU parity for complex (Hermitian positive-definite) matrices: the drop-in
API on complex128 / complex64 tensors against the reference's own outputs
(tests/golden/complex.npz: its test suite's complex grid and seeded
Hermitian shapes) and against the oracle.  Bars: 1e-12 relative (complex128,
Frobenius per stack), 1e-5 (complex64); mixed precision 1e-9."""

import numpy as np
import pytest
import torch

import oracle
import serinv_gb300 as sg
from serinv_gb300.synthetic import generate

from _golden import load_cases, rel_err

pytestmark = pytest.mark.gpu

COMPLEX = load_cases("complex.npz")


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    return t.cpu().numpy()


def run_gpu(D, Lo, Ar, T, B, **kw):
    d = [dev(x) for x in (D, Lo, Ar, T)]
    sg.pobtaf(*d, **kw)
    L = [host(x) for x in d]
    sg.pobtasi(*d, **kw)
    X = [host(x) for x in d]
    dl = [dev(x) for x in L]
    bt = dev(B)
    sg.pobtas(*dl, bt, trans="N", **kw)
    sg.pobtas(*dl, bt, trans="C", **kw)
    return L, X, host(bt)


def run_oracle(D, Lo, Ar, T, B):
    D, Lo, Ar, T, B = (x.copy() for x in (D, Lo, Ar, T, B))
    oracle.pobtaf(D, Lo, Ar, T)
    L = [x.copy() for x in (D, Lo, Ar, T)]
    oracle.pobtasi(D, Lo, Ar, T)
    oracle.pobtas(*L, B, trans="N")
    oracle.pobtas(*L, B, trans="C")
    return L, [D, Lo, Ar, T], B


def check(got, ref, tol):
    (Lg, Xg, xg), (Lr, Xr, xr) = got, ref
    for name, g, r in zip(("diag", "lower", "arrow", "tip"), Lg, Lr):
        if r.size:
            assert g.dtype == r.dtype
            assert rel_err(g, r) <= tol, ("factor", name, rel_err(g, r))
    for name, g, r in zip(("diag", "lower", "arrow", "tip"), Xg, Xr):
        if r.size:
            assert rel_err(g, r) <= tol, ("inverse", name, rel_err(g, r))
    assert rel_err(xg, xr) <= tol, ("solve", rel_err(xg, xr))


@pytest.mark.parametrize("case", COMPLEX, ids=[c[0] for c in COMPLEX])
def test_complex_golden(case):
    key, inp, L, X, x = case
    got = run_gpu(*(inp[k] for k in ("D", "Lo", "Ar", "T", "B")))
    check(got, (list(L), list(X), x), 1e-12)


@pytest.mark.parametrize("shape,dtype", [
    ((5, 64, 16, 2), np.complex128),    # real embedding b = 128: persistent column-block kernel
    ((4, 100, 33, 3), np.complex128),   # ragged
    ((6, 48, 0, 2), np.complex128),     # no arrowhead
    ((1, 40, 8, 1), np.complex128),     # one block
    ((5, 32, 4, 2), np.complex64),
])
def test_complex_against_oracle(shape, dtype):
    n, b, a, r = shape
    m = generate(n, b, a, r, seed=90 + n, dtype=dtype)
    tol = 1e-12 if dtype == np.complex128 else 1e-5
    check(run_gpu(m.D, m.Lo, m.Ar, m.T, m.B), run_oracle(m.D, m.Lo, m.Ar, m.T, m.B), tol)


def test_complex_mixed_precision():
    """complex128 with the tensor-core slice products (6 slices)."""
    m = generate(4, 128, 16, 2, seed=7, dtype=np.complex128)
    check(run_gpu(m.D, m.Lo, m.Ar, m.T, m.B, precision="mixed"), run_oracle(m.D, m.Lo, m.Ar, m.T, m.B), 1e-9)


def test_complex_mode_flags():
    """factorize_last_block / invert_last_block / partial on complex data."""
    m = generate(4, 24, 5, 2, seed=8, dtype=np.complex128)
    d = [dev(x) for x in m.arrays()]
    sg.pobtaf(*d, factorize_last_block=False)
    ref = [x.copy() for x in m.arrays()]
    oracle.pobtaf(*ref, factorize_last_block=False)
    # the last diagonal block and the tip are updated, not factored: their
    # lower triangles are the result (the strict upper parts are not kept)
    assert rel_err(np.tril(host(d[0])), np.tril(ref[0])) <= 1e-12
    assert rel_err(host(d[1]), ref[1]) <= 1e-12
    assert rel_err(host(d[2]), ref[2]) <= 1e-12
    assert rel_err(np.tril(host(d[3])), np.tril(ref[3])) <= 1e-12
    B = m.B.copy()
    L = [x.copy() for x in m.arrays()]
    oracle.pobtaf(*L)
    bt = dev(B)
    sg.pobtas(*[dev(x) for x in L], bt, trans="N", partial=True)
    oracle.pobtas(*L, B, trans="N", partial=True)
    assert rel_err(host(bt), B) <= 1e-12


def test_complex_host_arrays_and_conj_views():
    """NumPy complex arrays are written back in place; lazily conjugated
    torch views are read and written through the view."""
    m = generate(3, 16, 4, 2, seed=9, dtype=np.complex128)
    D, Lo, Ar, T = (x.copy() for x in m.arrays())
    sg.pobtaf(D, Lo, Ar, T)
    ref = [x.copy() for x in m.arrays()]
    oracle.pobtaf(*ref)
    for g, r in zip((D, Lo, Ar, T), ref):
        assert rel_err(g, r) <= 1e-12
    # B given as the conjugate view of its conjugate
    bc = dev(m.B.conj())
    view = bc.conj()
    assert view.is_conj()
    sg.pobtas(*[dev(x) for x in ref], view, trans="N")
    B = m.B.copy()
    oracle.pobtas(*ref, B, trans="N")
    assert rel_err(host(view.resolve_conj()), B) <= 1e-12


def test_complex_not_spd_reports_complex_row():
    """A non-positive pivot is reported at its complex row (1-based)."""
    m = generate(3, 8, 2, 1, seed=10, dtype=np.complex128)
    D = m.D.copy()
    D[1, 3, 3] = -50.0  # block 1, row 3 -> global row 1 * 8 + 3 + 1 = 12
    with pytest.raises(np.linalg.LinAlgError, match="^12-th"):
        sg.pobtaf(dev(D), dev(m.Lo), dev(m.Ar), dev(m.T))
