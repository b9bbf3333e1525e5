"""CPU: the oracle against the reference's own outputs and against dense NumPy."""

import numpy as np
import pytest

import oracle
from serinv_gb300.synthetic import generate, flops

from _golden import all_full_cases, bench_digest, load_cases, rel_err

CASES = all_full_cases()


def _tol(dtype):
    return 1e-12 if np.dtype(dtype) == np.float64 else 2e-5


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_reference_outputs(case):
    key, inp, Lref, Xref, xref = case
    tol = _tol(inp["D"].dtype)
    D, Lo, Ar, T, B = (inp[k].copy() for k in ("D", "Lo", "Ar", "T", "B"))
    oracle.pobtaf(D, Lo, Ar, T)
    for got, ref in zip((D, Lo, Ar, T), Lref):
        assert got.dtype == ref.dtype
        assert rel_err(got, ref) <= tol
    L = [x.copy() for x in (D, Lo, Ar, T)]
    oracle.pobtasi(D, Lo, Ar, T)
    for got, ref in zip((D, Lo, Ar, T), Xref):
        assert rel_err(got, ref) <= tol
    oracle.pobtas(*L, B, trans="N")
    oracle.pobtas(*L, B, trans="C")
    assert rel_err(B, xref) <= tol


@pytest.mark.parametrize("case", CASES[::7], ids=[c[0] for c in CASES[::7]])
def test_oracle_matches_dense_numpy(case):
    key, inp, *_ = case
    if inp["D"].dtype != np.float64:
        pytest.skip("dense check in float64 only")
    D, Lo, Ar, T, B = (inp[k].copy() for k in ("D", "Lo", "Ar", "T", "B"))
    n, b, a = D.shape[0], D.shape[1], Ar.shape[1]
    A = oracle.bta_to_dense(D, Lo, Ar, T)
    # the reference tests symmetrize; the lower stacks define the matrix
    Lden = np.linalg.cholesky(A)
    Xden = np.linalg.inv(A)
    xden = np.linalg.solve(A, B)
    oracle.pobtaf(D, Lo, Ar, T)
    Ld = oracle.dense_to_bta(Lden, n, b, a)
    for got, ref in zip((D, Lo, Ar, T), Ld):
        assert rel_err(got, ref) <= 1e-12
    L = [x.copy() for x in (D, Lo, Ar, T)]
    oracle.pobtasi(D, Lo, Ar, T)
    Xd = oracle.dense_to_bta(Xden, n, b, a)
    for got, ref in zip((D, Lo, Ar, T), Xd):
        assert rel_err(got, ref) <= 1e-12
    oracle.pobtas(*L, B, trans="N")
    oracle.pobtas(*L, B, trans="T")
    assert rel_err(B, xden) <= 1e-12


def test_generator_is_pinned_to_golden():
    """The seeded generator still produces the inputs the golden digest was made from."""
    dig = bench_digest()
    m = generate(128, 64, 16, 1, seed=0)
    got = np.array([m.D.sum(), m.Lo.sum(), m.Ar.sum(), m.T.sum(), m.B.sum()])
    np.testing.assert_allclose(got, dig["in_checksum"], rtol=1e-13)


def test_oracle_bench_shape_digest():
    """n=128, b=64, a=16: block norms and edge blocks against the reference run."""
    dig = bench_digest()
    m = generate(128, 64, 16, 1, seed=0)
    D, Lo, Ar, T = m.arrays()
    oracle.pobtaf(D, Lo, Ar, T)
    for name, arr in zip(("D", "Lo", "Ar"), (D, Lo, Ar)):
        nrm = np.linalg.norm(arr.reshape(arr.shape[0], -1), axis=1)
        np.testing.assert_allclose(nrm, dig[f"L_{name}_blocknorm"], rtol=1e-12)
        np.testing.assert_allclose(arr[-2:], dig[f"L_{name}_last2"], rtol=1e-11, atol=1e-14)
    np.testing.assert_allclose(T, dig["L_T"], rtol=1e-12, atol=1e-14)
    L = [x.copy() for x in (D, Lo, Ar, T)]
    oracle.pobtasi(D, Lo, Ar, T)
    for name, arr in zip(("D", "Lo", "Ar"), (D, Lo, Ar)):
        nrm = np.linalg.norm(arr.reshape(arr.shape[0], -1), axis=1)
        np.testing.assert_allclose(nrm, dig[f"X_{name}_blocknorm"], rtol=1e-12)
        np.testing.assert_allclose(arr[:2], dig[f"X_{name}_first2"], rtol=1e-11, atol=1e-15)
    B = m.B
    oracle.pobtas(*L, B, trans="N")
    oracle.pobtas(*L, B, trans="C")
    assert rel_err(B, dig["x"]) <= 1e-12


def test_generator_is_spd_and_dominant():
    m = generate(4, 8, 3, 1, seed=3)
    A = oracle.bta_to_dense(*m.arrays())
    assert np.allclose(A, A.T)
    # the shift is added to the existing diagonal entry (in [-2, 2)), so
    # every row satisfies diag >= offdiag_sum - 1 and the matrix is SPD
    off = np.abs(A).sum(axis=1) - np.abs(np.diag(A))
    assert np.all(np.diag(A) - off >= -1.0)
    assert np.linalg.eigvalsh(A).min() > 0


def test_pobtas_rejects_bad_trans():
    m = generate(2, 4, 2, 1, seed=0)
    with pytest.raises(ValueError):
        oracle.pobtas(*m.arrays(), m.B, trans="X")


def test_oracle_not_spd_raises():
    m = generate(3, 4, 2, 1, seed=0)
    m.D[1] = -np.eye(4)
    with pytest.raises(np.linalg.LinAlgError):
        oracle.pobtaf(*m.arrays())


def test_flop_counts():
    f = flops(512, 512, 64, 16)
    assert abs(f["pobtaf"] / 1e9 - 187.2) < 0.1
    assert abs(f["pobtasi"] / 1e9 - 497.5) < 0.1
    assert abs(f["pobtas"] / 1e9 - 13.9) < 0.1


from _golden import permuted_cases  # noqa: E402
from _permuted import workflow  # noqa: E402

PERM = permuted_cases()


def _oracle_fn():
    return dict(pobtaf=oracle.pobtaf, pobtasi=oracle.pobtasi,
                pobtas=lambda D, Lo, Ar, T, B, tr: oracle.pobtas(D, Lo, Ar, T, B, trans=tr),
                pobtaf_p=oracle.pobtaf_permuted, pobtasi_p=oracle.pobtasi_permuted,
                pobtas_p=lambda D, Lo, Ar, T, buf, B, tr: oracle.pobtas_permuted(D, Lo, Ar, T, B, buf, trans=tr))


@pytest.mark.parametrize("case", PERM, ids=[c[0] for c in PERM])
def test_oracle_permuted_matches_reference(case):
    """The permuted restatements, driven through the middle-partition
    workflow, reproduce the reference's own outputs."""
    key, inp, F, X, x = case
    D, Lo, Ar, T, B = (inp[k].copy() for k in ("D", "Lo", "Ar", "T", "B"))
    Fo, Xo, xo = workflow(_oracle_fn(), D, Lo, Ar, T, B,
                          zeros=lambda shape, ref: np.zeros(shape, dtype=ref.dtype), copy=lambda v: v.copy())
    for got, name in zip(Fo, ("D", "Lo", "Ar", "T")):
        assert rel_err(got, F[name]) <= 1e-14, ("F", name)
    assert rel_err(Fo[4][1:], F["buf"][1:]) <= 1e-14
    for got, name in zip(Xo, ("D", "Lo", "Ar", "T")):
        assert rel_err(got, X[name]) <= 1e-14, ("X", name)
    assert rel_err(xo, x) <= 1e-14


@pytest.mark.parametrize("case", PERM, ids=[c[0] for c in PERM])
def test_permuted_workflow_is_the_inverse(case):
    """The golden workflow's results are A^{-1} on the BTA pattern and A^{-1} B."""
    key, inp, F, X, x = case
    A = oracle.bta_to_dense(inp["D"], inp["Lo"], inp["Ar"], inp["T"])
    n, b, a = inp["D"].shape[0], inp["D"].shape[1], inp["Ar"].shape[1]
    Ainv = np.linalg.inv(A)
    D, Lo, Ar, T = oracle.dense_to_bta(Ainv, n, b, a)
    for got, ref in ((X["D"], D), (X["Lo"], Lo), (X["Ar"], Ar), (X["T"], T)):
        assert rel_err(got, ref) <= 1e-10
    assert rel_err(x, np.linalg.solve(A, inp["B"])) <= 1e-10


COMPLEX = load_cases("complex.npz")


def _oracle_run(D, Lo, Ar, T, B):
    oracle.pobtaf(D, Lo, Ar, T)
    L = [x.copy() for x in (D, Lo, Ar, T)]
    oracle.pobtasi(D, Lo, Ar, T)
    oracle.pobtas(*L, B, trans="N")
    oracle.pobtas(*L, B, trans="C")
    return L, [D, Lo, Ar, T], B


@pytest.mark.parametrize("case", COMPLEX, ids=[c[0] for c in COMPLEX])
def test_oracle_complex_matches_reference(case):
    """complex128: the restatement (conjugate transposes throughout) against
    the reference's own outputs, and the outputs against dense NumPy."""
    key, inp, L, X, x = case
    D, Lo, Ar, T, B = (inp[k].copy() for k in ("D", "Lo", "Ar", "T", "B"))
    Lg, Xg, xg = _oracle_run(D, Lo, Ar, T, B)
    for got, ref in zip(Lg, L):
        if ref.size:
            assert rel_err(got, ref) <= 1e-12
    for got, ref in zip(Xg, X):
        if ref.size:
            assert rel_err(got, ref) <= 1e-12
    assert rel_err(xg, x) <= 1e-12
    A = oracle.bta_to_dense(inp["D"], inp["Lo"], inp["Ar"], inp["T"])
    assert rel_err(xg, np.linalg.solve(A, inp["B"])) <= 1e-10
