"""GPU parity: the CUDA path through the drop-in API against the oracle and
against the reference's own outputs (tests/golden).  FP64 bar: 1e-12
relative (Frobenius, per stack); FP32 bar: 1e-5 relative."""

import numpy as np
import pytest
import torch

import oracle
import serinv_gb300 as sg
from serinv_gb300.synthetic import generate

from _golden import all_full_cases, bench_digest, rel_err

pytestmark = pytest.mark.gpu

TOL = {np.dtype(np.float64): 1e-12, np.dtype(np.float32): 1e-5}


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    return t.cpu().numpy()


def run_gpu(D, Lo, Ar, T, B, precision="fp64"):
    """pobtaf -> (copy) pobtasi ; pobtas N then C on the factor."""
    d = [dev(x) for x in (D, Lo, Ar, T)]
    sg.pobtaf(*d, precision=precision)
    L = [host(x) for x in d]
    sg.pobtasi(*d, precision=precision)
    X = [host(x) for x in d]
    dl = [dev(x) for x in L]
    bt = dev(B)
    sg.pobtas(*dl, bt, trans="N", precision=precision)
    sg.pobtas(*dl, bt, trans="C", precision=precision)
    return L, X, host(bt)


def run_oracle(D, Lo, Ar, T, B):
    D, Lo, Ar, T, B = (x.copy() for x in (D, Lo, Ar, T, B))
    oracle.pobtaf(D, Lo, Ar, T)
    L = [x.copy() for x in (D, Lo, Ar, T)]
    oracle.pobtasi(D, Lo, Ar, T)
    X = [D, Lo, Ar, T]
    oracle.pobtas(*L, B, trans="N")
    oracle.pobtas(*L, B, trans="C")
    return L, X, B


def spd_generate(n, b, a, r, seed, dtype):
    """The seeded generator, moving to the next seed while the matrix is not SPD.

    With b = 1 the dominance shift can leave a negative diagonal entry
    (the drawn entry lies in [-2, 2)); larger blocks are SPD by a wide margin.
    """
    for s in range(seed, seed + 100):
        m = generate(n, b, a, r, seed=s, dtype=dtype)
        if n * b + a > 2048 or np.linalg.eigvalsh(oracle.bta_to_dense(*m.arrays()).astype(np.float64)).min() > 0:
            return m
    raise AssertionError("no SPD draw")


def assert_close(got, ref, tol, what):
    for name, g, r in zip(("diag", "lower", "arrow", "tip"), got, ref):
        assert g.shape == r.shape, (what, name)
        e = rel_err(g, r)
        assert e <= tol, f"{what} {name}: rel err {e:.3e} > {tol:.0e}"


CASES = all_full_cases()


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_golden_reference_outputs(case):
    key, inp, Lref, Xref, xref = case
    tol = TOL[inp["D"].dtype]
    L, X, x = run_gpu(inp["D"], inp["Lo"], inp["Ar"], inp["T"], inp["B"])
    assert_close(L, Lref, tol, "L")
    assert_close(X, Xref, tol, "X")
    assert rel_err(x, xref) <= tol
    # the factor keeps the reference's exact zeros above the diagonal
    assert np.all(np.triu(L[0], 1) == 0)
    if L[3].size:
        assert np.all(np.triu(L[3], 1) == 0)


def test_golden_bench_shape_n128_b64_a16():
    dig = bench_digest()
    m = generate(128, 64, 16, 1, seed=0)
    L, X, x = run_gpu(m.D, m.Lo, m.Ar, m.T, m.B)
    for tag, st in (("L", L), ("X", X)):
        for name, arr in zip(("D", "Lo", "Ar"), st[:3]):
            nrm = np.linalg.norm(arr.reshape(arr.shape[0], -1), axis=1)
            np.testing.assert_allclose(nrm, dig[f"{tag}_{name}_blocknorm"], rtol=1e-12)
            assert rel_err(arr[:2], dig[f"{tag}_{name}_first2"]) <= 1e-12
            assert rel_err(arr[-2:], dig[f"{tag}_{name}_last2"]) <= 1e-12
        assert rel_err(st[3], dig[f"{tag}_T"]) <= 1e-12
    assert rel_err(x, dig["x"]) <= 1e-12


SHAPES = [
    (1, 1, 0, 1), (1, 5, 3, 2), (2, 31, 1, 3), (2, 32, 32, 1), (3, 33, 5, 4), (5, 40, 0, 2),
    (4, 65, 17, 3), (3, 100, 33, 5), (2, 128, 64, 16), (3, 512, 64, 16), (7, 64, 1, 1),
    (4, 200, 24, 4),
]


@pytest.mark.parametrize("shape", SHAPES, ids=[f"n{n}_b{b}_a{a}_r{r}" for n, b, a, r in SHAPES])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_against_oracle(shape, dtype):
    n, b, a, r = shape
    if dtype == np.float32 and b >= 512:
        pytest.skip("covered in float64")
    m = spd_generate(n, b, a, r, seed=n * 1000 + b * 10 + a, dtype=dtype)
    Lr, Xr, xr = run_oracle(m.D, m.Lo, m.Ar, m.T, m.B)
    L, X, x = run_gpu(m.D, m.Lo, m.Ar, m.T, m.B)
    tol = TOL[np.dtype(dtype)]
    assert_close(L, Lr, tol, "L")
    assert_close(X, Xr, tol, "X")
    assert rel_err(x, xr) <= tol


def test_factorize_last_block_false():
    m = generate(4, 40, 6, 1, seed=11)
    ref = m.copy()
    oracle.pobtaf(*ref.arrays(), factorize_last_block=False)
    d = [dev(x) for x in m.arrays()]
    sg.pobtaf(*d, factorize_last_block=False)
    assert_close([host(x) for x in d], ref.arrays(), 1e-12, "partial L")


def test_invert_last_block_false():
    m = generate(4, 40, 6, 1, seed=12)
    oracle.pobtaf(*m.arrays())
    # seed the last diagonal/arrow blocks and the tip with the exact inverse
    full = m.copy()
    oracle.pobtasi(*full.arrays())
    part = m.copy()
    part.D[-1], part.Ar[-1], part.T[:] = full.D[-1], full.Ar[-1], full.T
    ref = part.copy()
    oracle.pobtasi(*ref.arrays(), invert_last_block=False)
    d = [dev(x) for x in part.arrays()]
    sg.pobtasi(*d, invert_last_block=False)
    assert_close([host(x) for x in d], ref.arrays(), 1e-12, "partial X")


@pytest.mark.parametrize("trans", ["N", "T", "C"])
def test_pobtas_partial(trans):
    m = generate(5, 24, 4, 3, seed=13)
    oracle.pobtaf(*m.arrays())
    Bref = m.B.copy()
    oracle.pobtas(*m.arrays(), Bref, trans=trans, partial=True)
    d = [dev(x) for x in m.arrays()]
    bt = dev(m.B)
    sg.pobtas(*d, bt, trans=trans, partial=True)
    assert rel_err(host(bt), Bref) <= 1e-12


def test_numpy_host_arrays_in_place():
    m = generate(3, 48, 8, 2, seed=14)
    ref = m.copy()
    Lr, Xr, xr = run_oracle(*ref.arrays(), ref.B)
    D, Lo, Ar, T = m.arrays()
    sg.pobtaf(D, Lo, Ar, T)
    assert_close((D, Lo, Ar, T), Lr, 1e-12, "host L")
    L = [x.copy() for x in (D, Lo, Ar, T)]
    sg.pobtasi(D, Lo, Ar, T)
    assert_close((D, Lo, Ar, T), Xr, 1e-12, "host X")
    B = m.B
    sg.pobtas(*L, B, trans="N")
    sg.pobtas(*L, B, trans="T")
    assert rel_err(B, xr) <= 1e-12


def test_non_contiguous_device_arrays():
    m = generate(3, 20, 4, 1, seed=15)
    Lr, Xr, _ = run_oracle(*m.arrays(), m.B)
    # Fortran-ordered storage: transposed views of transposed copies
    d = [dev(np.ascontiguousarray(np.swapaxes(x, -1, -2))).transpose(-1, -2) for x in m.arrays()]
    assert not d[0].is_contiguous()
    sg.pobtaf(*d)
    assert_close([host(x) for x in d], Lr, 1e-12, "strided L")
    sg.pobtasi(*d)
    assert_close([host(x) for x in d], Xr, 1e-12, "strided X")


def test_not_spd_raises_with_row():
    m = generate(4, 16, 3, 1, seed=16)
    m.D[2][5, 5] = -1e6  # block 2, local row 5 -> global row 2*16+5+1 (1-based)
    d = [dev(x) for x in m.arrays()]
    with pytest.raises(np.linalg.LinAlgError, match="38-th"):
        sg.pobtaf(*d)


def test_mismatched_dtypes_rejected():
    m = generate(2, 8, 2, 1, seed=17)
    d = [dev(x) for x in m.arrays()]
    d[1] = d[1].float()
    with pytest.raises(TypeError):
        sg.pobtaf(*d)


def test_bad_shapes_rejected():
    m = generate(2, 8, 2, 1, seed=18)
    d = [dev(x) for x in m.arrays()]
    with pytest.raises(ValueError):
        sg.pobtaf(d[0], d[1][:, :4], d[2], d[3])
    with pytest.raises(ValueError):
        sg.pobtas(*d, dev(np.zeros((5, 1))))


BT_CASES = [c for c in CASES if c[1]["Ar"].shape[1] == 0]


@pytest.mark.parametrize("case", BT_CASES, ids=[c[0] for c in BT_CASES])
def test_bt_family_golden(case):
    """pobtf / pobtsi / pobts (the arrow-free family) against the reference's
    own pobtf / pobtsi / pobts outputs."""
    key, inp, L, X, x = case
    tol = TOL[inp["D"].dtype]
    d = [dev(inp["D"]), dev(inp["Lo"])]
    sg.pobtf(*d)
    Lg = [host(t) for t in d]
    sg.pobtsi(*d)
    Xg = [host(t) for t in d]
    dl = [dev(t) for t in Lg]
    bt = dev(inp["B"])
    sg.pobts(*dl, bt, trans="N")
    sg.pobts(*dl, bt, trans="C")
    for got, ref in zip(Lg, L[:2]):
        if ref.size:
            assert rel_err(got, ref) <= tol
    for got, ref in zip(Xg, X[:2]):
        if ref.size:
            assert rel_err(got, ref) <= tol
    assert rel_err(host(bt), x) <= tol


def test_bt_family_rejects_unknown_kwargs():
    m = generate(3, 8, 0, 1, seed=1)
    with pytest.raises(TypeError):
        sg.pobtf(dev(m.D), dev(m.Lo), bogus=1)
    with pytest.raises(TypeError):
        sg.pobtsi(dev(m.D), dev(m.Lo), bogus=1)
