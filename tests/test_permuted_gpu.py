"""GPU parity of the permuted (buffer=) forms: the middle-partition workflow
of the reference's permuted tests (permuted pobtaf -> natural factorization,
inversion and solve of the reduced system of blocks 0, n-1 and the tip ->
permuted pobtasi / pobtas), driven through the drop-in API, against the
reference's own outputs (tests/golden/permuted.npz) and against the oracle.
FP64 bar: 1e-12 relative (Frobenius, per stack); FP32 bar: 1e-5."""

import numpy as np
import pytest
import torch

import oracle
import serinv_gb300 as sg
from serinv_gb300.synthetic import generate

from _golden import permuted_cases, rel_err
from _permuted import workflow

pytestmark = pytest.mark.gpu

TOL = {np.dtype(np.float64): 1e-12, np.dtype(np.float32): 1e-5, np.dtype(np.complex128): 1e-12,
       np.dtype(np.complex64): 1e-5}
PERM = permuted_cases()


def _lib_fn(**extra):
    return dict(
        pobtaf=lambda D, Lo, Ar, T: sg.pobtaf(D, Lo, Ar, T, **extra),
        pobtasi=lambda D, Lo, Ar, T: sg.pobtasi(D, Lo, Ar, T, **extra),
        pobtas=lambda D, Lo, Ar, T, B, tr: sg.pobtas(D, Lo, Ar, T, B, trans=tr, **extra),
        pobtaf_p=lambda D, Lo, Ar, T, buf: sg.pobtaf(D, Lo, Ar, T, buffer=buf, **extra),
        pobtasi_p=lambda D, Lo, Ar, T, buf: sg.pobtasi(D, Lo, Ar, T, buffer=buf, **extra),
        pobtas_p=lambda D, Lo, Ar, T, buf, B, tr: sg.pobtas(D, Lo, Ar, T, B, trans=tr, buffer=buf, **extra))


def _bt_fn():
    """The arrow-free family (pobtf / pobtsi / pobts) in the same workflow."""
    nb = lambda D: D.shape[0] * D.shape[1]  # noqa: E731
    return dict(
        pobtaf=lambda D, Lo, Ar, T: sg.pobtf(D, Lo),
        pobtasi=lambda D, Lo, Ar, T: sg.pobtsi(D, Lo),
        pobtas=lambda D, Lo, Ar, T, B, tr: sg.pobts(D, Lo, B[:nb(D)], trans=tr),
        pobtaf_p=lambda D, Lo, Ar, T, buf: sg.pobtf(D, Lo, buffer=buf),
        pobtasi_p=lambda D, Lo, Ar, T, buf: sg.pobtsi(D, Lo, buffer=buf),
        pobtas_p=lambda D, Lo, Ar, T, buf, B, tr: sg.pobts(D, Lo, B[:nb(D)], trans=tr, buffer=buf))


def _oracle_fn():
    return dict(pobtaf=oracle.pobtaf, pobtasi=oracle.pobtasi,
                pobtas=lambda D, Lo, Ar, T, B, tr: oracle.pobtas(D, Lo, Ar, T, B, trans=tr),
                pobtaf_p=oracle.pobtaf_permuted, pobtasi_p=oracle.pobtasi_permuted,
                pobtas_p=lambda D, Lo, Ar, T, buf, B, tr: oracle.pobtas_permuted(D, Lo, Ar, T, B, buf, trans=tr))


def _run_torch(fn, D, Lo, Ar, T, B):
    d = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (D, Lo, Ar, T, B)]
    F, X, x = workflow(fn, *d, zeros=lambda shape, ref: torch.zeros(shape, dtype=ref.dtype, device=ref.device),
                       copy=lambda v: v.clone())
    return [t.cpu().numpy() for t in F], [t.cpu().numpy() for t in X], x.cpu().numpy()


def _run_oracle(D, Lo, Ar, T, B):
    return workflow(_oracle_fn(), *(x.copy() for x in (D, Lo, Ar, T, B)),
                    zeros=lambda shape, ref: np.zeros(shape, dtype=ref.dtype), copy=lambda v: v.copy())


def _compare(got, ref, tol, n):
    (Fg, Xg, xg), (Fr, Xr, xr) = got, ref
    names = ("D", "Lo", "Ar", "T")
    for g, r, nm in zip(Fg[:4], Fr[:4], names):
        if r.size:
            assert rel_err(g, r) <= tol, ("factor", nm, rel_err(g, r))
    # buffer[0] is not written by the permuted factorization
    assert rel_err(Fg[4][1:], Fr[4][1:]) <= tol, ("factor buffer", rel_err(Fg[4][1:], Fr[4][1:]))
    for g, r, nm in zip(Xg[:4], Xr[:4], names):
        if r.size:
            assert rel_err(g, r) <= tol, ("inverse", nm, rel_err(g, r))
    assert rel_err(xg, xr) <= tol, ("solve", rel_err(xg, xr))


@pytest.mark.parametrize("case", PERM, ids=[c[0] for c in PERM])
def test_permuted_golden(case):
    """Against the reference's own permuted pobtaf / pobtasi / pobtas outputs."""
    key, inp, F, X, x = case
    got = _run_torch(_lib_fn(), *(inp[k] for k in ("D", "Lo", "Ar", "T", "B")))
    ref = ([F[k] for k in ("D", "Lo", "Ar", "T", "buf")], [X[k] for k in ("D", "Lo", "Ar", "T", "buf")], x)
    _compare(got, ref, TOL[inp["D"].dtype], inp["D"].shape[0])


@pytest.mark.parametrize("shape,dtype", [
    ((70, 8, 2, 2), np.float64),     # crosses the 64-block chunk of the selected inversion
    ((10, 64, 16, 3), np.float64),
    ((6, 130, 5, 2), np.float64),    # ragged tiles
    ((8, 48, 0, 2), np.float64),     # no arrowhead
    ((6, 32, 4, 2), np.float32),
    ((2, 16, 4, 1), np.float64),     # nothing to eliminate: n = 2
])
def test_permuted_against_oracle(shape, dtype):
    n, b, a, r = shape
    m = generate(n, b, a, r, seed=31 + n, dtype=dtype)
    got = _run_torch(_lib_fn(), m.D, m.Lo, m.Ar, m.T, m.B)
    ref = _run_oracle(m.D, m.Lo, m.Ar, m.T, m.B)
    _compare(got, ref, TOL[np.dtype(dtype)], n)


def test_bt_family_permuted():
    """pobtf / pobtsi / pobts with buffer= (pobtf.py:125-185, pobtsi.py:128-179,
    pobts.py:121-165) against the oracle with an empty arrowhead."""
    m = generate(9, 40, 0, 2, seed=77)
    got = _run_torch(_bt_fn(), m.D, m.Lo, m.Ar, m.T, m.B)
    ref = _run_oracle(m.D, m.Lo, m.Ar, m.T, m.B)
    _compare(got, ref, 1e-12, 9)


def test_permuted_numpy_host_arrays_in_place():
    """Host arrays, buffer included, are written back in place."""
    m = generate(7, 24, 3, 2, seed=5)
    D, Lo, Ar, T = (x.copy() for x in m.arrays())
    buf = np.zeros_like(D)
    sg.pobtaf(D, Lo, Ar, T, buffer=buf)
    Do, Loo, Aro, To = (x.copy() for x in m.arrays())
    bufo = np.zeros_like(Do)
    oracle.pobtaf_permuted(Do, Loo, Aro, To, bufo)
    for g, r in ((D, Do), (Lo, Loo), (Ar, Aro), (T, To), (buf[1:], bufo[1:])):
        assert rel_err(g, r) <= 1e-12


def test_permuted_rejects_bad_buffer():
    m = generate(4, 8, 2, 1, seed=3)
    d = [torch.from_numpy(x).cuda() for x in m.arrays()]
    with pytest.raises(ValueError):
        sg.pobtaf(*d, buffer=torch.zeros((4, 8, 4), dtype=torch.float64, device="cuda"))
    with pytest.raises(TypeError):
        sg.pobtaf(*d, buffer=torch.zeros((4, 8, 8), dtype=torch.float32, device="cuda"))


@pytest.mark.parametrize("shape", [
    (70, 128, 16, 2),    # column-block kernel with L_ii^{-T}; crosses the 64-block chunk
    (5, 512, 64, 2),     # the benchmark's block size: three-term products cut into tensor-core groups
    (6, 100, 0, 2),      # no arrowhead
    (6, 64, 8, 2),       # launch-based diagonal tiles, tensor-core products
])
def test_permuted_mixed_against_oracle(shape):
    """The permuted forms in the mixed form (FP64 storage, block products as
    bf16 slice products on the tensor cores) inside the middle-partition
    workflow, against the oracle at the mixed-precision bar 1e-9."""
    n, b, a, r = shape
    m = generate(n, b, a, r, seed=91 + n + b, dtype=np.float64)
    got = _run_torch(_lib_fn(precision="mixed"), m.D, m.Lo, m.Ar, m.T, m.B)
    ref = _run_oracle(m.D, m.Lo, m.Ar, m.T, m.B)
    _compare(got, ref, 1e-9, n)


def test_permuted_mixed_rejects_float32():
    m = generate(4, 16, 2, 1, seed=3, dtype=np.float32)
    d = [torch.from_numpy(x).cuda() for x in m.arrays()]
    buf = torch.zeros_like(d[0])
    with pytest.raises(NotImplementedError):
        sg.pobtaf(*d, buffer=buf, precision="mixed")
