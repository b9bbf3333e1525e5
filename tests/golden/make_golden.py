"""Generate the golden vectors by running the reference implementation itself.

Run in a container where the reference source tree is available:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /root/reference

It imports the reference's own ``pobtaf`` / ``pobtasi`` / ``pobtas`` (and, for
arrow width 0, ``pobtf`` / ``pobtsi`` / ``pobts``), runs them on

* the reference test suite's own input family (``dd_bta`` + ``symmetrize``
  from its ``tests/testing_utils.py``, seed 63) over its parameter grid
  (b in {2,3}, a in {2,3}, n in {1..4}, nrhs in {1,2,3}), and
* the seeded synthetic generator of this repository at small and at the
  CPU-runnable benchmark shape (n=128, b=64, a=16, 1 RHS),

and the permuted middle-partition workflow (``buffer=``, as the
reference's permuted tests drive it) on small synthetic inputs, and stores
inputs and outputs (full arrays for small cases, a digest plus edge blocks
for the 128x64 case) as compressed ``.npz`` files beside this script, with
the NumPy/SciPy versions in ``versions.json``.  ``--only=permuted`` and
``--only=complex`` write the permuted or the complex128 file alone.
"""

from __future__ import annotations

import importlib.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def _load_reference(ref_root: str):
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        import serinv  # noqa: F401
        from serinv.algs import pobtaf, pobtasi, pobtas, pobtf, pobtsi, pobts
    spec = importlib.util.spec_from_file_location(
        "ref_testing_utils", os.path.join(ref_root, "tests", "testing_utils.py"))
    tu = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(tu)
    return dict(pobtaf=pobtaf, pobtasi=pobtasi, pobtas=pobtas, pobtf=pobtf,
                pobtsi=pobtsi, pobts=pobts), tu


def _run_reference(ref, D, Lo, Ar, T, B):
    """Return (L stacks, X stacks, solution) from the reference on copies."""
    a = Ar.shape[1]
    L = [x.copy() for x in (D, Lo, Ar, T)]
    if a == 0:
        ref["pobtf"](L[0], L[1])
    else:
        ref["pobtaf"](*L)
    X = [x.copy() for x in L]
    if a == 0:
        ref["pobtsi"](X[0], X[1])
    else:
        ref["pobtasi"](*X)
    x = B.copy()
    if a == 0:
        ref["pobts"](L[0], L[1], x, trans="N")
        ref["pobts"](L[0], L[1], x, trans="C")
    else:
        ref["pobtas"](*L, x, trans="N")
        ref["pobtas"](*L, x, trans="C")
    return L, X, x


def _pack(prefix, D, Lo, Ar, T, B, L, X, x):
    out = {}
    for name, arr in zip(("D", "Lo", "Ar", "T", "B"), (D, Lo, Ar, T, B)):
        out[f"{prefix}in_{name}"] = arr
    for name, arr in zip(("D", "Lo", "Ar", "T"), L):
        out[f"{prefix}L_{name}"] = arr
    for name, arr in zip(("D", "Lo", "Ar", "T"), X):
        out[f"{prefix}X_{name}"] = arr
    out[f"{prefix}x"] = x
    return out


def _reduced(D, Ar, T, buf):
    """The reduced system of a middle partition (blocks 0 and n-1, the tip),
    as the reference's permuted tests build it
    (tests/tests_algs/permuted/test_bta/test_pobtasi_permuted.py:94-115)."""
    b, a = D.shape[1], Ar.shape[1]
    rD = np.zeros((2, b, b), dtype=D.dtype)
    rLo = np.zeros((1, b, b), dtype=D.dtype)
    rAr = np.zeros((2, a, b), dtype=D.dtype)
    rD[0], rD[1] = D[0], D[-1]
    rLo[0] = buf[-1].conj().T
    rAr[0], rAr[1] = Ar[0], Ar[-1]
    return rD, rLo, rAr, T.copy()


def _map_back(D, Ar, T, buf, rD, rLo, rAr, rT):
    D[0], D[-1] = rD[0], rD[1]
    buf[-1] = rLo[0].conj().T
    Ar[0], Ar[-1] = rAr[0], rAr[1]
    T[:, :] = rT


def permuted_cases(ref, generate):
    """The middle-partition workflow of the reference's permuted tests:
    permuted pobtaf -> reduced system (pobtaf, then pobtasi or pobtas) ->
    permuted pobtasi / permuted pobtas N and C, on seeded synthetic inputs;
    one case of the arrow-free family (pobtf / pobtsi / pobts)."""
    out = {}
    cases = []
    for (n, b, a, nrhs, seed, dt) in [(3, 5, 3, 2, 11, np.float64), (4, 16, 4, 3, 12, np.float64),
                                      (6, 40, 7, 2, 13, np.float64), (5, 33, 1, 1, 14, np.float64),
                                      (5, 12, 3, 2, 15, np.complex128)]:
        m = generate(n, b, a, nrhs, seed=seed, dtype=dt)
        D, Lo, Ar, T, B = (x.copy() for x in (m.D, m.Lo, m.Ar, m.T, m.B))
        buf = np.zeros_like(D)
        ref["pobtaf"](D, Lo, Ar, T, buffer=buf)
        F = [x.copy() for x in (D, Lo, Ar, T, buf)]
        rD, rLo, rAr, rT = _reduced(D, Ar, T, buf)
        ref["pobtaf"](rD, rLo, rAr, rT)
        rL = [x.copy() for x in (rD, rLo, rAr, rT)]
        # selected inversion
        XD, XLo, XAr, XT, Xbuf = (x.copy() for x in (D, Lo, Ar, T, buf))
        sD, sLo, sAr, sT = (x.copy() for x in rL)
        ref["pobtasi"](sD, sLo, sAr, sT)
        _map_back(XD, XAr, XT, Xbuf, sD, sLo, sAr, sT)
        ref["pobtasi"](XD, XLo, XAr, XT, buffer=Xbuf)
        # solve
        LD, LLo, LAr, LT, Lbuf = (x.copy() for x in (D, Lo, Ar, T, buf))
        _map_back(LD, LAr, LT, Lbuf, *rL)
        x = B.copy()
        ref["pobtas"](LD, LLo, LAr, LT, x, buffer=Lbuf, trans="N")
        rB = np.concatenate([x[:b], x[(n - 1) * b:n * b], x[n * b:]])
        ref["pobtas"](*rL, rB, trans="N")
        ref["pobtas"](*rL, rB, trans="C")
        x[:b], x[(n - 1) * b:n * b], x[n * b:] = rB[:b], rB[b:2 * b], rB[2 * b:]
        ref["pobtas"](LD, LLo, LAr, LT, x, buffer=Lbuf, trans="C")
        key = f"n{n}_b{b}_a{a}_r{nrhs}_s{seed}_" + ("c128_" if dt == np.complex128 else "")
        for name, arr in zip(("D", "Lo", "Ar", "T", "B"), (m.D, m.Lo, m.Ar, m.T, m.B)):
            out[f"{key}in_{name}"] = arr
        for name, arr in zip(("D", "Lo", "Ar", "T", "buf"), F):
            out[f"{key}F_{name}"] = arr
        for name, arr in zip(("D", "Lo", "Ar", "T", "buf"), (XD, XLo, XAr, XT, Xbuf)):
            out[f"{key}X_{name}"] = arr
        out[f"{key}x"] = x
        cases.append(key)
    # the arrow-free family (pobtf / pobtsi / pobts with buffer=), same workflow
    for (n, b, nrhs, seed) in [(5, 24, 2, 16)]:
        m = generate(n, b, 0, nrhs, seed=seed)
        D, Lo, B = m.D.copy(), m.Lo.copy(), m.B.copy()
        buf = np.zeros_like(D)
        ref["pobtf"](D, Lo, buffer=buf)
        F = [x.copy() for x in (D, Lo, buf)]
        rD = np.stack([D[0], D[-1]])
        rLo = buf[-1].conj().T[None].copy()
        ref["pobtf"](rD, rLo)
        rL = [rD.copy(), rLo.copy()]
        XD, XLo, Xbuf = D.copy(), Lo.copy(), buf.copy()
        sD, sLo = rD.copy(), rLo.copy()
        ref["pobtsi"](sD, sLo)
        XD[0], XD[-1], Xbuf[-1] = sD[0], sD[1], sLo[0].conj().T
        ref["pobtsi"](XD, XLo, buffer=Xbuf)
        LD, LLo, Lbuf = D.copy(), Lo.copy(), buf.copy()
        LD[0], LD[-1], Lbuf[-1] = rL[0][0], rL[0][1], rL[1][0].conj().T
        x = B.copy()
        ref["pobts"](LD, LLo, x, buffer=Lbuf, trans="N")
        rB = np.concatenate([x[:b], x[(n - 1) * b:n * b]])
        ref["pobts"](*rL, rB, trans="N")
        ref["pobts"](*rL, rB, trans="C")
        x[:b], x[(n - 1) * b:n * b] = rB[:b], rB[b:]
        ref["pobts"](LD, LLo, x, buffer=Lbuf, trans="C")
        key = f"bt_n{n}_b{b}_a0_r{nrhs}_s{seed}_"
        ear, et = np.zeros((n, 0, b)), np.zeros((0, 0))
        for name, arr in zip(("D", "Lo", "Ar", "T", "B"), (m.D, m.Lo, ear, et, m.B)):
            out[f"{key}in_{name}"] = arr
        for name, arr in zip(("D", "Lo", "Ar", "T", "buf"), (F[0], F[1], ear, et, F[2])):
            out[f"{key}F_{name}"] = arr
        for name, arr in zip(("D", "Lo", "Ar", "T", "buf"), (XD, XLo, ear, et, Xbuf)):
            out[f"{key}X_{name}"] = arr
        out[f"{key}x"] = x
        cases.append(key)
    out["cases"] = np.array(cases)
    np.savez_compressed(os.path.join(HERE, "permuted.npz"), **out)


def complex_cases(ref, tu, generate):
    """complex128: the reference suite's grid with its complex inputs
    (``dd_bta(..., dtype="complex128")`` + ``symmetrize`` and ``rhs``, as its
    tests run them) and seeded synthetic Hermitian shapes with non-zero
    imaginary parts."""
    out = {}
    cases = []
    for b in (2, 3):
        for a in (2, 3):
            for n in (1, 2, 3, 4):
                nrhs = 2
                # the dtype as its tests pass it (the string): the matrix is
                # complex with real entries, the right-hand side complex
                A = tu.dd_bta(b, a, n, device_array=False, dtype="complex128")
                tu.symmetrize(A)
                B = tu.rhs(nrhs, b, a, n, device_array=False, dtype="complex128")
                (D, Lo, _, Ar, _, T) = tu.bta_dense_to_arrays(A, b, a, n)
                L, X, x = _run_reference(ref, D, Lo, Ar, T, B)
                key = f"suite_b{b}_a{a}_n{n}_r{nrhs}_"
                out.update(_pack(key, D, Lo, Ar, T, B, L, X, x))
                cases.append(key)
    for (n, b, a, nrhs, seed) in [(3, 24, 7, 3, 21), (4, 33, 5, 1, 22), (5, 32, 0, 2, 23), (2, 16, 4, 2, 24),
                                  (6, 40, 3, 2, 25)]:
        m = generate(n, b, a, nrhs, seed=seed, dtype=np.complex128)
        L, X, x = _run_reference(ref, m.D, m.Lo, m.Ar, m.T, m.B)
        key = f"n{n}_b{b}_a{a}_r{nrhs}_s{seed}_"
        out.update(_pack(key, m.D, m.Lo, m.Ar, m.T, m.B, L, X, x))
        cases.append(key)
    out["cases"] = np.array(cases)
    np.savez_compressed(os.path.join(HERE, "complex.npz"), **out)


def main(ref_root: str, only: str | None = None) -> None:
    ref, tu = _load_reference(ref_root)
    from serinv_gb300.synthetic import generate
    if only == "permuted":
        permuted_cases(ref, generate)
        return
    if only == "complex":
        complex_cases(ref, tu, generate)
        return

    # 1) The reference test suite's own input family and parameter grid.
    suite = {}
    cases = []
    for b in (2, 3):
        for a in (2, 3):
            for n in (1, 2, 3, 4):
                for nrhs in (1, 2, 3):
                    A = tu.dd_bta(b, a, n, device_array=False, dtype=np.float64)
                    tu.symmetrize(A)
                    B = tu.rhs(nrhs, b, a, n, device_array=False, dtype=np.float64)
                    (D, Lo, _, Ar, _, T) = tu.bta_dense_to_arrays(A, b, a, n)
                    L, X, x = _run_reference(ref, D, Lo, Ar, T, B)
                    key = f"b{b}_a{a}_n{n}_r{nrhs}_"
                    suite.update(_pack(key, D, Lo, Ar, T, B, L, X, x))
                    cases.append(key)
    suite["cases"] = np.array(cases)
    np.savez_compressed(os.path.join(HERE, "reference_suite_grid.npz"), **suite)

    # 2) Seeded synthetic generator, small and odd shapes (full arrays).
    synth = {}
    cases = []
    for (n, b, a, nrhs, seed, dt) in [
        (1, 8, 3, 2, 1, np.float64),
        (2, 5, 0, 1, 2, np.float64),
        (3, 24, 7, 3, 3, np.float64),
        (5, 32, 0, 2, 4, np.float64),
        (8, 16, 4, 4, 5, np.float64),
        (4, 33, 5, 1, 6, np.float64),
        (6, 16, 4, 4, 7, np.float32),
        (3, 64, 16, 16, 8, np.float64),
    ]:
        m = generate(n, b, a, nrhs, seed=seed, dtype=dt)
        L, X, x = _run_reference(ref, m.D, m.Lo, m.Ar, m.T, m.B)
        key = f"n{n}_b{b}_a{a}_r{nrhs}_s{seed}_{np.dtype(dt).name}_"
        synth.update(_pack(key, m.D, m.Lo, m.Ar, m.T, m.B, L, X, x))
        cases.append(key)
    synth["cases"] = np.array(cases)
    np.savez_compressed(os.path.join(HERE, "synthetic_small.npz"), **synth)

    # 3) The CPU-runnable benchmark shape: n=128, b=64, a=16, 1 RHS, seed 0.
    m = generate(128, 64, 16, 1, seed=0)
    L, X, x = _run_reference(ref, m.D, m.Lo, m.Ar, m.T, m.B)
    dig = {
        "in_checksum": np.array([m.D.sum(), m.Lo.sum(), m.Ar.sum(), m.T.sum(), m.B.sum()]),
        "x": x,
    }
    for tag, stacks in (("L", L), ("X", X)):
        for name, arr in zip(("D", "Lo", "Ar"), stacks[:3]):
            dig[f"{tag}_{name}_blocknorm"] = np.linalg.norm(arr.reshape(arr.shape[0], -1), axis=1)
            dig[f"{tag}_{name}_first2"] = arr[:2]
            dig[f"{tag}_{name}_last2"] = arr[-2:]
        dig[f"{tag}_T"] = stacks[3]
    np.savez_compressed(os.path.join(HERE, "bench_n128_b64_a16.npz"), **dig)

    # 4) The permuted (middle-partition) variants.
    permuted_cases(ref, generate)

    # 5) complex128 (a fresh load of the test utilities restarts their seed).
    ref, tu = _load_reference(ref_root)
    complex_cases(ref, tu, generate)

    import scipy
    with open(os.path.join(HERE, "versions.json"), "w") as f:
        json.dump({"numpy": np.__version__, "scipy": scipy.__version__,
                   "reference_version": "0.1.0 (src/serinv/__about__.py:3)"}, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    args = [x for x in sys.argv[1:] if not x.startswith("--only=")]
    only = next((x.split("=", 1)[1] for x in sys.argv[1:] if x.startswith("--only=")), None)
    if len(args) != 1:
        sys.exit("usage: make_golden.py REFERENCE_ROOT [--only=permuted|complex]")
    main(args[0], only)
