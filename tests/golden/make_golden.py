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

and stores inputs and outputs (full arrays for small cases, a digest plus
edge blocks for the 128x64 case) as compressed ``.npz`` files beside this
script, with the NumPy/SciPy versions in ``versions.json``.
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


def main(ref_root: str) -> None:
    ref, tu = _load_reference(ref_root)
    from serinv_gb300.synthetic import generate

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

    import scipy
    with open(os.path.join(HERE, "versions.json"), "w") as f:
        json.dump({"numpy": np.__version__, "scipy": scipy.__version__,
                   "reference_version": "0.1.0 (src/serinv/__about__.py:3)"}, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
