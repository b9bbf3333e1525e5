"""Loading helpers for the golden vectors in tests/golden/ (made by make_golden.py)."""

from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_cases(fname: str):
    """Yield (key, inputs dict, L stacks, X stacks, x) for every full case in a file."""
    z = np.load(os.path.join(GOLDEN, fname))
    out = []
    for key in z["cases"]:
        key = str(key)
        inp = {k: z[f"{key}in_{k}"] for k in ("D", "Lo", "Ar", "T", "B")}
        L = tuple(z[f"{key}L_{k}"] for k in ("D", "Lo", "Ar", "T"))
        X = tuple(z[f"{key}X_{k}"] for k in ("D", "Lo", "Ar", "T"))
        out.append((key, inp, L, X, z[f"{key}x"]))
    return out


def all_full_cases():
    return load_cases("reference_suite_grid.npz") + load_cases("synthetic_small.npz")


def permuted_cases():
    """(key, inputs, after permuted pobtaf, final selected inverse, final solution)
    for the middle-partition workflow cases (make_golden.py, permuted_cases)."""
    z = np.load(os.path.join(GOLDEN, "permuted.npz"))
    out = []
    for key in z["cases"]:
        key = str(key)
        inp = {k: z[f"{key}in_{k}"] for k in ("D", "Lo", "Ar", "T", "B")}
        F = {k: z[f"{key}F_{k}"] for k in ("D", "Lo", "Ar", "T", "buf")}
        X = {k: z[f"{key}X_{k}"] for k in ("D", "Lo", "Ar", "T", "buf")}
        out.append((key, inp, F, X, z[f"{key}x"]))
    return out


def bench_digest():
    return dict(np.load(os.path.join(GOLDEN, "bench_n128_b64_a16.npz")))


def rel_err(x, ref) -> float:
    dt = np.complex128 if (np.iscomplexobj(x) or np.iscomplexobj(ref)) else np.float64
    x = np.asarray(x, dtype=dt)
    ref = np.asarray(ref, dtype=dt)
    den = np.linalg.norm(ref)
    if den == 0:
        return float(np.linalg.norm(x))
    return float(np.linalg.norm(x - ref) / den)
