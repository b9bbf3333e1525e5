"""CPU: the seeded generator that feeds the benchmarks and the parity tests
reproduces the inputs stored with the golden vectors exactly (its real path
must not drift), and its complex matrices are Hermitian positive definite."""

import re

import numpy as np
import pytest

import oracle
from serinv_gb300.synthetic import generate

from _golden import load_cases, permuted_cases

SYNTH = load_cases("synthetic_small.npz")


@pytest.mark.parametrize("case", SYNTH, ids=[c[0] for c in SYNTH])
def test_generator_reproduces_golden_inputs(case):
    key, inp, *_ = case
    n, b, a, r, s, dt = re.match(r"n(\d+)_b(\d+)_a(\d+)_r(\d+)_s(\d+)_(\w+?)_$", key).groups()
    m = generate(int(n), int(b), int(a), int(r), seed=int(s), dtype=np.dtype(dt))
    for got, name in zip((m.D, m.Lo, m.Ar, m.T, m.B), ("D", "Lo", "Ar", "T", "B")):
        np.testing.assert_array_equal(got, inp[name])


def test_generator_reproduces_permuted_golden_inputs():
    for key, inp, *_ in permuted_cases():
        g = re.match(r"(?:bt_)?n(\d+)_b(\d+)_a(\d+)_r(\d+)_s(\d+)_(c128_)?$", key).groups()
        n, b, a, r, s = map(int, g[:5])
        m = generate(n, b, a, r, seed=s, dtype=np.complex128 if g[5] else np.float64)
        np.testing.assert_array_equal(m.D, inp["D"])
        np.testing.assert_array_equal(m.B, inp["B"])


@pytest.mark.parametrize("shape", [(3, 5, 2), (4, 8, 0), (1, 6, 3)])
def test_complex_generator_is_hermitian_positive_definite(shape):
    n, b, a = shape
    m = generate(n, b, a, 1, seed=4, dtype=np.complex128)
    A = oracle.bta_to_dense(*m.arrays())
    np.testing.assert_array_equal(A, A.conj().T)
    assert np.linalg.eigvalsh(A).min() > 0
    assert np.abs(m.D.imag).max() > 0  # genuinely complex
