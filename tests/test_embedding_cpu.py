"""CPU: the real embedding that the library runs complex matrices through.
With E(z) = [x -y; y x] entry-wise, the oracle's real sweeps on the embedded
stacks (blocks 2b, arrow 2a) give exactly the embedding of the complex
results: the factor, the selected inverse and the solve (N then C)."""

import numpy as np
import pytest

import oracle
from serinv_gb300.synthetic import generate

from _golden import rel_err


def embed(z, herm_diag=False):
    """(..., r, c) complex -> (..., 2r, 2c) real."""
    z = np.array(z, copy=True)
    if herm_diag:
        idx = np.arange(z.shape[-1])
        z[..., idx, idx] = z[..., idx, idx].real
    out = np.zeros(z.shape[:-2] + (2 * z.shape[-2], 2 * z.shape[-1]))
    out[..., 0::2, 0::2] = z.real
    out[..., 0::2, 1::2] = -z.imag
    out[..., 1::2, 0::2] = z.imag
    out[..., 1::2, 1::2] = z.real
    return out


def compress(r):
    """Entries (2i, 2j) and (2i+1, 2j) -> complex (..., i, j)."""
    return r[..., 0::2, 0::2] + 1j * r[..., 1::2, 0::2]


@pytest.mark.parametrize("shape", [(4, 6, 3), (3, 5, 0), (1, 4, 2)])
def test_embedding_reproduces_complex_sweeps(shape):
    n, b, a = shape
    m = generate(n, b, a, 2, seed=11, dtype=np.complex128)
    # complex oracle
    C = [x.copy() for x in m.arrays()]
    oracle.pobtaf(*C)
    Lc = [x.copy() for x in C]
    oracle.pobtasi(*C)
    xc = m.B.copy()
    oracle.pobtas(*Lc, xc, trans="N")
    oracle.pobtas(*Lc, xc, trans="C")
    # real oracle on the embedding
    R = [embed(m.D, True), embed(m.Lo), embed(m.Ar), embed(m.T, True)]
    oracle.pobtaf(*R)
    Lr = [x.copy() for x in R]
    oracle.pobtasi(*R)
    Br = np.zeros((2 * m.B.shape[0], m.B.shape[1]))
    Br[0::2], Br[1::2] = m.B.real, m.B.imag
    oracle.pobtas(*Lr, Br, trans="N")
    oracle.pobtas(*Lr, Br, trans="T")
    for got, ref in zip(Lr, Lc):
        if ref.size:
            assert rel_err(compress(got), ref) <= 1e-13
    for got, ref in zip(R, C):
        if ref.size:
            assert rel_err(compress(got), ref) <= 1e-13
    assert rel_err(Br[0::2] + 1j * Br[1::2], xc) <= 1e-13
