"""GPU: the mixed-precision form (FP64 storage, block products as exact bf16
slice products on the tensor cores) against the oracle.

Stated tolerances (relative Frobenius error per stack, against the FP64
oracle): precision="mixed" (6 slices) <= 1e-9; "mixed:5" <= 1e-7;
"mixed:7" (FP64-class) <= 1e-11; "mixed:6:7" (7 slices for the products
with an explicit triangular inverse) <= 1e-9; "mixed:7:7" (7 slices
everywhere, TRSMs through the explicit inverse) <= 1e-11.
"""

import numpy as np
import pytest
import torch

import oracle
import serinv_gb300 as sg
from serinv_gb300.synthetic import generate

from _golden import rel_err

pytestmark = pytest.mark.gpu

TOL = {"mixed": 1e-9, "mixed:5": 1e-7, "mixed:7": 1e-11, "mixed:6:7": 1e-9, "mixed:7:7": 1e-11}


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


@pytest.mark.parametrize("precision", ["mixed", "mixed:5", "mixed:7", "mixed:6:7", "mixed:7:7"])
@pytest.mark.parametrize("shape", [(4, 64, 16), (3, 100, 33), (2, 512, 64), (5, 40, 0), (1, 128, 8)])
def test_mixed_against_oracle(precision, shape):
    n, b, a = shape
    m = generate(n, b, a, 2, seed=100 + n + b + a)
    ref = m.copy()
    oracle.pobtaf(*ref.arrays())
    Lr = [x.copy() for x in ref.arrays()]
    oracle.pobtasi(*ref.arrays())
    d = [dev(x) for x in m.arrays()]
    sg.pobtaf(*d, precision=precision)
    for name, g, r in zip(("diag", "lower", "arrow", "tip"), d, Lr):
        if r.size:
            e = rel_err(g.cpu().numpy(), r)
            assert e <= TOL[precision], (name, e)
    sg.pobtasi(*d, precision=precision)
    for name, g, r in zip(("diag", "lower", "arrow", "tip"), d, ref.arrays()):
        if r.size:
            e = rel_err(g.cpu().numpy(), r)
            assert e <= TOL[precision], (name, e)


def test_mixed_rejects_float32():
    m = generate(2, 16, 4, 1, seed=3, dtype=np.float32)
    d = [dev(x) for x in m.arrays()]
    with pytest.raises(NotImplementedError):
        sg.pobtaf(*d, precision="mixed")


def test_mixed_medium_against_fp64_gpu():
    """n=16 blocks of the benchmark block size against the (oracle-pinned) FP64 GPU path."""
    m = generate(16, 512, 64, 1, seed=1)
    a64 = [dev(x) for x in m.arrays()]
    amx = [x.clone() for x in a64]
    sg.pobtaf(*a64)
    sg.pobtasi(*a64)
    sg.pobtaf(*amx, precision="mixed")
    sg.pobtasi(*amx, precision="mixed")
    for x, y in zip(amx, a64):
        e = float(torch.linalg.norm(x - y) / torch.linalg.norm(y))
        assert e <= 1e-9, e


def test_mixed_bench_block_size_against_oracle():
    """The benchmark's block size (b=512, a=64) at n=32 against the oracle:
    factor, selected inverse and the 16-right-hand-side solve with the mixed
    factor, each within the stated 1e-9."""
    m = generate(32, 512, 64, 16, seed=512)
    ref = m.copy()
    oracle.pobtaf(*ref.arrays())
    Lr = [x.copy() for x in ref.arrays()]
    xr = m.B.copy()
    oracle.pobtas(*Lr, xr, trans="N")
    oracle.pobtas(*Lr, xr, trans="T")
    oracle.pobtasi(*ref.arrays())
    d = [dev(x) for x in m.arrays()]
    sg.pobtaf(*d, precision="mixed")
    L = [x.clone() for x in d]
    for name, g, r in zip(("diag", "lower", "arrow", "tip"), L, Lr):
        e = rel_err(g.cpu().numpy(), r)
        assert e <= TOL["mixed"], ("factor", name, e)
    x = dev(m.B)
    sg.pobtas(*L, x, trans="N", precision="mixed")
    sg.pobtas(*L, x, trans="T", precision="mixed")
    e = rel_err(x.cpu().numpy(), xr)
    assert e <= TOL["mixed"], ("solution", e)
    sg.pobtasi(*d, precision="mixed")
    for name, g, r in zip(("diag", "lower", "arrow", "tip"), d, ref.arrays()):
        e = rel_err(g.cpu().numpy(), r)
        assert e <= TOL["mixed"], ("selected inverse", name, e)
