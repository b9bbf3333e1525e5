"""GPU: the symmetric BTA product against the dense matrix, and the refined
solve: with a mixed-precision factor, refinement against the original A
brings the solution to the FP64 solve's accuracy."""

import numpy as np
import pytest
import torch

import oracle
import serinv_gb300 as sg
from serinv_gb300.synthetic import generate

from _golden import rel_err

pytestmark = pytest.mark.gpu


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


@pytest.mark.parametrize("shape", [(1, 8, 3, 1), (2, 5, 0, 2), (3, 33, 7, 3), (6, 64, 16, 9), (4, 100, 1, 17),
                                   (5, 40, 0, 8)])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_bta_matvec_against_dense(shape, dtype):
    n, b, a, r = shape
    m = generate(n, b, a, r, seed=n + b + a, dtype=dtype)
    A = oracle.bta_to_dense(*m.arrays()).astype(np.float64)
    D, T = m.D.copy(), m.T.copy()
    # only the lower triangles may be read: poison the strict upper parts
    iu = np.triu_indices(b, 1)
    D[:, iu[0], iu[1]] = np.nan
    if a:
        it = np.triu_indices(a, 1)
        T[it] = np.nan
    x = np.random.default_rng(1).uniform(-1, 1, (n * b + a, r)).astype(dtype)
    y = sg.bta_matvec(dev(D), dev(m.Lo), dev(m.Ar), dev(T), dev(x)).cpu().numpy()
    tol = 1e-13 if dtype == np.float64 else 1e-5
    assert rel_err(y, A @ x.astype(np.float64)) <= tol
    # alpha / beta
    y0 = np.random.default_rng(2).uniform(-1, 1, x.shape).astype(dtype)
    yt = dev(y0)
    sg.bta_matvec(dev(D), dev(m.Lo), dev(m.Ar), dev(T), dev(x), alpha=-2.0, beta=0.5, y=yt)
    assert rel_err(yt.cpu().numpy(), 0.5 * y0 - 2.0 * (A @ x.astype(np.float64))) <= tol


def test_refine_recovers_fp64_accuracy_from_mixed_factor():
    """kappa ~1e5: the mixed factor's solve carries ~1e-9 relative error;
    two refinement steps reach the FP64 solve's level."""
    n, b, a = 6, 128, 16
    m = generate(n, b, a, 4, seed=3, shift=0.0)
    A = oracle.bta_to_dense(*m.arrays())
    ev = np.linalg.eigvalsh(A)
    sigma = (ev[-1] - 1e5 * ev[0]) / (1e5 - 1)  # kappa(A + sigma I) = 1e5
    D, T = m.D.copy(), m.T.copy()
    D[:, np.arange(b), np.arange(b)] += sigma
    T[np.arange(a), np.arange(a)] += sigma
    A = oracle.bta_to_dense(D, m.Lo, m.Ar, T)
    x_ref = np.linalg.solve(A, m.B)
    orig = [dev(v) for v in (D, m.Lo, m.Ar, T)]
    errs = {}
    for prec in ("mixed", "fp64"):
        L = [v.clone() for v in orig]
        sg.pobtaf(*L, precision=prec)
        for iters in (0, 2):
            x = dev(m.B)
            sg.pobtas_refine(*orig, *L, x, iters=iters)
            errs[(prec, iters)] = rel_err(x.cpu().numpy(), x_ref)
    assert errs[("mixed", 0)] > 1e-13          # the mixed factor's error shows
    assert errs[("mixed", 2)] <= 5 * errs[("fp64", 0)] + 1e-14
    assert errs[("fp64", 2)] <= 1e-11
    # iters = 0 is the plain solve
    L = [v.clone() for v in orig]
    sg.pobtaf(*L)
    x0 = dev(m.B)
    sg.pobtas_refine(*orig, *L, x0, iters=0)
    x1 = dev(m.B)
    sg.pobtas(*L, x1, trans="N")
    sg.pobtas(*L, x1, trans="C")
    assert rel_err(x0.cpu().numpy(), x1.cpu().numpy()) <= 1e-15


def test_refine_rejects_mismatched_structures():
    m = generate(3, 16, 4, 1, seed=1)
    A = [dev(v) for v in m.arrays()]
    m2 = generate(3, 16, 2, 1, seed=1)
    L = [dev(v) for v in m2.arrays()]
    with pytest.raises(ValueError):
        sg.pobtas_refine(*A, *L, dev(m.B))
