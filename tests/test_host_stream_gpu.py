"""GPU: pinned host stacks take the streamed path (blocks uploaded in sweep
order and downloaded as soon as they are final, overlapped with the
computation) and give the device path's results, in place."""

import numpy as np
import pytest
import torch

import oracle
import serinv_gb300 as sg
from serinv_gb300.synthetic import generate

from _golden import rel_err

pytestmark = pytest.mark.gpu


def pinned_numpy(x):
    t = torch.empty(x.shape, dtype=torch.from_numpy(x).dtype, pin_memory=True)
    out = t.numpy()
    np.copyto(out, x)
    return out


def run_oracle(D, Lo, Ar, T, **kw):
    st = [x.copy() for x in (D, Lo, Ar, T)]
    oracle.pobtaf(*st, **kw)
    return st


@pytest.mark.parametrize("shape,dtype", [
    ((20, 64, 16), np.float64),    # several upload / download groups
    ((9, 130, 5), np.float64),     # ragged tiles
    ((1, 40, 8), np.float64),
    ((12, 48, 0), np.float64),     # no arrowhead
    ((17, 32, 4), np.float32),
])
def test_streamed_pobtaf_pobtasi_match_oracle(shape, dtype):
    n, b, a = shape
    m = generate(n, b, a, 1, seed=n + b, dtype=dtype)
    host = [pinned_numpy(x) for x in m.arrays()]
    assert torch.from_numpy(host[0]).is_pinned()
    sg.pobtaf(*host)
    ref = run_oracle(*m.arrays())
    tol = 1e-12 if dtype == np.float64 else 1e-5
    for g, r in zip(host, ref):
        if r.size:
            assert rel_err(g, r) <= tol
    sg.pobtasi(*host)
    oracle.pobtasi(*ref)
    for g, r in zip(host, ref):
        if r.size:
            assert rel_err(g, r) <= tol


def test_streamed_torch_pinned_and_mode_flags():
    m = generate(11, 72, 9, 1, seed=4)
    host = [torch.from_numpy(x.copy()).pin_memory() for x in m.arrays()]
    sg.pobtaf(*host, factorize_last_block=False)
    ref = run_oracle(*m.arrays(), factorize_last_block=False)
    for g, r in zip(host, ref):
        assert rel_err(np.tril(g.numpy()) if g.dim() == 2 else g.numpy(), np.tril(r) if r.ndim == 2 else r) <= 1e-12
    # invert_last_block=False: the last blocks and the tip given as inverted
    m2 = generate(10, 64, 8, 1, seed=5)
    L = run_oracle(*m2.arrays())
    full = [x.copy() for x in L]
    oracle.pobtasi(*full)
    part = [x.copy() for x in L]
    part[0][-1], part[2][-1], part[3][:] = full[0][-1], full[2][-1], full[3]
    host = [pinned_numpy(x) for x in part]
    sg.pobtasi(*host, invert_last_block=False)
    for g, r in zip(host, full):
        assert rel_err(g, r) <= 1e-12


def test_streamed_mixed_precision():
    m = generate(16, 128, 16, 1, seed=6)
    host = [pinned_numpy(x) for x in m.arrays()]
    sg.pobtaf(*host, precision="mixed")
    sg.pobtasi(*host, precision="mixed")
    ref = run_oracle(*m.arrays())
    oracle.pobtasi(*ref)
    for g, r in zip(host, ref):
        assert rel_err(g, r) <= 1e-9


def test_streamed_not_spd_raises_with_row():
    m = generate(6, 32, 4, 1, seed=7)
    D = m.D.copy()
    D[3, 5, 5] = -100.0
    host = [pinned_numpy(x) for x in (D, m.Lo, m.Ar, m.T)]
    with pytest.raises(np.linalg.LinAlgError, match=f"^{3 * 32 + 5 + 1}-th"):
        sg.pobtaf(*host)


def test_pageable_host_arrays_take_the_copy_path():
    m = generate(5, 40, 4, 1, seed=8)
    D, Lo, Ar, T = (x.copy() for x in m.arrays())
    assert not torch.from_numpy(D).is_pinned()
    sg.pobtaf(D, Lo, Ar, T)
    ref = run_oracle(*m.arrays())
    for g, r in zip((D, Lo, Ar, T), ref):
        assert rel_err(g, r) <= 1e-12
