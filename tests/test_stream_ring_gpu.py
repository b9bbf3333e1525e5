"""GPU: host-resident stacks streamed through a ring of device blocks
(``device_streaming=True`` on host arrays; the reference's streaming mode,
src/serinv/algs/pobtaf.py:284-524, pobtasi.py:247-496, for matrices larger
than device memory).

Small rings force every path: slots reused many times, pobtasi chunks of
ring/2 blocks with the block above each chunk kept resident, ragged tiles,
no arrowhead, float32, the mixed form and the mode flags.  Results must
equal the device path's (same kernels; 1e-13) and the oracle's (1e-12 in
FP64, 1e-5 in float32, 1e-9 mixed).
"""

import numpy as np
import pytest
import torch

import oracle
import serinv_gb300 as sg
from serinv_gb300.synthetic import generate

from _golden import rel_err

pytestmark = pytest.mark.gpu


def _device_result(m, precision, **kw):
    d = [torch.from_numpy(x.copy()).cuda() for x in m.arrays()]
    sg.pobtaf(*d, precision=precision, factorize_last_block=kw.get("flb", True))
    L = [x.cpu().numpy() for x in d]
    sg.pobtasi(*d, precision=precision, invert_last_block=kw.get("ilb", True))
    return L, [x.cpu().numpy() for x in d]


@pytest.mark.parametrize("shape,dtype,precision,rings", [
    ((13, 64, 16), np.float64, "fp64", (2, 2)),     # every slot reused six times
    ((13, 64, 16), np.float64, "fp64", (3, 6)),     # odd pobtaf ring, chunks of 3
    ((9, 130, 5), np.float64, "fp64", (4, 4)),      # ragged tiles, column-block kernel
    ((10, 48, 0), np.float64, "fp64", (2, 4)),      # no arrowhead
    ((1, 40, 8), np.float64, "fp64", (2, 2)),       # a single block
    ((11, 32, 4), np.float32, "fp64", (3, 4)),
    ((7, 128, 16), np.float64, "mixed", (2, 4)),
])
def test_ring_matches_device_path_and_oracle(shape, dtype, precision, rings):
    n, b, a = shape
    m = generate(n, b, a, 1, seed=300 + n + b, dtype=dtype)
    Ld, Xd = _device_result(m, precision)
    ref = [x.copy() for x in m.arrays()]
    oracle.pobtaf(*ref)
    Lr = [x.copy() for x in ref]
    oracle.pobtasi(*ref)

    host = [x.copy() for x in m.arrays()]
    sg.pobtaf(*host, precision=precision, device_streaming=True, ring_blocks=rings[0])
    tol = {"fp64": 1e-12, "mixed": 1e-9}[precision] if dtype == np.float64 else 1e-5
    for g, d, r in zip(host, Ld, Lr):
        if r.size:
            assert rel_err(g, d) <= (1e-13 if dtype == np.float64 else 1e-6)
            assert rel_err(g, r) <= tol
    sg.pobtasi(*host, precision=precision, device_streaming=True, ring_blocks=rings[1])
    for g, d, r in zip(host, Xd, ref):
        if r.size:
            assert rel_err(g, d) <= (1e-13 if dtype == np.float64 else 1e-6)
            assert rel_err(g, r) <= tol


def test_ring_mode_flags_and_torch_host_tensors():
    m = generate(12, 72, 9, 1, seed=8)
    Ld, Xd = _device_result(m, "fp64", flb=False, ilb=False)
    host = [torch.from_numpy(x.copy()).pin_memory() for x in m.arrays()]
    sg.pobtaf(*host, factorize_last_block=False, device_streaming=True, ring_blocks=2)
    for g, d in zip(host, Ld):
        assert rel_err(g.numpy(), d) <= 1e-13
    sg.pobtasi(*host, invert_last_block=False, device_streaming=True, ring_blocks=4)
    for g, d in zip(host, Xd):
        assert rel_err(g.numpy(), d) <= 1e-13


def test_ring_non_contiguous_host_arrays_written_back():
    m = generate(6, 40, 4, 1, seed=9)
    Ld, _ = _device_result(m, "fp64")
    # Fortran-ordered copies: the call works on contiguous copies and writes back
    host = [np.asfortranarray(x.copy()) for x in m.arrays()]
    sg.pobtaf(*host, device_streaming=True, ring_blocks=2)
    for g, d in zip(host, Ld):
        if d.size:
            assert rel_err(g, d) <= 1e-13


def test_ring_reports_not_spd_row():
    m = generate(8, 64, 8, 1, seed=11)
    m.D[5][10, 10] = -1e6
    host = [x.copy() for x in m.arrays()]
    with pytest.raises(np.linalg.LinAlgError, match=f"{5 * 64 + 11}-th leading minor"):
        sg.pobtaf(*host, device_streaming=True, ring_blocks=3)


def test_ring_rejects_device_arrays_like_the_reference():
    m = generate(3, 16, 2, 1, seed=1)
    d = [torch.from_numpy(x).cuda() for x in m.arrays()]
    with pytest.raises(NotImplementedError, match="host-arrays"):
        sg.pobtaf(*d, device_streaming=True)
    with pytest.raises(NotImplementedError, match="host-arrays"):
        sg.pobtasi(*d, device_streaming=True)


def test_ring_too_small_is_rejected():
    m = generate(4, 16, 2, 1, seed=2)
    host = [x.copy() for x in m.arrays()]
    with pytest.raises(ValueError):
        sg.pobtaf(*host, device_streaming=True, ring_blocks=1)
