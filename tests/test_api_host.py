"""CPU: the Python drop-in mirrors the reference's argument handling
(src/serinv/algs/pobtaf.py:50-53, pobtasi.py:45-48, pobtas.py:27-62,160-161)
and fails loudly without a GPU instead of falling back to the CPU."""

import numpy as np
import pytest
import torch

import serinv_gb300 as sg
from serinv_gb300.synthetic import generate


@pytest.fixture
def m():
    return generate(3, 4, 2, 2, seed=1)


def test_unknown_kwarg_pobtaf(m):
    with pytest.raises(TypeError):
        sg.pobtaf(*m.arrays(), bogus=1)


def test_unknown_kwarg_pobtasi(m):
    with pytest.raises(TypeError):
        sg.pobtasi(*m.arrays(), factorize_last_block=True)


def test_bad_trans(m):
    with pytest.raises(ValueError):
        sg.pobtas(*m.arrays(), m.B, trans="Q")


def test_pobtas_streaming_not_implemented(m):
    with pytest.raises(NotImplementedError):
        sg.pobtas(*m.arrays(), m.B, device_streaming=True)


def test_permuted_streaming_solve_not_implemented(m):
    """pobtas.py:31-36 and pobts.py:29-32: streaming is refused for the permuted solve."""
    buf = np.empty_like(m.D)
    with pytest.raises(NotImplementedError, match="permuted"):
        sg.pobtas(*m.arrays(), m.B, buffer=buf, device_streaming=True)
    with pytest.raises(NotImplementedError, match="Permuted"):
        sg.pobts(m.D, m.Lo, m.B[:m.D.shape[0] * m.D.shape[1]], buffer=buf, device_streaming=True)


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU behaviour")
def test_permuted_no_gpu_fails_loudly(m):
    buf = np.zeros_like(m.D)
    before = m.D.copy()
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        sg.pobtaf(*m.arrays(), buffer=buf)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        sg.pobtasi(*m.arrays(), buffer=buf)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        sg.pobtas(*m.arrays(), m.B, buffer=buf)
    np.testing.assert_array_equal(m.D, before)


def test_bad_precision(m):
    with pytest.raises(ValueError):
        sg.pobtaf(*m.arrays(), precision="fp16")


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU behaviour")
def test_no_gpu_fails_loudly(m):
    before = m.D.copy()
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        sg.pobtaf(*m.arrays())
    np.testing.assert_array_equal(m.D, before)


def test_pinned_host_stack_detection_rejects_unsuitable_arrays(m):
    """Only C-contiguous, writable, real, pinned host stacks take the streamed
    path; everything else keeps the copy path."""
    from serinv_gb300.algs import _pinned_host_stacks
    arrs = list(m.arrays())
    assert _pinned_host_stacks(arrs) is None  # pageable NumPy memory
    ro = [x.copy() for x in arrs]
    ro[0].flags.writeable = False
    assert _pinned_host_stacks(ro) is None
    nc = [x.copy() for x in arrs]
    nc[0] = np.asfortranarray(nc[0])
    assert _pinned_host_stacks(nc) is None
    cx = [x.astype(np.complex128) for x in arrs]
    assert _pinned_host_stacks(cx) is None
