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


def test_permuted_buffer_not_implemented(m):
    buf = np.empty_like(m.D)
    with pytest.raises(NotImplementedError):
        sg.pobtaf(*m.arrays(), buffer=buf)
    with pytest.raises(NotImplementedError):
        sg.pobtasi(*m.arrays(), buffer=buf)
    with pytest.raises(NotImplementedError):
        sg.pobtas(*m.arrays(), m.B, buffer=buf)


def test_bad_precision(m):
    with pytest.raises(ValueError):
        sg.pobtaf(*m.arrays(), precision="fp16")


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU behaviour")
def test_no_gpu_fails_loudly(m):
    before = m.D.copy()
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        sg.pobtaf(*m.arrays())
    np.testing.assert_array_equal(m.D, before)
