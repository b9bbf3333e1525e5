"""GPU: the FP64 products with few columns (N <= 8, the solves' right-hand
sides) run the skinny kernel; against torch FP64 on the same operands."""

import pytest
import torch

import serinv_gb300 as sg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,K", [(1, 1), (31, 17), (32, 256), (100, 600), (300, 33), (513, 512)])
@pytest.mark.parametrize("N", [1, 4, 8])
@pytest.mark.parametrize("transA", [False, True])
def test_skinny_against_torch(M, K, N, transA):
    g = torch.Generator(device="cuda").manual_seed(M * 1000 + K * 10 + N)
    A = torch.rand((K, M) if transA else (M, K), dtype=torch.float64, device="cuda", generator=g) - 0.5
    B = torch.rand((K, N), dtype=torch.float64, device="cuda", generator=g) - 0.5
    C0 = torch.rand((M, N), dtype=torch.float64, device="cuda", generator=g) - 0.5
    C = C0.clone()
    sg.dgemm(A, B, C, alpha=-1.5, beta=0.75, transA=transA)
    ref = 0.75 * C0 - 1.5 * ((A.T if transA else A) @ B)
    scale = float(((A.T if transA else A).abs() @ B.abs()).max()) + 1.0
    assert float((C - ref).abs().max()) <= 1e-14 * scale * max(1, K) ** 0.5


def test_skinny_is_deterministic():
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.rand((700, 900), dtype=torch.float64, device="cuda", generator=g)
    B = torch.rand((900, 6), dtype=torch.float64, device="cuda", generator=g)
    C1 = sg.dgemm(A, B)
    C2 = sg.dgemm(A, B)
    assert torch.equal(C1, C2)
