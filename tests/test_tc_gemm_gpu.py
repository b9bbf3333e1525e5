"""GPU: the tensor-core (tcgen05) slice-product FP64 GEMM against cuBLAS FP64
(torch) and against exact integer arithmetic.

* integer-valued operands: every slice product and every level sum is an
  exact integer below 2^24 units, so the result must equal the exact product
  bit for bit (this also checks that the FP32 tensor-core accumulation adds
  those values exactly);
* random operands: normwise relative error within the slice truncation
  bound, K * 2^-(7S-1) relative to |A||B| (a generous form of 2^-(7S+1));
* rows and columns of very different magnitude (per-row scaling);
* all transposition combinations, ragged sizes, K up to the exactness bound
  and beyond it (chunked), alpha/beta.
"""

import math

import pytest
import torch

import serinv_gb300 as sg

pytestmark = pytest.mark.gpu


def ref(A, B, C, alpha, beta, ta, tb):
    a = A.T if ta else A
    b = B.T if tb else B
    out = alpha * (a @ b)
    if C is not None and beta != 0:
        out = out + beta * C
    return out


def bound(A, B, ta, tb, S):
    """Per-element error bound relative to sum_k |a_k||b_k|.

    Digit truncation: 2^-(7S+1) of the row (column) maximum per operand,
    i.e. a few 2^-(7S) relative to |a||b| for uniform entries; plus the
    rounding of the FP64 reference product itself (K * 2^-53)."""
    K = (A.T if ta else A).shape[1]
    return 8.0 * 2.0 ** (-7 * S) + max(K, 1) * 2.0 ** -52


@pytest.mark.parametrize("S", [3, 5, 7])
@pytest.mark.parametrize("shape", [(128, 64, 32), (512, 512, 512), (100, 37, 65), (1, 1, 1), (300, 200, 576)])
@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
def test_random_vs_fp64(S, shape, ta, tb):
    M, N, K = shape
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K + S)
    A = torch.rand((K, M) if ta else (M, K), generator=g, device="cuda", dtype=torch.float64) * 2 - 1
    B = torch.rand((N, K) if tb else (K, N), generator=g, device="cuda", dtype=torch.float64) * 2 - 1
    C0 = torch.rand((M, N), generator=g, device="cuda", dtype=torch.float64)
    C = C0.clone()
    sg.dgemm(A, B, C, alpha=-1.0, beta=1.0, transA=ta, transB=tb, precision=f"mixed:{S}")
    R = ref(A, B, C0, -1.0, 1.0, ta, tb)
    absprod = (A.T if ta else A).abs() @ (B.T if tb else B).abs()
    err = float(((C - R).abs() / (absprod + 1e-300)).max())
    assert err <= bound(A, B, ta, tb, S), (err, bound(A, B, ta, tb, S))


@pytest.mark.parametrize("S", [3, 5, 7])
def test_integer_operands_exact(S):
    """Small integers are represented exactly by the first slice; the result is exact."""
    g = torch.Generator(device="cuda").manual_seed(5)
    M, N, K = 256, 192, 512
    A = torch.randint(-100, 101, (M, K), generator=g, device="cuda").double()
    B = torch.randint(-100, 101, (K, N), generator=g, device="cuda").double()
    # force every row/column maximum to 100 so all rows share one scale
    A[:, 0] = 100
    B[0, :] = 100
    C = sg.dgemm(A, B, precision=f"mixed:{S}")
    exact = A @ B  # integer-valued, |partial sums| < 2^53: exact in FP64
    assert torch.equal(C, exact)


def test_full_width_integer_digits_exact():
    """Operands whose first digit uses the full 8 bits (|d0| up to 128)."""
    g = torch.Generator(device="cuda").manual_seed(6)
    M, N, K = 128, 64, 576
    A = torch.randint(-127, 128, (M, K), generator=g, device="cuda").double()
    B = torch.randint(-127, 128, (K, N), generator=g, device="cuda").double()
    A[:, 0] = 127
    B[0, :] = -127
    C = sg.dgemm(A, B, precision="mixed:3")
    exact = A @ B  # integer-valued, |partial sums| < 2^53: exact in FP64
    assert torch.equal(C, exact)


def test_row_and_column_scaling():
    g = torch.Generator(device="cuda").manual_seed(7)
    M, N, K = 192, 128, 256
    A = torch.rand((M, K), generator=g, device="cuda", dtype=torch.float64) - 0.5
    B = torch.rand((K, N), generator=g, device="cuda", dtype=torch.float64) - 0.5
    rs = torch.logspace(-150, 150, M, device="cuda", dtype=torch.float64)
    cs = torch.logspace(100, -100, N, device="cuda", dtype=torch.float64)
    A = A * rs[:, None]
    B = B * cs[None, :]
    C = sg.dgemm(A, B, precision="mixed:7")
    R = A @ B
    absprod = A.abs() @ B.abs()
    err = float(((C - R).abs() / absprod).max())
    assert err <= 8.0 * 2.0 ** -49 + K * 2.0 ** -52


def test_long_k_is_chunked():
    g = torch.Generator(device="cuda").manual_seed(8)
    M, N, K = 64, 64, 2000
    A = torch.rand((M, K), generator=g, device="cuda", dtype=torch.float64) - 0.5
    B = torch.rand((K, N), generator=g, device="cuda", dtype=torch.float64) - 0.5
    C = sg.dgemm(A, B, precision="mixed:7")
    R = A @ B
    err = float((C - R).abs().max() / (A.abs() @ B.abs()).max())
    assert err <= 1e-14


def test_native_dgemm_matches_torch():
    g = torch.Generator(device="cuda").manual_seed(9)
    A = torch.rand((70, 90), generator=g, device="cuda", dtype=torch.float64)
    B = torch.rand((90, 50), generator=g, device="cuda", dtype=torch.float64)
    C = sg.dgemm(A, B, precision="fp64")
    assert float((C - A @ B).abs().max()) <= 1e-13


def test_zero_rows_and_k0():
    A = torch.zeros((130, 40), device="cuda", dtype=torch.float64)
    B = torch.rand((40, 70), device="cuda", dtype=torch.float64)
    C = sg.dgemm(A, B, precision="mixed")
    assert torch.equal(C, torch.zeros_like(C))
    A0 = torch.zeros((5, 0), device="cuda", dtype=torch.float64)
    B0 = torch.zeros((0, 6), device="cuda", dtype=torch.float64)
    C = torch.ones((5, 6), device="cuda", dtype=torch.float64)
    sg.dgemm(A0, B0, C, beta=2.0, precision="mixed")
    assert torch.equal(C, 2 * torch.ones_like(C))
    assert math.isfinite(float(C.sum()))
