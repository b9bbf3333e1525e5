"""GPU, full benchmark shape (n=512, b=512, a=64, 16 RHS, FP64): properties
that do not need a CPU reference of the same size.

* backward error of the solve, ||A x - b|| / (||A|| ||x||), at FP64 level;
* selected-inverse columns: for sampled global columns j, the blocks of
  X = A^{-1} on the BTA pattern equal the matching entries of A^{-1} e_j
  obtained from an independent pobtas solve (1e-12 relative);
* the factor reproduces A on probe vectors: ||L L^T v - A v|| / (||A|| ||v||);
* the kernels are deterministic (bit-identical reruns).
"""

import numpy as np
import pytest
import torch

import serinv_gb300 as sg
from serinv_gb300.synthetic import generate

pytestmark = pytest.mark.gpu

N_, B_, A_, R_ = 512, 512, 64, 16


def bta_matvec(D, Lo, Ar, T, x):
    """y = A x for the symmetric BTA matrix given by its lower stacks (torch, on the GPU)."""
    n, b = D.shape[0], D.shape[1]
    a = Ar.shape[1]
    xb = x[: n * b].view(n, b, -1)
    xt = x[n * b:]
    y = torch.bmm(D, xb)
    if n > 1:
        y[1:] += torch.bmm(Lo, xb[:-1])
        y[:-1] += torch.bmm(Lo.transpose(1, 2), xb[1:])
    out = torch.empty_like(x)
    if a:
        y += torch.matmul(Ar.transpose(1, 2), xt)
        out[n * b:] = torch.einsum("nab,nbr->ar", Ar, xb) + T @ xt
    out[: n * b] = y.reshape(n * b, -1)
    return out


def l_matvec(L, Lo, Ar, Lt, x, trans):
    n, b = L.shape[0], L.shape[1]
    a = Ar.shape[1]
    xb = x[: n * b].view(n, b, -1)
    xt = x[n * b:]
    out = torch.zeros_like(x)
    if not trans:  # y = L x
        y = torch.bmm(L, xb)
        if n > 1:
            y[1:] += torch.bmm(Lo, xb[:-1])
        out[: n * b] = y.reshape(n * b, -1)
        if a:
            out[n * b:] = torch.einsum("nab,nbr->ar", Ar, xb) + Lt @ xt
    else:  # y = L^T x
        y = torch.bmm(L.transpose(1, 2), xb)
        if n > 1:
            y[:-1] += torch.bmm(Lo.transpose(1, 2), xb[1:])
        if a:
            y += torch.matmul(Ar.transpose(1, 2), xt)
            out[n * b:] = Lt.T @ xt
        out[: n * b] = y.reshape(n * b, -1)
    return out


@pytest.fixture(scope="module")
def full():
    m = generate(N_, B_, A_, R_, seed=0)
    A = [torch.from_numpy(x).cuda() for x in m.arrays()]
    Bt = torch.from_numpy(m.B).cuda()
    del m
    L = [x.clone() for x in A]
    sg.pobtaf(*L)
    torch.cuda.synchronize()
    return A, L, Bt


def test_solve_backward_error(full):
    A, L, Bt = full
    x = Bt.clone()
    sg.pobtas(*L, x, trans="N")
    sg.pobtas(*L, x, trans="C")
    r = bta_matvec(*A, x) - Bt
    # ||A||_inf bound: the diagonal entries dominate every row (each is
    # 1 + the off-diagonal row sum + a value in [-2, 2)), so 2 max|a_ii| + 2
    # bounds every absolute row sum.
    anorm = 2.0 * float(A[0].diagonal(dim1=1, dim2=2).abs().max()) + 2.0
    berr = float(torch.linalg.norm(r, ord=float("inf")) / (anorm * torch.linalg.norm(x, ord=float("inf"))))
    assert berr < 1e-14, berr


def test_factor_reproduces_matrix(full):
    A, L, _ = full
    g = torch.Generator(device="cuda").manual_seed(1)
    v = torch.rand((N_ * B_ + A_, 4), generator=g, device="cuda", dtype=torch.float64) - 0.5
    lhs = l_matvec(*L, l_matvec(*L, v, trans=True), trans=False)
    rhs = bta_matvec(*A, v)
    err = float(torch.linalg.norm(lhs - rhs) / torch.linalg.norm(rhs))
    assert err < 1e-14, err


def test_selected_inverse_columns(full):
    A, L, _ = full
    X = [x.clone() for x in L]
    sg.pobtasi(*X)
    XD, XLo, XA, XT = X
    n, b, a = N_, B_, A_
    cols = [0, 5, 77 * b + 301, (n // 2) * b + 3, (n - 1) * b + b - 1, n * b + 7]
    E = torch.zeros((n * b + a, len(cols)), dtype=torch.float64, device="cuda")
    for c, j in enumerate(cols):
        E[j, c] = 1.0
    Y = E.clone()
    sg.pobtas(*L, Y, trans="N")
    sg.pobtas(*L, Y, trans="C")
    for c, j in enumerate(cols):
        y = Y[:, c]
        if j < n * b:
            k, jj = divmod(j, b)
            pairs = [(y[k * b:(k + 1) * b], XD[k][:, jj])]
            if k + 1 < n:
                pairs.append((y[(k + 1) * b:(k + 2) * b], XLo[k][:, jj]))
            if k > 0:
                pairs.append((y[(k - 1) * b:k * b], XLo[k - 1][jj, :]))
            pairs.append((y[n * b:], XA[k][:, jj]))
        else:
            t = j - n * b
            pairs = [(y[n * b:], XT[:, t]), (y[:b], XA[0][t, :]), (y[(n - 1) * b:n * b], XA[n - 1][t, :])]
        for ref, got in pairs:
            e = float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))
            assert e < 1e-12, (j, e)
    # X_D is symmetric up to rounding
    asym = float(torch.linalg.norm(XD - XD.transpose(1, 2)) / torch.linalg.norm(XD))
    assert asym < 1e-13


def test_deterministic(full):
    A, L, _ = full
    L2 = [x.clone() for x in A]
    sg.pobtaf(*L2)
    for u, v in zip(L, L2):
        assert torch.equal(u, v)
