"""GPU: the differentiable logdet(A) + y^T A^{-1} y whose backward is the
selected inversion, against dense FP64 torch autograd and central finite
differences."""

import numpy as np
import pytest
import torch

from serinv_gb300.autograd import bta_logdet_quad
from serinv_gb300.synthetic import generate

pytestmark = pytest.mark.gpu


def dense_loss(D, Lo, Ar, T, y):
    """The same loss through dense torch ops, reading only the lower triangles of D and T."""
    n, b, a = D.shape[0], D.shape[1], Ar.shape[1]
    N = n * b + a
    Ds = torch.tril(D) + torch.tril(D, -1).transpose(1, 2)
    rows = []
    blocks = {}
    for i in range(n):
        blocks[(i, i)] = Ds[i]
        if i < n - 1:
            blocks[(i + 1, i)] = Lo[i]
            blocks[(i, i + 1)] = Lo[i].T
        if a:
            blocks[(n, i)] = Ar[i]
            blocks[(i, n)] = Ar[i].T
    if a:
        blocks[(n, n)] = torch.tril(T) + torch.tril(T, -1).T
    sizes = [b] * n + ([a] if a else [])
    for bi, sb in enumerate(sizes):
        row = []
        for bj, sj in enumerate(sizes):
            row.append(blocks.get((bi, bj), D.new_zeros((sb, sj))))
        rows.append(torch.cat(row, dim=1))
    A = torch.cat(rows, dim=0)
    Lc = torch.linalg.cholesky(A)
    logdet = 2.0 * torch.log(torch.diagonal(Lc)).sum()
    yy = y.reshape(N, -1)
    x = torch.cholesky_solve(yy, Lc)
    return logdet + (yy * x).sum()


def make(n, b, a, seed, k=1):
    m = generate(n, b, a, k, seed=seed)
    ts = [torch.from_numpy(x).cuda().requires_grad_(True) for x in m.arrays()]
    y = torch.from_numpy(m.B[:, 0].copy() if k == 1 else m.B.copy()).cuda().requires_grad_(True)
    return ts, y


@pytest.mark.parametrize("shape", [(4, 8, 3, 1), (16, 32, 8, 1), (3, 40, 0, 1), (5, 24, 4, 3),
                                   (16, 256, 32, 1)])  # the last: the benchmark's b and a at n = 16
def test_against_dense_autograd(shape):
    n, b, a, k = shape
    ts, y = make(n, b, a, seed=n + b, k=k)
    loss = bta_logdet_quad(*ts, y)
    loss.backward()
    ours = [t.grad.clone() for t in ts] + [y.grad.clone()]
    ts2 = [t.detach().clone().requires_grad_(True) for t in ts]
    y2 = y.detach().clone().requires_grad_(True)
    ref = dense_loss(*ts2, y2)
    ref.backward()
    lv, rv = float(loss.detach()), float(ref.detach())
    assert abs(lv - rv) <= 1e-11 * abs(rv)
    for got, t in zip(ours, ts2 + [y2]):
        if t.grad is None:
            continue
        den = float(torch.linalg.norm(t.grad))
        if den == 0:
            continue
        e = float(torch.linalg.norm(got - t.grad)) / den
        assert e <= 1e-10, e


def test_central_finite_differences():
    n, b, a = 8, 64, 16
    ts, y = make(n, b, a, seed=3)
    loss = bta_logdet_quad(*ts, y)
    loss.backward()
    rng = np.random.default_rng(0)
    h = 1e-6
    for _ in range(16):
        which = int(rng.integers(0, 4))
        t = ts[which]
        if t.numel() == 0:
            continue
        idx = tuple(int(rng.integers(0, s)) for s in t.shape)
        if which in (0, 3) and idx[-1] > idx[-2]:
            idx = idx[:-2] + (idx[-1], idx[-2])  # the lower triangle is the parameter
        with torch.no_grad():
            base = [x.detach().clone() for x in ts]
            plus = [x.clone() for x in base]
            minus = [x.clone() for x in base]
            plus[which][idx] += h
            minus[which][idx] -= h
            fp = float(bta_logdet_quad(*plus, y.detach()))
            fm = float(bta_logdet_quad(*minus, y.detach()))
        fd = (fp - fm) / (2 * h)
        g = float(t.grad[idx])
        assert abs(fd - g) <= 1e-5 * max(1.0, abs(g)), (which, idx, fd, g)


def test_central_finite_differences_at_benchmark_size():
    """n=1024, b=256, a=32 (N = 262,176): 64 seeded entries of the four
    stacks, central differences with h = 1e-6 against the selected-inversion
    gradient.  The loss is ~1e6, so the difference quotient's rounding floor
    is ~eps |loss| / h ~ 2e-4; the bar is 1e-3 relative to max(1, |g|)."""
    n, b, a = 1024, 256, 32
    ts, y = make(n, b, a, seed=0)
    loss = bta_logdet_quad(*ts, y)
    loss.backward()
    rng = np.random.default_rng(0)
    h = 1e-6
    base = [x.detach().clone() for x in ts]
    worst = 0.0
    for _ in range(64):
        which = int(rng.integers(0, 4))
        t = ts[which]
        idx = tuple(int(rng.integers(0, s_)) for s_ in t.shape)
        if which in (0, 3) and idx[-1] > idx[-2]:
            idx = idx[:-2] + (idx[-1], idx[-2])
        with torch.no_grad():
            old = float(base[which][idx])
            base[which][idx] = old + h
            fp = float(bta_logdet_quad(*base, y.detach()))
            base[which][idx] = old - h
            fm = float(bta_logdet_quad(*base, y.detach()))
            base[which][idx] = old
        g = float(t.grad[idx])
        dev = abs((fp - fm) / (2 * h) - g) / max(1.0, abs(g))
        worst = max(worst, dev)
    assert worst <= 1e-3, worst
