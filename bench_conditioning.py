"""Conditioning control for BTA test matrices (the kappa sweep of bench.py).

Measurement tooling beside the benchmark, not part of the library package.

``bta_matvec`` applies the symmetric BTA matrix given by its lower stacks;
``lanczos_extremes`` estimates the extreme eigenvalues of a symmetric
operator with a fully reorthogonalised Lanczos run on the GPU;
``shift_for_kappa`` picks sigma so that A0 + sigma I has a target
condition number, from the extremes of the (possibly indefinite) A0; and
``kappa_of`` measures the condition number actually achieved, using
lambda_min(A) = 1 / lambda_max(A^{-1}) with A^{-1} applied through the FP64
factor (pobtaf once, pobtas twice per product).
"""

from __future__ import annotations

import torch


def bta_matvec(D, Lo, Ar, T, x):
    """y = A x for the symmetric BTA matrix with lower stacks D, Lo, Ar, T (x: (N, k))."""
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


def lanczos_extremes(op, N: int, steps: int = 80, seed: int = 0, device="cuda"):
    """(smallest, largest) Ritz values of the symmetric operator op after `steps` Lanczos steps."""
    g = torch.Generator(device=device).manual_seed(seed)
    q = torch.rand((N, 1), generator=g, device=device, dtype=torch.float64) - 0.5
    q /= torch.linalg.norm(q)
    Q = [q]
    alphas, betas = [], []
    beta = 0.0
    q_prev = torch.zeros_like(q)
    for _ in range(steps):
        w = op(q) - beta * q_prev
        alpha = float((q * w).sum())
        w = w - alpha * q
        Qm = torch.cat(Q, dim=1)  # full reorthogonalisation
        w = w - Qm @ (Qm.T @ w)
        beta = float(torch.linalg.norm(w))
        alphas.append(alpha)
        if beta < 1e-12:
            break
        betas.append(beta)
        q_prev, q = q, w / beta
        Q.append(q)
    k = len(alphas)
    Tm = torch.zeros((k, k), dtype=torch.float64)
    for i in range(k):
        Tm[i, i] = alphas[i]
        if i + 1 < k:
            Tm[i, i + 1] = Tm[i + 1, i] = betas[i]
    ev = torch.linalg.eigvalsh(Tm)
    return float(ev[0]), float(ev[-1])


def shift_for_kappa(lmin0: float, lmax0: float, kappa: float) -> float:
    """sigma with (lmax0 + sigma) / (lmin0 + sigma) = kappa."""
    return (lmax0 - kappa * lmin0) / (kappa - 1.0)


def kappa_of(D, Lo, Ar, T, steps: int = 60):
    """(kappa, lambda_min, lambda_max) of the SPD BTA matrix, measured on the GPU."""
    from serinv_gb300.algs import pobtaf, pobtas

    n, b, a = D.shape[0], D.shape[1], Ar.shape[1]
    N = n * b + a
    _, lmax = lanczos_extremes(lambda v: bta_matvec(D, Lo, Ar, T, v), N, steps)
    L = [x.clone() for x in (D, Lo, Ar, T)]
    pobtaf(*L)

    def inv(v):
        y = v.clone()
        pobtas(*L, y, trans="N")
        pobtas(*L, y, trans="T")
        return y

    _, imax = lanczos_extremes(inv, N, steps, seed=1)
    lmin = 1.0 / imax
    return lmax / lmin, lmin, lmax
