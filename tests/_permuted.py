"""The middle-partition workflow of the reference's permuted tests, written
against a set of functions (the oracle's or the library's), so that tests
drive both the same way: permuted factorization -> reduced system of blocks
0 and n-1 and the tip (factored, inverted or solved with the natural
algorithms) -> permuted selected inversion / permuted solve."""

from __future__ import annotations

import numpy as np


def reduced(D, Ar, T, buf, zeros):
    b, a = D.shape[1], Ar.shape[1]
    rD = zeros((2, b, b), D)
    rLo = zeros((1, b, b), D)
    rAr = zeros((2, a, b), D)
    rT = zeros((a, a), D)
    rD[0], rD[1] = D[0], D[-1]
    rLo[0] = buf[-1].conj().T
    rAr[0], rAr[1] = Ar[0], Ar[-1]
    rT[:, :] = T
    return rD, rLo, rAr, rT


def map_back(D, Ar, T, buf, rD, rLo, rAr, rT):
    D[0], D[-1] = rD[0], rD[1]
    buf[-1] = rLo[0].conj().T
    Ar[0], Ar[-1] = rAr[0], rAr[1]
    T[:, :] = rT


def workflow(fn, D, Lo, Ar, T, B, zeros, copy):
    """fn: dict with pobtaf, pobtasi, pobtas (natural) and pobtaf_p,
    pobtasi_p, pobtas_p (permuted, buffer as the last stack argument).
    Returns (factor stacks + buffer, selected inverse stacks + buffer, x)."""
    n, b = D.shape[0], D.shape[1]
    buf = zeros(D.shape, D)
    fn["pobtaf_p"](D, Lo, Ar, T, buf)
    F = [copy(x) for x in (D, Lo, Ar, T, buf)]
    rL = reduced(D, Ar, T, buf, zeros)
    fn["pobtaf"](*rL)
    # selected inversion
    X = [copy(x) for x in F]
    s = [copy(x) for x in rL]
    fn["pobtasi"](*s)
    map_back(X[0], X[2], X[3], X[4], *s)
    fn["pobtasi_p"](*X)
    # solve
    L = [copy(x) for x in F]
    map_back(L[0], L[2], L[3], L[4], *rL)
    x = copy(B)
    fn["pobtas_p"](*L, x, "N")
    rB = np.concatenate([np.asarray(v) for v in (to_np(x[:b]), to_np(x[(n - 1) * b:n * b]), to_np(x[n * b:]))])
    rB = like(x, rB)
    fn["pobtas"](*rL, rB, "N")
    fn["pobtas"](*rL, rB, "C")
    x[:b], x[(n - 1) * b:n * b], x[n * b:] = rB[:b], rB[b:2 * b], rB[2 * b:]
    fn["pobtas_p"](*L, x, "C")
    return F, X, x


def to_np(t):
    return t.cpu().numpy() if hasattr(t, "cpu") else np.asarray(t)


def like(ref, arr):
    if hasattr(ref, "cpu"):
        import torch
        return torch.from_numpy(np.ascontiguousarray(arr)).to(ref.device)
    return np.ascontiguousarray(arr)
