"""Seeded synthetic BTA workloads.

The generator follows the workload description the benchmark is quoted on:

* ``rng = numpy.random.default_rng(seed)``; draw order R ``(n,b,b)``,
  Lo ``(n-1,b,b)``, Ar ``(n,a,b)``, S ``(a,a)``, B ``(n*b+a, nrhs)``, all
  uniform in [-1, 1);
* ``D_i = R_i + R_i^T`` and ``T = S + S^T``;
* every diagonal entry gets ``1 + sum |off-diagonal entries of its full
  symmetric row|`` added to it.  The entry itself lies in [-2, 2), so each
  row has ``diag >= offdiag_sum - 1``; the matrices are SPD with a wide
  margin (smallest eigenvalue ~13 at b=16).

The full row of block row ``i`` holds ``D_i``, ``Lo[i-1]`` (left),
``Lo[i]^T`` (right) and ``Ar[i]^T`` (arrow columns); a tip row holds ``T`` and
every ``Ar[j]``.

``kappa_shift`` replaces the dominance shift by ``sigma * I`` (the
conditioning sweep): the caller picks sigma for a target condition number.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class BTA:
    D: np.ndarray
    Lo: np.ndarray
    Ar: np.ndarray
    T: np.ndarray
    B: np.ndarray | None

    @property
    def n(self) -> int:
        return self.D.shape[0]

    @property
    def b(self) -> int:
        return self.D.shape[1]

    @property
    def a(self) -> int:
        return self.Ar.shape[1]

    def copy(self) -> "BTA":
        return BTA(self.D.copy(), self.Lo.copy(), self.Ar.copy(), self.T.copy(),
                   None if self.B is None else self.B.copy())

    def arrays(self):
        return self.D, self.Lo, self.Ar, self.T


def _u(rng: np.random.Generator, shape) -> np.ndarray:
    return rng.uniform(-1.0, 1.0, size=shape)


def generate(n: int, b: int, a: int, nrhs: int = 1, seed: int = 0,
             dtype=np.float64, shift: str | float = "dd") -> BTA:
    """Build one SPD BTA matrix and its right-hand side.

    ``shift="dd"`` applies the diagonal-dominance shift; a float applies
    ``D_i += shift * I`` and ``T += shift * I`` instead (no dominance shift).
    Values are drawn in float64 and rounded once to ``dtype``.  Complex
    dtypes give a Hermitian positive-definite matrix: the imaginary parts
    are drawn after the real ones (same order, same distribution), the
    diagonal blocks and tip are ``R + R^H``, and the shift uses the moduli.
    """
    if n < 1 or b < 1 or a < 0 or nrhs < 0:
        raise ValueError("need n >= 1, b >= 1, a >= 0, nrhs >= 0")
    rng = np.random.default_rng(seed)
    R = _u(rng, (n, b, b))
    Lo = _u(rng, (n - 1, b, b))
    Ar = _u(rng, (n, a, b))
    S = _u(rng, (a, a))
    B = _u(rng, (n * b + a, nrhs))
    if np.issubdtype(np.dtype(dtype), np.complexfloating):
        # imaginary parts drawn after the real ones, in the same order
        R = R + 1j * _u(rng, R.shape)
        Lo = Lo + 1j * _u(rng, Lo.shape)
        Ar = Ar + 1j * _u(rng, Ar.shape)
        S = S + 1j * _u(rng, S.shape)
        B = B + 1j * _u(rng, B.shape)

    D = R + R.conj().transpose(0, 2, 1)   # Hermitian: real diagonal
    del R
    T = S + S.conj().T

    if isinstance(shift, str):
        if shift != "dd":
            raise ValueError(f"unknown shift {shift!r}")
        # Off-diagonal absolute row sums of the full symmetric matrix.
        absD = np.abs(D)
        rows = absD.sum(axis=2) - np.abs(np.diagonal(D, axis1=1, axis2=2))  # (n, b)
        absLo = np.abs(Lo)
        if n > 1:
            rows[1:] += absLo.sum(axis=2)       # Lo[i-1] row r, left of block row i
            rows[:-1] += absLo.sum(axis=1)      # Lo[i]^T row r = column r of Lo[i]
        if a:
            absAr = np.abs(Ar)
            rows += absAr.sum(axis=1)           # Ar[i]^T row r = column r of Ar[i]
            tip_rows = np.abs(T).sum(axis=1) - np.abs(np.diag(T)) + absAr.sum(axis=(0, 2))
        idx = np.arange(b)
        D[:, idx, idx] += 1.0 + rows
        if a:
            ti = np.arange(a)
            T[ti, ti] += 1.0 + tip_rows
    else:
        sigma = float(shift)
        idx = np.arange(b)
        D[:, idx, idx] += sigma
        if a:
            ti = np.arange(a)
            T[ti, ti] += sigma

    dt = np.dtype(dtype)
    return BTA(np.ascontiguousarray(D, dtype=dt), np.ascontiguousarray(Lo, dtype=dt),
               np.ascontiguousarray(Ar, dtype=dt), np.ascontiguousarray(T, dtype=dt),
               np.ascontiguousarray(B, dtype=dt))


def batch_shapes(count: int = 256, seed: int = 0):
    """Shapes of the uneven batch: matrix i has n ~ U{16..256}, b drawn from
    {32, 64, 128, 256} and a from {0, 4, 16} (one ``default_rng(seed)``
    stream, drawn n, b, a per matrix in order); the first ``count // 2`` are
    float32, the rest float64.  Matrix i's values come from
    ``generate(n, b, a, 4, seed=i, dtype=...)``.  Returns a list of
    ``(n, b, a, numpy dtype)``."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(16, 257))
        b = int(rng.choice([32, 64, 128, 256]))
        a = int(rng.choice([0, 4, 16]))
        out.append((n, b, a, np.dtype(np.float32) if i < count // 2 else np.dtype(np.float64)))
    return out


def flops(n: int, b: int, a: int, nrhs: int = 0) -> dict:
    """Canonical (LAPACK-convention) flop counts of the three routines.

    pobtaf  = n (7/3 b^3 + 3 a b^2 + a^2 b) + a^3/3
    pobtasi = n (19/3 b^3 + 7 a b^2 + 2 a^2 b) + a^3/3 + a^3
    pobtas  = 2 nrhs (n b^2 + 2 (n-1) b^2 + 2 n a b) + 2 nrhs a^2   (forward + backward)
    """
    f = n * (7.0 / 3.0 * b ** 3 + 3.0 * a * b * b + a * a * b) + a ** 3 / 3.0
    si = n * (19.0 / 3.0 * b ** 3 + 7.0 * a * b * b + 2.0 * a * a * b) + a ** 3 / 3.0 + a ** 3
    s = 2.0 * nrhs * (n * b * b + 2.0 * (n - 1) * b * b + 2.0 * n * a * b) + 2.0 * nrhs * a * a
    return {"pobtaf": f, "pobtasi": si, "pobtas": s}


def nbytes_sweep(n: int, b: int, a: int, itemsize: int = 8) -> float:
    """Algorithmic bytes of one sweep: every stored block read once and written once."""
    return 2.0 * itemsize * (n * b * b + max(n - 1, 0) * b * b + n * a * b + a * a)


def generate_torch(n: int, b: int, a: int, nrhs: int = 1, seed: int = 0, dtype=None, device="cuda",
                   shift: str | float = "dd"):
    """The same construction as ``generate`` drawn with torch's generator on the GPU.

    Same draw order, distributions and dominance shift; different random
    numbers (torch's Philox stream, not NumPy's PCG64).  Used where the
    inputs are too large to draw on the host in reasonable time; parity
    tests use ``generate``.  Complex dtypes as in ``generate``.  Returns
    (D, Lo, Ar, T, B) torch tensors.
    """
    import torch

    dtype = dtype or torch.float64
    g = torch.Generator(device=device).manual_seed(seed)

    def u(*shape):
        return torch.rand(shape, generator=g, device=device, dtype=torch.float64) * 2.0 - 1.0

    R = u(n, b, b)
    Lo = u(n - 1, b, b)
    Ar = u(n, a, b)
    S = u(a, a)
    B = u(n * b + a, nrhs)
    if dtype.is_complex:
        # imaginary parts drawn after the real ones, in the same order
        R = torch.complex(R, u(n, b, b))
        Lo = torch.complex(Lo, u(n - 1, b, b))
        Ar = torch.complex(Ar, u(n, a, b))
        S = torch.complex(S, u(a, a))
        B = torch.complex(B, u(n * b + a, nrhs))
    D = R + R.transpose(1, 2).conj()   # Hermitian: real diagonal
    del R
    T = S + S.T.conj()
    idx = torch.arange(b, device=device)
    if isinstance(shift, str):
        rows = D.abs().sum(dim=2) - torch.diagonal(D, dim1=1, dim2=2).abs()
        if n > 1:
            absLo = Lo.abs()
            rows[1:] += absLo.sum(dim=2)
            rows[:-1] += absLo.sum(dim=1)
        if a:
            absAr = Ar.abs()
            rows += absAr.sum(dim=1)
            tip_rows = T.abs().sum(dim=1) - torch.diagonal(T).abs() + absAr.sum(dim=(0, 2))
        D[:, idx, idx] += 1.0 + rows
        if a:
            ti = torch.arange(a, device=device)
            T[ti, ti] += 1.0 + tip_rows
    else:
        D[:, idx, idx] += float(shift)
        if a:
            ti = torch.arange(a, device=device)
            T[ti, ti] += float(shift)
    return tuple(x.to(dtype).contiguous() for x in (D, Lo, Ar, T, B))
