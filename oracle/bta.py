"""NumPy/SciPy restatement of the reference's BTA algorithms (natural ordering
and the permuted middle-partition variants).

Test infrastructure only (see the package docstring): the CUDA product path
never imports this module.

Every function follows the reference's per-block operation sequence and calls
the same dense primitives (``scipy.linalg.cholesky(lower=True)``,
``scipy.linalg.solve_triangular`` and ``@``), so on identical inputs it
reproduces the reference's results to the last bit on the same BLAS build.
Citations are ``file:line`` inside the reference project (``src/serinv/...``).

Storage (C-contiguous, in place), with n diagonal blocks of size b and arrow
width a:

* ``D``  ``(n, b, b)``   diagonal blocks
* ``Lo`` ``(n-1, b, b)`` lower-diagonal blocks, ``Lo[i] = A[i+1, i]``
* ``Ar`` ``(n, a, b)``   lower arrow blocks, ``Ar[i] = A[tip, i]``
* ``T``  ``(a, a)``      arrow tip
* ``B``  ``(n*b + a, nrhs)`` right-hand sides
"""

from __future__ import annotations

import numpy as np
import scipy.linalg as la


def _chol(x: np.ndarray) -> np.ndarray:
    # src/serinv/__init__.py:150-151: partial(scipy cholesky, lower=True,
    # overwrite_a=False, check_finite=False).  Returns L with a zero upper
    # triangle; raises numpy.linalg.LinAlgError on a non-SPD block.
    return la.cholesky(x, lower=True, overwrite_a=False, check_finite=False)


def pobtaf(D, Lo, Ar, T, factorize_last_block: bool = True) -> None:
    """In-place block Cholesky, after ``_pobtaf`` (src/serinv/algs/pobtaf.py:97-183)."""
    n = D.shape[0]
    for i in range(n - 1):  # pobtaf.py:115
        D[i] = _chol(D[i])  # :117
        # :120-128  L_{i+1,i} = A_{i+1,i} L_ii^{-T}
        Lo[i] = la.solve_triangular(D[i], Lo[i].conj().T, lower=True).conj().T
        # :131-139  L_{a,i} = A_{a,i} L_ii^{-T}
        Ar[i] = la.solve_triangular(D[i], Ar[i].conj().T, lower=True).conj().T
        D[i + 1] = D[i + 1] - Lo[i] @ Lo[i].conj().T  # :143-147
        Ar[i + 1] = Ar[i + 1] - Ar[i] @ Lo[i].conj().T  # :150-153
        T[:, :] = T - Ar[i] @ Ar[i].conj().T  # :156-159
    if factorize_last_block:  # :161
        D[-1] = _chol(D[-1])  # :163
        Ar[-1] = la.solve_triangular(D[-1], Ar[-1].conj().T, lower=True).conj().T  # :166-174
        T[:, :] = T - Ar[-1] @ Ar[-1].conj().T  # :177-180
        T[:, :] = _chol(T)  # :183


def pobtasi(D, Lo, Ar, T, invert_last_block: bool = True) -> None:
    """In-place selected inversion, after ``_pobtasi`` (src/serinv/algs/pobtasi.py:92-172)."""
    n = D.shape[0]
    b = D.shape[1]
    eye = np.eye(b, dtype=D.dtype)
    if invert_last_block:  # pobtasi.py:114
        Ltip_inv = la.solve_triangular(T, np.eye(T.shape[0], dtype=T.dtype), lower=True)  # :115-117
        T[:, :] = Ltip_inv.conj().T @ Ltip_inv  # :119
        ar_last = Ar[-1].copy()  # :122
        Linv = la.solve_triangular(D[-1], eye, lower=True)  # :124-128
        Ar[-1] = -T @ ar_last @ Linv  # :131-133
        D[-1] = (Linv.conj().T - Ar[-1].conj().T @ ar_last) @ Linv  # :136-139
    for i in range(n - 2, -1, -1):  # :141
        lo_i = Lo[i].copy()  # :142
        ar_i = Ar[i].copy()  # :143
        Linv = la.solve_triangular(D[i], eye, lower=True)  # :145-149
        Lo[i] = (-D[i + 1] @ lo_i - Ar[i + 1].conj().T @ ar_i) @ Linv  # :153-156
        Ar[i] = (-Ar[i + 1] @ lo_i - T @ ar_i) @ Linv  # :160-163
        D[i] = (Linv.conj().T - Lo[i].conj().T @ lo_i - Ar[i].conj().T @ ar_i) @ Linv  # :167-172


def pobtas(D, Lo, Ar, T, B, trans: str = "N", partial: bool = False) -> None:
    """In-place block triangular solve, after ``_pobtas`` (src/serinv/algs/pobtas.py:65-161).

    For ``a == 0`` the reference's arrow slice ``B[-0:]`` aliases the whole
    right-hand side and the call fails (pobtas.py:94,114,124).  This
    restatement then follows the arrow-free solve ``_pobts``
    (src/serinv/algs/pobts.py:57-118), which is what the formulas reduce to.
    """
    n, b = D.shape[0], D.shape[1]
    a = Ar.shape[1]
    if trans not in ("N", "T", "C"):
        raise ValueError(f"Invalid transpose argument: {trans}.")  # pobtas.py:160-161
    tip = slice(n * b, n * b + a)

    def blk(i):
        return slice(i * b, (i + 1) * b)

    if trans == "N":  # pobtas.py:80
        for i in range(n - 1):
            B[blk(i)] = la.solve_triangular(D[i], B[blk(i)], lower=True)  # :83-87
            B[blk(i + 1)] -= Lo[i] @ B[blk(i)]  # :89-92
            if a:
                B[tip] -= Ar[i] @ B[blk(i)]  # :94-97
        if not partial:  # :99
            B[blk(n - 1)] = la.solve_triangular(D[n - 1], B[blk(n - 1)], lower=True)  # :102-112
            if a:
                B[tip] -= Ar[-1] @ B[blk(n - 1)]  # :114-121
                B[tip] = la.solve_triangular(T, B[tip], lower=True)  # :124-126
    else:  # "T" / "C", pobtas.py:127
        if not partial:
            if a:
                B[tip] = la.solve_triangular(T, B[tip], lower=True, trans="C")  # :131-136
                rhs = B[blk(n - 1)] - Ar[-1].conj().T @ B[tip]  # :139-147
            else:
                rhs = B[blk(n - 1)]  # pobts.py:98-104
            B[blk(n - 1)] = la.solve_triangular(D[-1], rhs, lower=True, trans="C")
        for i in range(n - 2, -1, -1):  # pobtas.py:149
            rhs = B[blk(i)] - Lo[i].conj().T @ B[blk(i + 1)]  # :151-159
            if a:
                rhs = rhs - Ar[i].conj().T @ B[tip]
            B[blk(i)] = la.solve_triangular(D[i], rhs, lower=True, trans="C")


def pobtaf_permuted(D, Lo, Ar, T, buf) -> None:
    """Block Cholesky of a middle partition with the two-sided fill-in column
    ``buf`` (n, b, b), after ``_pobtaf_permuted`` (src/serinv/algs/pobtaf.py:
    186-281).  Blocks 1..n-2 are eliminated; block 0 (top), block n-1 and the
    tip receive the Schur updates and form the reduced system."""
    n = D.shape[0]
    buf[1] = Lo[0].conj().T  # pobtaf.py:203
    for i in range(1, n - 1):  # :206
        D[i] = _chol(D[i])  # :208
        Lo[i] = la.solve_triangular(D[i], Lo[i].conj().T, lower=True).conj().T  # :212-220
        buf[i] = la.solve_triangular(D[i], buf[i].conj().T, lower=True).conj().T  # :223-231
        Ar[i] = la.solve_triangular(D[i], Ar[i].conj().T, lower=True).conj().T  # :234-242
        D[i + 1] = D[i + 1] - Lo[i] @ Lo[i].conj().T  # :246-250
        Ar[i + 1] = Ar[i + 1] - Ar[i] @ Lo[i].conj().T  # :253-256
        T[:, :] = T - Ar[i] @ Ar[i].conj().T  # :260-263
        D[0] = D[0] - buf[i] @ buf[i].conj().T  # :267-269
        buf[i + 1] = -buf[i] @ Lo[i].conj().T  # :272-274
        Ar[0] = Ar[0] - Ar[i] @ buf[i].conj().T  # :278-281


def pobtasi_permuted(D, Lo, Ar, T, buf) -> None:
    """Selected inversion of a middle partition, after ``_pobtasi_permuted``
    (src/serinv/algs/pobtasi.py:175-244).  On entry blocks 0, n-1, the tip,
    ``Ar[0]``, ``Ar[-1]`` and ``buf[-1]`` already hold the selected inverse of
    the reduced system; blocks n-2..1 are filled in."""
    n, b = D.shape[0], D.shape[1]
    eye = np.eye(b, dtype=D.dtype)
    for i in range(n - 2, 0, -1):  # pobtasi.py:199
        lo_i = Lo[i].copy()  # :200
        ar_i = Ar[i].copy()  # :201
        buf_i = buf[i].copy()  # :202
        Linv = la.solve_triangular(D[i], eye, lower=True)  # :204-208
        # :211-216  X_{i+1,i}
        Lo[i] = (-buf[i + 1].conj().T @ buf_i - D[i + 1] @ lo_i - Ar[i + 1].conj().T @ ar_i) @ Linv
        # :219-223  X_{top,i}
        buf[i] = (-buf[i + 1] @ lo_i - D[0] @ buf_i - Ar[0].conj().T @ ar_i) @ Linv
        # :227-231  X_{A,i}
        Ar[i] = (-Ar[i + 1] @ lo_i - Ar[0] @ buf_i - T @ ar_i) @ Linv
        # :234-241  X_{i,i}
        D[i] = (Linv.conj().T - Lo[i].conj().T @ lo_i - buf[i].conj().T @ buf_i
                - Ar[i].conj().T @ ar_i) @ Linv
    Lo[0] = buf[1].conj().T  # :244


def pobtas_permuted(D, Lo, Ar, T, B, buf, trans: str = "N") -> None:
    """Block triangular solve of a middle partition, after ``_pobtas_permuted``
    (src/serinv/algs/pobtas.py:164-218).  Blocks 1..n-2 are solved; block 0
    and the tip receive the updates (the reduced system's right-hand side)."""
    n, b = D.shape[0], D.shape[1]
    a = Ar.shape[1]
    tip = slice(n * b, n * b + a)

    def blk(i):
        return slice(i * b, (i + 1) * b)

    if trans == "N":  # pobtas.py:179
        for i in range(1, n - 1):
            B[blk(i)] = la.solve_triangular(D[i], B[blk(i)], lower=True)  # :182-186
            B[blk(i + 1)] -= Lo[i] @ B[blk(i)]  # :189-192
            B[blk(0)] -= buf[i] @ B[blk(i)]  # :195-197
            B[tip] -= Ar[i] @ B[blk(i)]  # :200-203
    elif trans in ("T", "C"):  # :204-216
        for i in range(n - 2, 0, -1):
            rhs = (B[blk(i)] - Lo[i].conj().T @ B[blk(i + 1)] - Ar[i].conj().T @ B[tip]
                   - buf[i].conj().T @ B[blk(0)])  # :208-212
            B[blk(i)] = la.solve_triangular(D[i], rhs, lower=True, trans="C")  # :207-216
    else:
        raise ValueError(f"Invalid transpose argument: {trans}.")  # :217-218


def bta_to_dense(D, Lo, Ar, T, symmetric: bool = True) -> np.ndarray:
    """Assemble the dense matrix (lower blocks mirrored when ``symmetric``).

    Mirrors the block placement of the reference's test helper
    ``bta_dense_to_arrays`` (tests/testing_utils.py:17-122), run backwards.
    """
    n, b = D.shape[0], D.shape[1]
    a = Ar.shape[1]
    N = n * b + a
    A = np.zeros((N, N), dtype=D.dtype)
    for i in range(n):
        A[i * b:(i + 1) * b, i * b:(i + 1) * b] = D[i]
        if i < n - 1:
            A[(i + 1) * b:(i + 2) * b, i * b:(i + 1) * b] = Lo[i]
            if symmetric:
                A[i * b:(i + 1) * b, (i + 1) * b:(i + 2) * b] = Lo[i].conj().T
        if a:
            A[n * b:, i * b:(i + 1) * b] = Ar[i]
            if symmetric:
                A[i * b:(i + 1) * b, n * b:] = Ar[i].conj().T
    if a:
        A[n * b:, n * b:] = T
    return A


def dense_to_bta(A: np.ndarray, n: int, b: int, a: int):
    """Extract the lower BTA stacks of a dense matrix (tests/testing_utils.py:17-122)."""
    D = np.stack([A[i * b:(i + 1) * b, i * b:(i + 1) * b] for i in range(n)]).copy()
    Lo = np.zeros((max(n - 1, 0), b, b), dtype=A.dtype)
    for i in range(n - 1):
        Lo[i] = A[(i + 1) * b:(i + 2) * b, i * b:(i + 1) * b]
    Ar = np.zeros((n, a, b), dtype=A.dtype)
    for i in range(n):
        Ar[i] = A[n * b:, i * b:(i + 1) * b]
    T = A[n * b:, n * b:].copy()
    return D, Lo, Ar, T
