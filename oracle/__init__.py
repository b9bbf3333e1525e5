"""CPU oracle for the BTA hot path (test infrastructure only).

This package restates, in NumPy/SciPy, the reference's sequential algorithms
for symmetric positive-definite block-tridiagonal-with-arrowhead matrices:
``pobtaf`` (block Cholesky), ``pobtasi`` (selected inversion) and ``pobtas``
(block triangular solve).  It exists to check the CUDA implementation and to
time the reference algorithm on host cores.  Nothing in the product path
imports it: only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline leg (and ``bench.py --impl reference``) may use it.

Parity is pinned: ``tests/golden/`` holds vectors produced by running the
reference implementation itself (``tests/golden/make_golden.py``), and
``tests/test_oracle.py`` checks this restatement against them bit for bit
(same LAPACK/BLAS call sequence) and against dense NumPy factorizations.
"""

from .bta import pobtaf, pobtasi, pobtas, bta_to_dense, dense_to_bta  # noqa: F401
from .bta import pobtaf_permuted, pobtasi_permuted, pobtas_permuted  # noqa: F401
