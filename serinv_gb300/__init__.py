"""serinv_gb300 — GB300-native BTA Cholesky, selected inversion and solve.

Drop-in for the sequential hot path of serinv (``serinv.algs.pobtaf``,
``pobtasi``, ``pobtas``): same call signatures and in-place block-stack
layout, computed by hand-written sm_103a CUDA kernels behind the C ABI in
``include/serinv_gb300.h``.
"""

__version__ = "0.1.0"

from .algs import pobtaf, pobtasi, pobtas, pobtf, pobtsi, pobts  # noqa: E402,F401
from .dense import dgemm  # noqa: E402,F401
from .refine import bta_matvec, pobtas_refine  # noqa: E402,F401

__all__ = ["pobtaf", "pobtasi", "pobtas", "pobtf", "pobtsi", "pobts", "dgemm", "bta_matvec", "pobtas_refine",
           "__version__"]
