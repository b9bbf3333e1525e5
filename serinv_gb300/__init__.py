"""serinv_gb300 — GB300-native BTA Cholesky, selected inversion and solve.

Drop-in for the sequential hot path of serinv (``serinv.algs.pobtaf``,
``pobtasi``, ``pobtas``): same call signatures and in-place block-stack
layout, computed by hand-written sm_103a CUDA kernels behind the C ABI in
``include/serinv_gb300.h``.
"""

__version__ = "0.1.0"

import os as _os

# Batch plans replay a graph of many independent branches (one per worker
# stream).  The CUDA driver spreads concurrent work over
# CUDA_DEVICE_MAX_CONNECTIONS hardware queues, 8 unless set, and serialises
# branches beyond that: measured on the 256-matrix uneven batch (mixed form),
# 8 queues give 1155 ms per replay, 32 give 821 ms.  The variable only counts
# when it is set before the process creates its CUDA context, so it is set
# here, at import, unless the caller chose a value.
_os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from .algs import pobtaf, pobtasi, pobtas, pobtf, pobtsi, pobts  # noqa: E402,F401
from .dense import dgemm  # noqa: E402,F401
from .refine import bta_matvec, pobtas_refine  # noqa: E402,F401

__all__ = ["pobtaf", "pobtasi", "pobtas", "pobtf", "pobtsi", "pobts", "dgemm", "bta_matvec", "pobtas_refine",
           "__version__"]
