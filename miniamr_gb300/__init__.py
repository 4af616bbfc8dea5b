"""GB300 (sm_103a) back end for miniAMR's per-timestep hot path.

The product is a C-ABI shared library (include/miniamr_gb300.h) built from
miniamr_gb300/csrc/.  The reference's own C driver links the drop-in
translation units in miniamr_gb300/dropin/ over it; Python callers (tests,
bench.py) use the ctypes binding here.  :func:`load` returns the GPU
library and fails loudly when it has not been built or no CUDA device is
present -- there is no CPU fallback on the product path.
"""
from __future__ import annotations

import os

from .abi import (BLOCK_DTYPE, CONSOLIDATE_DTYPE, FP32, FP64, RUN_BATCHED,
                  RUN_GRAPH, RUN_PLAIN, SPLIT_DTYPE, Config, Context, Library,
                  MamrError)
from .build import LIB

__all__ = ["load", "Library", "Context", "Config", "MamrError", "FP64",
           "FP32", "RUN_PLAIN", "RUN_BATCHED", "RUN_GRAPH", "BLOCK_DTYPE",
           "SPLIT_DTYPE", "CONSOLIDATE_DTYPE", "LIB"]

_lib = None


def load() -> Library:
    """The GB300 library.  Raises if it is not built (run
    ``python -m miniamr_gb300.build``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(f"GB300 library not built: {LIB} is missing; "
                               "run python -m miniamr_gb300.build")
        _lib = Library(LIB)
    return _lib
