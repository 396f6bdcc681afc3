"""solidfmm-gb300: GB300 (sm_103a) CUDA implementation of solidfmm's
rotation-based translation operators M2M, M2L and L2L.

The compute lives in libsfmm_gb300.so (C ABI in include/sfmm.h, C++ drop-in
API in include/solidfmm/).  This package builds it (``build``) and binds it
for Python callers (``_native``).
"""
from ._native import (F32, F64, L2L, M2L, M2M, PLAIN, SPLIT, SPLIT_FF, TC_BF16, TC_BF16X6, TC_TF32, Context,  # noqa: F401
                      Plan, SfmmError, load)

__all__ = ["Context", "Plan", "SfmmError", "load", "F32", "F64", "M2M", "M2L", "L2L", "PLAIN", "SPLIT", "SPLIT_FF",
           "TC_TF32", "TC_BF16", "TC_BF16X6"]
