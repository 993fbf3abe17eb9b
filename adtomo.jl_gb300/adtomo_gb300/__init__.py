"""adtomo_gb300 -- GB300 (sm_103a) implementation of ADTomo.jl's Eikonal hot path.

The compute path is the CUDA library libadtomo_gpu.so (C ABI in
include/adtomo_gpu.h); this package binds it with ctypes and mirrors the
reference's Julia API (src/eikonal_op.jl).  There is no CPU fallback: if the
library cannot be loaded, or no GPU is present, calls raise AdtError.
"""
from ._lib import ADT_ADJ_AUTO, ADT_ADJ_CAUSAL, ADT_ADJ_SWEEPS, ADT_F32, ADT_F64, AdtError, lib  # noqa: F401
from .ops import (Batch3D, eikonal, eikonal3d, eikonal3d_grad, eikonal_batch,  # noqa: F401
                  eikonal_grad)

__version__ = "0.1.0"
