"""GB300 (sm_103a) implementation of the QMCkl basis-evaluation path behind the
qmckl `*_device` context API: C ABI in include/qmckl_gpu.h, native library in _lib/,
Python mirror in context.py, seeded workloads in systems.py."""
from .context import (ALLOCATION_FAILED, ALREADY_SET, FAILURE, INVALID_CONTEXT, NOT_PROVIDED, PRECISION_FP64,
                      PRECISION_SPLIT_BF16, SHARED_EXP_AUTO, SHARED_EXP_OFF, SHARED_EXP_ON, SUCCESS, Batch, Context,
                      QmcklError)
from .systems import System, config_adjoint, config_batched, config_medium, config_small

__all__ = ["Context", "Batch", "QmcklError", "System", "config_small", "config_medium", "config_batched", "config_adjoint",
           "SUCCESS", "FAILURE", "INVALID_CONTEXT", "ALLOCATION_FAILED", "NOT_PROVIDED", "ALREADY_SET",
           "PRECISION_FP64", "PRECISION_SPLIT_BF16", "SHARED_EXP_AUTO", "SHARED_EXP_OFF", "SHARED_EXP_ON"]
