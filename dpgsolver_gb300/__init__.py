"""GB300-native DG residual engine with the interface of DPGSolver's explicit/implicit DG path.

The residual, SSP-RK3 and Newton paths run as hand-written sm_103a CUDA behind the C ABI of include/dpg_gb300.h;
``api`` is a thin ctypes binding of that ABI.
"""
from .api import (Config, DpgError, GpuContext, Simulation, load_library, LIB_PATH, PREC_FP64, PREC_BF16X3,
                  PREC_TF32X3, PREC_BF16_SLICED, PRECOND_NONE, PRECOND_BLOCK_JACOBI, PRECOND_MLP, PRECOND_BLOCK_ILU,
                  JACOBIAN_TANGENT, JACOBIAN_FD, TileConfig)

__all__ = ["Config", "DpgError", "GpuContext", "Simulation", "load_library", "LIB_PATH", "PREC_FP64", "PREC_BF16X3",
           "PREC_TF32X3", "PREC_BF16_SLICED", "PRECOND_NONE", "PRECOND_BLOCK_JACOBI", "PRECOND_MLP", "PRECOND_BLOCK_ILU",
           "JACOBIAN_TANGENT", "JACOBIAN_FD", "TileConfig"]
