"""GB300 (sm_103a) implementation of FPDE_HPC's hot path.

The compute lives in libfpde_gb300.so (hand-written CUDA, C ABI in include/fpde_gb300.h).
This package is the host-side mirror used from Python: a thin ctypes layer plus the
problem generators of the benchmark configurations. Importing it does not need a GPU;
creating a context does, and every compute call runs on the GPU (no CPU fallback).
"""
from ._lib import FpdeError, LineDesc, LineTuning, load, check  # noqa: F401
from .api import Batch, Context, History, Line, Lod3D, weights_l1, weights_l1_lags, restricted_lags, gamma, line_coefs, do_weights, autotune_line, autotune_lod3d, sf_toeplitz_row  # noqa: F401

FPDE_PREC_FP64 = 0
FPDE_PREC_SPLIT_BF16 = 1
FPDE_PREC_SPLIT_F16 = 2
FPDE_PREC_SPLIT_BF16X3 = 3
FPDE_BC_DIRICHLET = 0
FPDE_BC_FLUX = 1
