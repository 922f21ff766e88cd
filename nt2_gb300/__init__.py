"""nt2_gb300 -- GB300 (sm_103a) evaluator for NT2 table expressions.

The compute path is libnt2cuda.so (hand-written CUDA kernels behind the C
ABI in include/nt2cuda.h).  This package builds it (nt2_gb300.build),
binds it with ctypes (nt2_gb300._lib) and exposes NT2-named functions over
torch tensors (nt2_gb300.api) and the request server (nt2_gb300.server).
"""
from ._lib import LIB_PATH, NT2CudaError, check, lib  # noqa: F401

__all__ = ["LIB_PATH", "NT2CudaError", "check", "lib"]
