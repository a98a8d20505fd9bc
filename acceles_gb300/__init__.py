"""GB300-native two-stage low-bit Top-K SpMV engine (AccelES method) behind a C ABI.

The compute path is libacceles.so (sm_103a CUDA kernels + C++ host code), reached through
``acceles_gb300.engine``.  See include/acceles.h for the ABI.
"""
from .engine import SpMV, AesError, default_params, gen_matrix, load  # noqa: F401

__all__ = ["SpMV", "AesError", "default_params", "gen_matrix", "load"]
