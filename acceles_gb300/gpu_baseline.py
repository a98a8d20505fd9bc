"""Library-SpMV comparison arm (libaes_baseline.so): cuSPARSE SpMV over the FP32 CSR, a full
sort of all row scores, the first K -- the method of the reference's GPU baselines
(src/gpu/host_spmv_topk_csr_gpu_int8.cu, SpMV :68-314).  For timing next to the two-stage path;
not a component of it."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _build
from .engine import AesError

EXPORTS = ["aes_baseline_cusparse_topk", "aes_baseline_last_error"]

_lib = None
_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_f32p = ctypes.POINTER(ctypes.c_float)


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(_build.BASELINE_LIB):
            _build.build()
        L = ctypes.CDLL(_build.BASELINE_LIB)
        L.aes_baseline_cusparse_topk.restype = ctypes.c_int
        L.aes_baseline_cusparse_topk.argtypes = [_u64p, _u32p, _f32p, ctypes.c_uint32,
                                                 ctypes.c_uint32, _f32p, ctypes.c_uint32,
                                                 ctypes.c_uint32, ctypes.c_int, _u32p, _f32p,
                                                 ctypes.POINTER(ctypes.c_double)]
        L.aes_baseline_last_error.restype = ctypes.c_char_p
        L.aes_baseline_last_error.argtypes = []
        _lib = L
    return _lib


def cusparse_topk(ptr, col, val, rows, cols, queries, k, device=0):
    """(rows [nq, k], scores [nq, k], device ms per query)."""
    L = load()
    ptr = np.ascontiguousarray(ptr, np.uint64)
    col = np.ascontiguousarray(col, np.uint32)
    val = np.ascontiguousarray(val, np.float32)
    Q = np.ascontiguousarray(np.atleast_2d(queries), np.float32)
    idx = np.zeros((Q.shape[0], k), np.uint32)
    sc = np.zeros((Q.shape[0], k), np.float32)
    ms = ctypes.c_double(0.0)
    rc = L.aes_baseline_cusparse_topk(ptr.ctypes.data_as(_u64p), col.ctypes.data_as(_u32p),
                                      val.ctypes.data_as(_f32p), rows, cols,
                                      Q.ctypes.data_as(_f32p), Q.shape[0], k, device,
                                      idx.ctypes.data_as(_u32p), sc.ctypes.data_as(_f32p),
                                      ctypes.byref(ms))
    if rc != 0:
        raise AesError(rc, L.aes_baseline_last_error().decode(errors="replace"))
    return idx, sc, ms.value
