"""Python host side of the GB300 Top-K SpMV engine: ctypes over the C ABI of include/acceles.h.

``SpMV`` mirrors the reference's quantised host driver ``struct SpMV``
(zhaijiaqi/AccelES, src/fpga/src/host_spmv_ucsr.cpp:134-829): the constructor packs and
uploads the matrix, ``Q_reset`` loads a query, calling the object runs the pass and returns the
device time in nanoseconds, ``Q_read_result`` appends the merged, sorted candidates to the
caller's lists.  ``read_topk`` returns the final FP32 Top-K of the two-stage method.

There is no CPU fallback: if the compiled library is missing or no GPU is present, the calls
raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _build

AES_OK = 0
AES_ERR_INVALID = -1
AES_ERR_UNSUPPORTED = -2
AES_ERR_CUDA = -3
AES_ERR_NOMEM = -4
AES_ERR_QUERY = -5
AES_ERR_STATE = -6
AES_ERR_NODEV = -7

QUANT_SYM_GLOBAL = 0
QUANT_UNSIGNED_ROW = 1
QUANT_UNSIGNED_GLOBAL = 2
QQ_NUMPY = 0
QQ_TRUNC = 1

GEN_UNIFORM_DEG = 0
GEN_FIXED_ABSNORMAL = 1
GEN_GAMMA_DEG = 2
GEN_FIXED_UNIFORM = 3

EXPORTS = ["aes_params_default", "aes_create", "aes_create_csr", "aes_create_quantized",
           "aes_create_view", "aes_destroy", "aes_get_info", "aes_set_query", "aes_set_query_quantized", "aes_run", "aes_read_candidates", "aes_run_device", "aes_finish",
           "aes_last_error", "aes_gen_matrix", "aes_pack_host", "aes_pack_tc_host", "aes_score_all", "aes_get_stats", "aes_run_noalloc", "aes_run_exact",
           "aes_retune", "aes_read_mtx", "aes_free", "aes_write_mtx", "aes_resparse"]

FLAG_PROFILE = 1
FLAG_GRAPHS = 2
FLAG_TENSOR = 4  # 4-bit matrices: batched candidate pass on the tensor cores (tcgen05, FP8)
FLAG_POSITIVE = 8  # read_candidates keeps scores above 0 only (Q_read_result's filter)
FLAG_TEST_IDLE_MMA = 16  # failure-path tests: the tensor-core pass's waits run out


class AesError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [("bits", ctypes.c_uint32), ("quant", ctypes.c_uint32),
                ("query_quant", ctypes.c_uint32), ("split", ctypes.c_uint32),
                ("ck", ctypes.c_uint32), ("k_max", ctypes.c_uint32),
                ("max_batch", ctypes.c_uint32), ("pack_parts", ctypes.c_uint32),
                ("sample_stride", ctypes.c_uint32), ("batch_tile", ctypes.c_uint32),
                ("device", ctypes.c_int32), ("flags", ctypes.c_uint32),
                ("seed", ctypes.c_uint64), ("mem_limit", ctypes.c_uint64),
                ("batch_warps", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_uint64), ("cand_launches", ctypes.c_uint64),
                ("cand_ms", ctypes.c_double), ("cand_timed", ctypes.c_uint64),
                ("repaired", ctypes.c_uint64)]


class Info(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_uint32), ("cols", ctypes.c_uint32), ("bits", ctypes.c_uint32),
                ("packet_elems", ctypes.c_uint32), ("nnz", ctypes.c_uint64),
                ("quantized_nnz", ctypes.c_uint64), ("packets", ctypes.c_uint64),
                ("tiles", ctypes.c_uint64), ("packet_bytes", ctypes.c_uint64),
                ("device_bytes", ctypes.c_uint64), ("split", ctypes.c_uint32),
                ("ck", ctypes.c_uint32), ("ck_effective", ctypes.c_uint32),
                ("sample_tiles", ctypes.c_uint32), ("sample_rows", ctypes.c_uint32),
                ("max_batch", ctypes.c_uint32), ("batch_tile", ctypes.c_uint32),
                ("tensor_tiles", ctypes.c_uint32), ("exact_pass", ctypes.c_uint32),
                ("batch_warps", ctypes.c_uint32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None
_u32p = ctypes.POINTER(ctypes.c_uint32)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_f32p = ctypes.POINTER(ctypes.c_float)
_i8p = ctypes.POINTER(ctypes.c_int8)


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libacceles.so (building it in-tree if asked and missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB):
        if not build_if_missing:
            raise RuntimeError(f"{_build.LIB} is not built")
        _build.build()
    L = ctypes.CDLL(_build.LIB)
    L.aes_params_default.restype = None
    L.aes_params_default.argtypes = [ctypes.POINTER(Params)]
    L.aes_create.restype = ctypes.c_int
    L.aes_create.argtypes = [_u32p, _u32p, _f32p, ctypes.c_uint32, ctypes.c_uint32,
                             ctypes.c_uint64, ctypes.POINTER(Params), ctypes.POINTER(ctypes.c_void_p)]
    L.aes_create_csr.restype = ctypes.c_int
    L.aes_create_csr.argtypes = [_u64p, _u32p, _f32p, ctypes.c_uint32, ctypes.c_uint32,
                                 ctypes.POINTER(Params), ctypes.POINTER(ctypes.c_void_p)]
    L.aes_create_quantized.restype = ctypes.c_int
    L.aes_create_quantized.argtypes = [_u32p, _u32p, _i8p, _f32p, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_uint64, ctypes.POINTER(Params),
                                       ctypes.POINTER(ctypes.c_void_p)]
    L.aes_set_query_quantized.restype = ctypes.c_int
    L.aes_set_query_quantized.argtypes = [ctypes.c_void_p, _i8p, _f32p, ctypes.c_uint32]
    L.aes_create_view.restype = ctypes.c_int
    L.aes_create_view.argtypes = [ctypes.c_void_p, ctypes.POINTER(Params),
                                  ctypes.POINTER(ctypes.c_void_p)]
    L.aes_destroy.restype = ctypes.c_int
    L.aes_destroy.argtypes = [ctypes.c_void_p]
    L.aes_get_info.restype = ctypes.c_int
    L.aes_get_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(Info)]
    L.aes_set_query.restype = ctypes.c_int
    L.aes_set_query.argtypes = [ctypes.c_void_p, _f32p, ctypes.c_uint32]
    L.aes_run.restype = ctypes.c_int
    L.aes_run.argtypes = [ctypes.c_void_p, ctypes.c_uint32, _u32p, _f32p, _u64p]
    L.aes_read_candidates.restype = ctypes.c_int
    L.aes_read_candidates.argtypes = [ctypes.c_void_p, ctypes.c_uint32, _u32p, _i32p, _f32p,
                                      ctypes.c_uint32, _u32p]
    L.aes_run_device.restype = ctypes.c_int
    L.aes_run_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                 ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.aes_finish.restype = ctypes.c_int
    L.aes_finish.argtypes = [ctypes.c_void_p, _u32p]
    L.aes_last_error.restype = ctypes.c_char_p
    L.aes_last_error.argtypes = []
    L.aes_gen_matrix.restype = ctypes.c_uint64
    L.aes_gen_matrix.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_uint64, _u64p,
                                 _u32p, _f32p]
    L.aes_pack_host.restype = ctypes.c_int
    L.aes_pack_host.argtypes = [_u64p, _u32p, _f32p, ctypes.c_uint32, ctypes.c_uint32,
                                ctypes.POINTER(Params), ctypes.c_void_p, ctypes.c_uint64, _u64p,
                                _u32p]
    L.aes_pack_tc_host.restype = ctypes.c_int
    L.aes_pack_tc_host.argtypes = [_u64p, _u32p, _f32p, ctypes.c_uint32, ctypes.c_uint32,
                                   ctypes.POINTER(Params), _u32p, ctypes.c_uint64, _u32p,
                                   ctypes.c_uint64, _u64p, _u64p]
    L.aes_run_noalloc.restype = ctypes.c_int
    L.aes_run_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.aes_run_exact.restype = ctypes.c_int
    L.aes_run_exact.argtypes = [ctypes.c_void_p, ctypes.c_uint32, _u32p, _f32p, _u64p]
    L.aes_read_mtx.restype = ctypes.c_int
    L.aes_read_mtx.argtypes = [ctypes.c_char_p, ctypes.c_uint32, _u32p, _u32p, _u64p,
                               ctypes.POINTER(_u32p), ctypes.POINTER(_u32p), ctypes.POINTER(_f32p)]
    L.aes_free.restype = None
    L.aes_free.argtypes = [ctypes.c_void_p]
    L.aes_write_mtx.restype = ctypes.c_int
    L.aes_write_mtx.argtypes = [ctypes.c_char_p, _u32p, _u32p, _f32p, ctypes.c_uint32,
                                ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32]
    L.aes_resparse.restype = ctypes.c_int
    L.aes_resparse.argtypes = [_u64p, _u32p, _f32p, ctypes.c_uint32, ctypes.c_uint32,
                               ctypes.c_double, _u64p, _u32p, _f32p, ctypes.c_uint64, _u64p]
    L.aes_retune.restype = ctypes.c_int
    L.aes_retune.argtypes = [ctypes.c_void_p, ctypes.POINTER(Params)]
    L.aes_get_stats.restype = ctypes.c_int
    L.aes_get_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(Stats), ctypes.c_int]
    L.aes_score_all.restype = ctypes.c_int
    L.aes_score_all.argtypes = [ctypes.c_void_p, _f32p, _u32p]
    _lib = L
    return L


def _check(rc):
    if rc != AES_OK:
        raise AesError(rc, load().aes_last_error().decode(errors="replace"))


def _p(a, t):
    return a.ctypes.data_as(t)


def default_params(**kw) -> Params:
    p = Params()
    load().aes_params_default(ctypes.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def gen_matrix(kind: int, rows: int, cols: int, p0: float, p1: float = 0.0, seed: int = 0):
    """Seeded synthetic CSR (ptr u64, col u32, val f32) sorted by (row, col)."""
    L = load()
    nnz = L.aes_gen_matrix(kind, rows, cols, p0, p1, seed, None, None, None)
    if nnz == (1 << 64) - 1:
        raise ValueError("bad generator arguments")
    ptr = np.zeros(rows + 1, np.uint64)
    col = np.zeros(max(nnz, 1), np.uint32)
    val = np.zeros(max(nnz, 1), np.float32)
    L.aes_gen_matrix(kind, rows, cols, p0, p1, seed, _p(ptr, _u64p), _p(col, _u32p), _p(val, _f32p))
    return ptr, col[:nnz], val[:nnz]


def pack_host(ptr, col, val, rows, cols, **params):
    """Host-only Ultra-CSR packing (no device): (packets [n, 64] u8, tile_rowbase u32)."""
    L = load()
    prm = default_params(**params)
    ptr = np.ascontiguousarray(ptr, np.uint64)
    col = np.ascontiguousarray(col, np.uint32)
    val = np.ascontiguousarray(val, np.float32)
    n = ctypes.c_uint64(0)
    _check(L.aes_pack_host(_p(ptr, _u64p), _p(col, _u32p), _p(val, _f32p), rows, cols,
                           ctypes.byref(prm), None, 0, ctypes.byref(n), None))
    pk = np.zeros((max(n.value, 1), 64), np.uint8)
    tiles = (n.value + 31) // 32
    trb = np.zeros(tiles + 1, np.uint32)
    _check(L.aes_pack_host(_p(ptr, _u64p), _p(col, _u32p), _p(val, _f32p), rows, cols,
                           ctypes.byref(prm), pk.ctypes.data_as(ctypes.c_void_p), n.value,
                           ctypes.byref(n), _p(trb, _u32p)))
    return pk[: n.value], trb


def pack_tc_host(ptr, col, val, rows, cols, **params):
    """Host-only tensor-core tile layout of a 4-bit matrix (no device): (tile_ptr u32,
    entries u32); empty arrays when the layout is not built."""
    L = load()
    prm = default_params(**params)
    ptr = np.ascontiguousarray(ptr, np.uint64)
    col = np.ascontiguousarray(col, np.uint32)
    val = np.ascontiguousarray(val, np.float32)
    n_ptr, n_ent = ctypes.c_uint64(0), ctypes.c_uint64(0)
    _check(L.aes_pack_tc_host(_p(ptr, _u64p), _p(col, _u32p), _p(val, _f32p), rows, cols,
                              ctypes.byref(prm), None, 0, None, 0, ctypes.byref(n_ptr),
                              ctypes.byref(n_ent)))
    tp = np.zeros(max(n_ptr.value, 1), np.uint32)
    ent = np.zeros(max(n_ent.value, 1), np.uint32)
    _check(L.aes_pack_tc_host(_p(ptr, _u64p), _p(col, _u32p), _p(val, _f32p), rows, cols,
                              ctypes.byref(prm), _p(tp, _u32p), n_ptr.value, _p(ent, _u32p),
                              n_ent.value, ctypes.byref(n_ptr), ctypes.byref(n_ent)))
    return tp[: n_ptr.value], ent[: n_ent.value]


MTX_ZERO_INDEXED = 1
MTX_SORT = 2
MTX_KEEP_DIRECTED = 4


def read_mtx(path, flags: int = 0):
    """Matrix Market coordinate file -> (rows, cols, row u32, col u32, val f32) COO."""
    L = load()
    rows, cols, nnz = ctypes.c_uint32(0), ctypes.c_uint32(0), ctypes.c_uint64(0)
    r, c, v = _u32p(), _u32p(), _f32p()
    _check(L.aes_read_mtx(os.fsencode(path), flags, ctypes.byref(rows), ctypes.byref(cols),
                          ctypes.byref(nnz), ctypes.byref(r), ctypes.byref(c), ctypes.byref(v)))
    try:
        n = nnz.value
        R = np.ctypeslib.as_array(r, shape=(max(n, 1),))[:n].copy()
        C = np.ctypeslib.as_array(c, shape=(max(n, 1),))[:n].copy()
        V = np.ctypeslib.as_array(v, shape=(max(n, 1),))[:n].copy()
    finally:
        for p in (r, c, v):
            L.aes_free(ctypes.cast(p, ctypes.c_void_p))
    return rows.value, cols.value, R, C, V


def write_mtx(path, rows, cols, row, col, val, flags: int = 0):
    row = np.ascontiguousarray(row, np.uint32)
    col = np.ascontiguousarray(col, np.uint32)
    val = np.ascontiguousarray(val, np.float32)
    _check(load().aes_write_mtx(os.fsencode(path), _p(row, _u32p), _p(col, _u32p),
                                _p(val, _f32p), rows, cols, row.shape[0], flags))


def resparse(ptr, col, val, rows, cols, keep):
    """ReSparse per-row pruning of a sorted CSR: (ptr u64, col u32, val f32) of the kept entries."""
    L = load()
    ptr = np.ascontiguousarray(ptr, np.uint64)
    col = np.ascontiguousarray(col, np.uint32)
    val = np.ascontiguousarray(val, np.float32)
    n = ctypes.c_uint64(0)
    optr = np.zeros(rows + 1, np.uint64)
    _check(L.aes_resparse(_p(ptr, _u64p), _p(col, _u32p), _p(val, _f32p), rows, cols,
                          float(keep), _p(optr, _u64p), None, None, 0, ctypes.byref(n)))
    ocol = np.zeros(max(n.value, 1), np.uint32)
    oval = np.zeros(max(n.value, 1), np.float32)
    _check(L.aes_resparse(_p(ptr, _u64p), _p(col, _u32p), _p(val, _f32p), rows, cols,
                          float(keep), _p(optr, _u64p), _p(ocol, _u32p), _p(oval, _f32p),
                          n.value, ctypes.byref(n)))
    return optr, ocol[:n.value], oval[:n.value]


class SpMV:
    """Device-resident two-stage low-bit Top-K SpMV over one matrix.

    Constructed from a COO (``row, col, val``) like the reference's quantised constructor
    (host_spmv_ucsr.cpp:198-218), or from a sorted CSR with ``ptr=``.
    """

    def __init__(self, rows, cols, row=None, col=None, val=None, ptr=None, qval=None,
                 _view_of=None, **params):
        """qval: the entries' pre-quantised B-bit values (int8) for the quantised constructor;
        val may then be None (no FP32 exact pass)."""
        L = load()
        self._h = ctypes.c_void_p()
        self.params = default_params(**params)
        self.rows, self.cols = int(rows), int(cols)
        if _view_of is not None:
            _check(L.aes_create_view(_view_of._h, ctypes.byref(self.params), ctypes.byref(self._h)))
        elif qval is not None:
            if ptr is not None:  # CSR given: expand to COO rows
                ptr = np.asarray(ptr, np.uint64)
                row = np.repeat(np.arange(self.rows, dtype=np.uint32), np.diff(ptr).astype(np.int64))
            row = np.ascontiguousarray(row, np.uint32)
            col = np.ascontiguousarray(col, np.uint32)
            qv = np.ascontiguousarray(qval, np.int8)
            vp = None
            if val is not None:
                val = np.ascontiguousarray(val, np.float32)
                vp = _p(val, _f32p)
            _check(L.aes_create_quantized(_p(row, _u32p), _p(col, _u32p), _p(qv, _i8p), vp,
                                          self.rows, self.cols, row.shape[0],
                                          ctypes.byref(self.params), ctypes.byref(self._h)))
        elif ptr is not None:
            ptr = np.ascontiguousarray(ptr, np.uint64)
            col = np.ascontiguousarray(col, np.uint32)
            val = np.ascontiguousarray(val, np.float32)
            _check(L.aes_create_csr(_p(ptr, _u64p), _p(col, _u32p), _p(val, _f32p), self.rows,
                                    self.cols, ctypes.byref(self.params), ctypes.byref(self._h)))
        else:
            row = np.ascontiguousarray(row, np.uint32)
            col = np.ascontiguousarray(col, np.uint32)
            val = np.ascontiguousarray(val, np.float32)
            _check(L.aes_create(_p(row, _u32p), _p(col, _u32p), _p(val, _f32p), self.rows,
                                self.cols, row.shape[0], ctypes.byref(self.params),
                                ctypes.byref(self._h)))
        self._nq = 0
        self._k = 0
        self._idx = None
        self._score = None

    # -- reference-shaped API ----------------------------------------------------------------
    def Q_reset(self, vec, debug=0):
        """Load one query or a [nq, cols] batch (host_spmv_ucsr.cpp:790-828)."""
        q = np.ascontiguousarray(np.atleast_2d(vec), np.float32)
        if q.shape[1] != self.cols:
            raise ValueError("query length != cols")
        _check(load().aes_set_query(self._h, _p(q, _f32p), q.shape[0]))
        self._nq = q.shape[0]
        return 0

    def Q_reset_quantized(self, qvec, q_f32=None):
        """Load pre-quantised queries ([nq, cols] int8, the reference's q_type vector of
        Q_reset, host_spmv_ucsr.cpp:790); q_f32 (optional) the same queries in FP32 for the
        exact pass."""
        q = np.ascontiguousarray(np.atleast_2d(qvec), np.int8)
        if q.shape[1] != self.cols:
            raise ValueError("query length != cols")
        fp = None
        if q_f32 is not None:
            qf = np.ascontiguousarray(np.atleast_2d(q_f32), np.float32)
            if qf.shape != q.shape:
                raise ValueError("q_f32 shape != query shape")
            fp = _p(qf, _f32p)
        _check(load().aes_set_query_quantized(self._h, _p(q, _i8p), fp, q.shape[0]))
        self._nq = q.shape[0]
        return 0

    def __call__(self, flag=True, debug=0, k=None):
        """Run the loaded queries; returns the device time in ns (operator(), :556-565)."""
        k = int(k or self.params.k_max)
        self._idx = np.zeros((self._nq, k), np.uint32)
        self._score = np.zeros((self._nq, k), np.float32)
        ns = ctypes.c_uint64(0)
        _check(load().aes_run(self._h, k, _p(self._idx, _u32p), _p(self._score, _f32p),
                              ctypes.byref(ns)))
        self._k = k
        return int(ns.value)

    def run_exact(self, k=None):
        """FP32-only Top-K of the loaded queries (no low-bit stage); returns (rows, scores, ns)."""
        k = int(k or self.params.k_max)
        idx = np.zeros((self._nq, k), np.uint32)
        sc = np.zeros((self._nq, k), np.float32)
        ns = ctypes.c_uint64(0)
        _check(load().aes_run_exact(self._h, k, _p(idx, _u32p), _p(sc, _f32p), ctypes.byref(ns)))
        return idx, sc, int(ns.value)

    def Q_read_result(self, res, idx, debug=0, query=0):
        """Append the candidates of `query`, sorted by (score desc, row desc)
        (host_spmv_ucsr.cpp:691-748)."""
        r, s, _ = self.read_candidates(query)
        idx.extend(int(x) for x in r)
        res.extend(int(x) for x in s)

    # -- results ------------------------------------------------------------------------------
    def read_topk(self):
        """Final Top-K of the last run: (rows [nq, k], FP32 scores [nq, k])."""
        return self._idx, self._score

    def read_candidates(self, query=0):
        cap = self.info()["ck"]
        idx = np.zeros(max(cap, 1), np.uint32)
        sc = np.zeros(max(cap, 1), np.int32)
        key = np.zeros(max(cap, 1), np.float32)
        n = ctypes.c_uint32(0)
        _check(load().aes_read_candidates(self._h, query, _p(idx, _u32p), _p(sc, _i32p),
                                          _p(key, _f32p), cap, ctypes.byref(n)))
        m = min(n.value, cap)
        return idx[:m].copy(), sc[:m].copy(), key[:m].copy()

    def run_device(self, d_queries: int, nq: int, k: int, d_idx: int, d_score: int, stream: int = 0):
        _check(load().aes_run_device(self._h, ctypes.c_void_p(d_queries), nq, k,
                                     ctypes.c_void_p(d_idx), ctypes.c_void_p(d_score),
                                     ctypes.c_void_p(stream) if stream else None))

    def run_noalloc(self, d_query: int, k: int, d_idx: int, d_score: int, stream: int = 0):
        """One device-resident query through the path without allocating (see acceles.h)."""
        _check(load().aes_run_noalloc(self._h, ctypes.c_void_p(d_query), k,
                                      ctypes.c_void_p(d_idx), ctypes.c_void_p(d_score),
                                      ctypes.c_void_p(stream) if stream else None))

    def view(self, **changes):
        """Another handle on this matrix (aes_create_view): its own stream and batch buffers, the
        matrix shared; `changes` override this handle's parameters (ck, max_batch, flags, ...)."""
        prm = {f: getattr(self.params, f) for f, _ in Params._fields_}
        prm.update(changes)
        return SpMV(self.rows, self.cols, _view_of=self, **prm)

    def retune(self, **changes):
        """Change ck, split, sample_stride, batch_tile, batch_warps, k_max, max_batch, flags,
        query_quant or mem_limit without packing the matrix again; loaded queries are dropped."""
        prm = Params()
        ctypes.memmove(ctypes.byref(prm), ctypes.byref(self.params), ctypes.sizeof(Params))
        for k, v in changes.items():
            if not hasattr(prm, k):
                raise KeyError(k)
            setattr(prm, k, v)
        _check(load().aes_retune(self._h, ctypes.byref(prm)))
        self.params = prm
        self._nq = 0
        self._idx = self._score = None

    def finish(self) -> int:
        n = ctypes.c_uint32(0)
        _check(load().aes_finish(self._h, ctypes.byref(n)))
        return n.value

    def score_all(self, vec):
        """Candidate-pass key of every row for one FP32 query (uint32 order-preserving)."""
        q = np.ascontiguousarray(vec, np.float32)
        keys = np.zeros(self.rows, np.uint32)
        _check(load().aes_score_all(self._h, _p(q, _f32p), _p(keys, _u32p)))
        return keys

    def stats(self, reset=True):
        st = Stats()
        _check(load().aes_get_stats(self._h, ctypes.byref(st), 1 if reset else 0))
        return {f: getattr(st, f) for f, _ in st._fields_}

    def info(self):
        inf = Info()
        _check(load().aes_get_info(self._h, ctypes.byref(inf)))
        return inf.as_dict()

    def close(self):
        if self._h:
            load().aes_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
