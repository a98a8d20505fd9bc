"""CPU oracle for the two-stage low-bit Top-K SpMV path (TEST INFRASTRUCTURE ONLY).

This module is the oracle.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs
import it; the product package ``acceles_gb300`` never does.  It wraps ``aes_oracle.c`` (a plain
C restatement of the reference path, built into ``oracle/_build/liboracle.so``) and, when it was
compiled on this machine, ``oracle/_ref/libaes_ref.so`` (the reference's own gold code from
zhaijiaqi/AccelES, see ``oracle/Makefile``).

Reference anchors (files of zhaijiaqi/AccelES):
  quantify_matrix / quantify_vector   src/resources/python/quantify/quantify_util.py:8-49
  split_approximate                   src/resources/python/quantify/quantify_util.py:173-196
  spmv_coo_gold_top_k(_2)             src/fpga/src/gold_algorithms/gold_algorithms.hpp:189-308
  sort_tuples                         src/common/utils/evaluation_utils.hpp:40-62
  Ultra-CSR packet layout             src/fpga/src/ip/fpga_utils.hpp:317-527, types.hpp:151-162
  resparse_spm                        src/resources/python/quantify/quantify_util.py:375-403
  ReSparse ratio search               src/resources/python/quantify/datasets/
                                      search_best_resparse_ratio.py:55-117
  compt_precision / convergence       src/resources/python/quantify/quantify_util.py:198-219,413-437
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libaes_ref.so")

QUANT_SYM_GLOBAL = 0
QUANT_UNSIGNED_ROW = 1
QUANT_UNSIGNED_GLOBAL = 2
QQ_NUMPY = 0
QQ_TRUNC = 1

_lib = None
_ref = None

_u8p = ctypes.POINTER(ctypes.c_uint8)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)


def build(ref: bool = False) -> None:
    """Compile the oracle (and, if asked and the reference sources exist, oracle/_ref)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _p(a, t):
    return a.ctypes.data_as(t)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_packet_size.restype = ctypes.c_int
        L.orc_maxabs.restype = ctypes.c_double
        L.orc_maxabs.argtypes = [_f32p, ctypes.c_uint64]
        L.orc_q_sym.restype = ctypes.c_int32
        L.orc_q_sym.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int]
        L.orc_q_unsigned.restype = ctypes.c_int32
        L.orc_q_unsigned.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int]
        L.orc_q_trunc.restype = ctypes.c_int32
        L.orc_q_trunc.argtypes = [ctypes.c_float, ctypes.c_int]
        L.orc_quantize_query.restype = ctypes.c_int
        L.orc_quantize_query.argtypes = [_f32p, ctypes.c_uint32, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, _i32p]
        L.orc_quantize_matrix.restype = ctypes.c_uint64
        L.orc_quantize_matrix.argtypes = [_u64p, _u32p, _f32p, ctypes.c_uint32, ctypes.c_uint32,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_uint64, _u64p,
                                          _u32p, _i32p, _f32p]
        L.orc_pack_ultracsr.restype = ctypes.c_uint64
        L.orc_pack_ultracsr.argtypes = [_u64p, _u32p, _i32p, ctypes.c_uint32, ctypes.c_int,
                                        ctypes.c_uint32, _u8p]
        L.orc_xdecode.restype = None
        L.orc_xdecode.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_uint32, _u32p]
        L.orc_unpack_packet.restype = None
        L.orc_unpack_packet.argtypes = [_u8p, ctypes.c_int, ctypes.c_int, _u64p, _u32p, _i32p]
        L.orc_int_scores.restype = None
        L.orc_int_scores.argtypes = [_u64p, _u32p, _i32p, ctypes.c_uint32, _i32p, _i32p]
        L.orc_key_i32.restype = ctypes.c_uint32
        L.orc_key_i32.argtypes = [ctypes.c_int32]
        L.orc_key_f32.restype = ctypes.c_uint32
        L.orc_key_f32.argtypes = [ctypes.c_float]
        L.orc_cand_keys.restype = None
        L.orc_cand_keys.argtypes = [_i32p, _f32p, ctypes.c_uint32, _u32p]
        L.orc_select_split.restype = ctypes.c_uint32
        L.orc_select_split.argtypes = [_u32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                       _u32p]
        L.orc_gold_topk2.restype = None
        L.orc_gold_topk2.argtypes = [_u32p, _u32p, _i32p, ctypes.c_uint64, _i32p, ctypes.c_int,
                                     _u32p, _i32p]
        L.orc_gold_topk_f32.restype = None
        L.orc_gold_topk_f32.argtypes = [_u32p, _u32p, _f32p, ctypes.c_uint64, _f32p,
                                        ctypes.c_int, _u32p, _f32p]
        L.orc_rescore_f32.restype = None
        L.orc_rescore_f32.argtypes = [_u64p, _u32p, _f32p, _f32p, _u32p, ctypes.c_uint32, _f32p]
        L.orc_scores_f64.restype = None
        L.orc_scores_f64.argtypes = [_u64p, _u32p, _f32p, _f32p, ctypes.c_uint32, _f64p]
        L.orc_sort_tuples_f32.restype = None
        L.orc_sort_tuples_f32.argtypes = [ctypes.c_uint32, _u32p, _f32p]
        L.orc_sort_tuples_i32.restype = None
        L.orc_sort_tuples_i32.argtypes = [ctypes.c_uint32, _u32p, _i32p]
        L.orc_two_stage.restype = ctypes.c_uint32
        L.orc_two_stage.argtypes = [_u64p, _u32p, _f32p, _u64p, _u32p, _i32p, _f32p,
                                    ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.c_uint32, _f32p, _u32p, _f32p, _u32p, _u32p]
        L.orc_bench_two_stage.restype = ctypes.c_double
        L.orc_bench_two_stage.argtypes = [_u64p, _u32p, _f32p, _u64p, _u32p, _i32p,
                                          ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                                          ctypes.c_uint32, ctypes.c_uint32, _f32p,
                                          ctypes.c_uint32, ctypes.c_int, ctypes.c_double, _u32p,
                                          _u32p]
        L.orc_bench_fp32_topk.restype = ctypes.c_double
        L.orc_bench_fp32_topk.argtypes = [_u64p, _u32p, _f32p, ctypes.c_uint32, ctypes.c_uint32,
                                          ctypes.c_uint32, _f32p, ctypes.c_uint32, ctypes.c_int,
                                          ctypes.c_double, _u32p]
        L.orc_gen_matrix.restype = ctypes.c_uint64
        L.orc_gen_matrix.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                     ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                     ctypes.c_int, _u64p, _u32p, _f32p]
        L.orc_two_stage_many.restype = None
        L.orc_two_stage_many.argtypes = [_u64p, _u32p, _f32p, _u64p, _u32p, _i32p, _f32p,
                                         ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_uint32,
                                         ctypes.c_uint32, ctypes.c_uint32, _f32p,
                                         ctypes.c_uint32, ctypes.c_int, _u32p, _f32p, _u32p]
        L.orc_topk_f64_many.restype = None
        L.orc_topk_f64_many.argtypes = [_u64p, _u32p, _f32p, ctypes.c_uint32, ctypes.c_uint32,
                                        _f32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                                        _u32p, _f64p]
        L.orc_topk_f32_many.restype = None
        L.orc_topk_f32_many.argtypes = [_u64p, _u32p, _f32p, ctypes.c_uint32, ctypes.c_uint32,
                                        _f32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                                        _u32p, _f32p]
        L.orc_rows_f64.restype = None
        L.orc_rows_f64.argtypes = [_u64p, _u32p, _f32p, ctypes.c_uint32, _f32p, ctypes.c_uint32,
                                   ctypes.c_uint32, _u32p, _f64p]
        L.orc_resparse.restype = ctypes.c_uint64
        L.orc_resparse.argtypes = [_u64p, _u32p, _f32p, ctypes.c_uint32, ctypes.c_uint32,
                                   ctypes.c_double, _u64p, _u32p, _f32p]
        _lib = L
    return _lib


def ref_lib():
    """The reference's own gold code compiled on this machine, or None."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        try:
            R = ctypes.CDLL(REF_PATH)
        except OSError:
            return None
        R.ref_gold_topk2_i32.restype = None
        R.ref_gold_topk2_i32.argtypes = [_u32p, _u32p, _i32p, ctypes.c_uint64, _i32p,
                                         ctypes.c_int, _u32p, _i32p]
        R.ref_gold_topk_f32.restype = None
        R.ref_gold_topk_f32.argtypes = [_u32p, _u32p, _f32p, ctypes.c_uint64, _f32p,
                                        ctypes.c_int, _u32p, _f32p]
        R.ref_gold4_f32.restype = None
        R.ref_gold4_f32.argtypes = [_u32p, _u32p, _f32p, ctypes.c_uint64, _f32p,
                                    ctypes.c_uint32, _f32p]
        R.ref_sort_tuples_f32.restype = None
        R.ref_sort_tuples_f32.argtypes = [ctypes.c_uint32, _u32p, _f32p]
        R.ref_sort_tuples_i32.restype = None
        R.ref_sort_tuples_i32.argtypes = [ctypes.c_uint32, _u32p, _i32p]
        R.ref_sort_pr_f32.restype = None
        R.ref_sort_pr_f32.argtypes = [ctypes.c_uint32, _f32p, _u32p]
        R.ref_read_mtx.restype = ctypes.c_uint32
        R.ref_read_mtx.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, _u32p, _u32p, _u32p, _u32p, _f32p,
                                   ctypes.c_uint32]
        _ref = R
    return _ref


# ---------------------------------------------------------------------------------------------
# numpy-facing wrappers
# ---------------------------------------------------------------------------------------------

def packet_size(bits: int) -> int:
    return lib().orc_packet_size(bits)


def csr_from_coo(rows, row, col, val):
    """Stable (row, col) sort -> (ptr u64, col u32, val f32)."""
    row = np.asarray(row, np.uint32)
    col = np.asarray(col, np.uint32)
    val = np.asarray(val, np.float32)
    order = np.lexsort((col, row))
    row, col, val = row[order], col[order], val[order]
    ptr = np.zeros(rows + 1, np.uint64)
    np.add.at(ptr, row.astype(np.int64) + 1, 1)
    ptr = np.cumsum(ptr).astype(np.uint64)
    return ptr, np.ascontiguousarray(col), np.ascontiguousarray(val)


def quantize_query(x, bits, quant=QUANT_SYM_GLOBAL, qq=QQ_NUMPY):
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros(x.shape[0], np.int32)
    rc = lib().orc_quantize_query(_p(x, _f32p), x.shape[0], bits, quant, qq, _p(out, _i32p))
    if rc != 0:
        raise ValueError("unsigned query quantiser needs non-negative entries")
    return out


def quantize_matrix(ptr, col, val, rows, cols, bits, quant=QUANT_SYM_GLOBAL, seed=0):
    nnz = int(ptr[-1])
    qptr = np.zeros(rows + 1, np.uint64)
    qcol = np.zeros(nnz + rows + 1, np.uint32)
    qval = np.zeros(nnz + rows + 1, np.int32)
    rs = np.zeros(max(rows, 1), np.float32)
    n = lib().orc_quantize_matrix(_p(ptr, _u64p), _p(col, _u32p), _p(val, _f32p), rows, cols,
                                  bits, quant, seed, _p(qptr, _u64p), _p(qcol, _u32p),
                                  _p(qval, _i32p), _p(rs, _f32p))
    if n == (1 << 64) - 1:
        raise ValueError("unsigned quantiser needs non-negative matrix values")
    return qptr, qcol[:n].copy(), qval[:n].copy(), (rs[:rows].copy() if quant == QUANT_UNSIGNED_ROW else None)


def pack_ultracsr(qptr, qcol, qval, rows, bits, parts=32):
    n = lib().orc_pack_ultracsr(_p(qptr, _u64p), _p(qcol, _u32p), _p(qval, _i32p), rows, bits,
                                parts, None)
    out = np.zeros(max(int(n), 1) * 64, np.uint8)
    lib().orc_pack_ultracsr(_p(qptr, _u64p), _p(qcol, _u32p), _p(qval, _i32p), rows, bits, parts,
                            _p(out, _u8p))
    return out[: int(n) * 64].reshape(int(n), 64)


def xdecode(flags: int, P: int, base: int = 0):
    out = np.zeros(P, np.uint32)
    lib().orc_xdecode(flags, P, base, _p(out, _u32p))
    return out


def unpack_packet(pkt, bits, is_signed=True):
    pkt = np.ascontiguousarray(pkt, np.uint8)
    P = packet_size(bits)
    f = np.zeros(1, np.uint64)
    c = np.zeros(P, np.uint32)
    v = np.zeros(P, np.int32)
    lib().orc_unpack_packet(_p(pkt, _u8p), bits, 1 if is_signed else 0, _p(f, _u64p),
                            _p(c, _u32p), _p(v, _i32p))
    return int(f[0]), c, v


def int_scores(qptr, qcol, qval, rows, qq):
    qq = np.ascontiguousarray(qq, np.int32)
    out = np.zeros(rows, np.int32)
    lib().orc_int_scores(_p(qptr, _u64p), _p(qcol, _u32p), _p(qval, _i32p), rows, _p(qq, _i32p),
                         _p(out, _i32p))
    return out


def cand_keys(scores, rowscale=None):
    scores = np.ascontiguousarray(scores, np.int32)
    keys = np.zeros(scores.shape[0], np.uint32)
    rs = None if rowscale is None else np.ascontiguousarray(rowscale, np.float32)
    lib().orc_cand_keys(_p(scores, _i32p), None if rs is None else _p(rs, _f32p),
                        scores.shape[0], _p(keys, _u32p))
    return keys


def key_f32(x: float) -> int:
    return lib().orc_key_f32(x)


def select_split(keys, split, ck):
    keys = np.ascontiguousarray(keys, np.uint32)
    out = np.zeros(max(ck, 1), np.uint32)
    n = lib().orc_select_split(_p(keys, _u32p), keys.shape[0], split, ck, _p(out, _u32p))
    return out[:n].copy()


def gold_topk2(coo_row, coo_col, coo_val, vec, k, use_ref=False):
    L = ref_lib() if use_ref else lib()
    coo_row = np.ascontiguousarray(coo_row, np.uint32)
    coo_col = np.ascontiguousarray(coo_col, np.uint32)
    coo_val = np.ascontiguousarray(coo_val, np.int32)
    vec = np.ascontiguousarray(vec, np.int32)
    idx = np.zeros(k, np.uint32)
    val = np.zeros(k, np.int32)
    fn = L.ref_gold_topk2_i32 if use_ref else L.orc_gold_topk2
    fn(_p(coo_row, _u32p), _p(coo_col, _u32p), _p(coo_val, _i32p), coo_row.shape[0],
       _p(vec, _i32p), k, _p(idx, _u32p), _p(val, _i32p))
    return idx, val


def gold_topk_f32(coo_row, coo_col, coo_val, vec, k, use_ref=False):
    L = ref_lib() if use_ref else lib()
    coo_row = np.ascontiguousarray(coo_row, np.uint32)
    coo_col = np.ascontiguousarray(coo_col, np.uint32)
    coo_val = np.ascontiguousarray(coo_val, np.float32)
    vec = np.ascontiguousarray(vec, np.float32)
    idx = np.zeros(k, np.uint32)
    val = np.zeros(k, np.float32)
    fn = L.ref_gold_topk_f32 if use_ref else L.orc_gold_topk_f32
    fn(_p(coo_row, _u32p), _p(coo_col, _u32p), _p(coo_val, _f32p), coo_row.shape[0],
       _p(vec, _f32p), k, _p(idx, _u32p), _p(val, _f32p))
    return idx, val


def rescore_f32(ptr, col, val, q, rows_sel):
    q = np.ascontiguousarray(q, np.float32)
    rows_sel = np.ascontiguousarray(rows_sel, np.uint32)
    out = np.zeros(rows_sel.shape[0], np.float32)
    lib().orc_rescore_f32(_p(ptr, _u64p), _p(col, _u32p), _p(val, _f32p), _p(q, _f32p),
                          _p(rows_sel, _u32p), rows_sel.shape[0], _p(out, _f32p))
    return out


def scores_f64(ptr, col, val, q, rows):
    q = np.ascontiguousarray(q, np.float32)
    out = np.zeros(rows, np.float64)
    lib().orc_scores_f64(_p(ptr, _u64p), _p(col, _u32p), _p(val, _f32p), _p(q, _f32p), rows,
                         _p(out, _f64p))
    return out


def sort_tuples_f32(idx, val, use_ref=False):
    idx = np.array(idx, np.uint32)
    val = np.array(val, np.float32)
    L = ref_lib() if use_ref else lib()
    fn = L.ref_sort_tuples_f32 if use_ref else L.orc_sort_tuples_f32
    fn(idx.shape[0], _p(idx, _u32p), _p(val, _f32p))
    return idx, val


class Matrix:
    """A synthetic matrix in the three forms the oracle needs (FP32 CSR, quantised CSR,
    Ultra-CSR packets)."""

    def __init__(self, rows, cols, ptr, col, val, bits, quant=QUANT_SYM_GLOBAL, seed=0,
                 parts=32):
        self.rows, self.cols, self.bits, self.quant = int(rows), int(cols), int(bits), int(quant)
        self.ptr = np.ascontiguousarray(ptr, np.uint64)
        self.col = np.ascontiguousarray(col, np.uint32)
        self.val = np.ascontiguousarray(val, np.float32)
        self.qptr, self.qcol, self.qval, self.rowscale = quantize_matrix(
            self.ptr, self.col, self.val, self.rows, self.cols, self.bits, self.quant, seed)
        self.parts = parts

    def packets(self):
        return pack_ultracsr(self.qptr, self.qcol, self.qval, self.rows, self.bits, self.parts)

    def int_scores(self, query_f32, qq=QQ_NUMPY):
        q = quantize_query(query_f32, self.bits, self.quant, qq)
        return int_scores(self.qptr, self.qcol, self.qval, self.rows, q)

    def keys(self, query_f32, qq=QQ_NUMPY):
        return cand_keys(self.int_scores(query_f32, qq),
                         self.rowscale if self.quant == QUANT_UNSIGNED_ROW else None)

    def two_stage(self, query_f32, split, ck, k, qq=QQ_NUMPY):
        q = np.ascontiguousarray(query_f32, np.float32)
        oi = np.zeros(max(k, 1), np.uint32)
        os_ = np.zeros(max(k, 1), np.float32)
        cand = np.zeros(max(ck, 1), np.uint32)
        cn = np.zeros(1, np.uint32)
        rs = self.rowscale if self.rowscale is not None else np.zeros(1, np.float32)
        n = lib().orc_two_stage(_p(self.ptr, _u64p), _p(self.col, _u32p), _p(self.val, _f32p),
                                _p(self.qptr, _u64p), _p(self.qcol, _u32p),
                                _p(self.qval, _i32p), _p(rs, _f32p), self.rows, self.cols,
                                self.bits, self.quant, qq, split, ck, k, _p(q, _f32p),
                                _p(oi, _u32p), _p(os_, _f32p), _p(cand, _u32p), _p(cn, _u32p))
        return oi[:n].copy(), os_[:n].copy(), cand[: int(cn[0])].copy()


GEN_UNIFORM_DEG = 0
GEN_FIXED_ABSNORMAL = 1
GEN_GAMMA_DEG = 2
GEN_FIXED_UNIFORM = 3


def gen_matrix(kind, rows, cols, p0, p1=0.0, seed=0, nthreads=None):
    """The engine's seeded synthetic CSR (ptr u64, col u32, val f32), built by the oracle."""
    L = lib()
    nt = nthreads or (os.cpu_count() or 1)
    nnz = L.orc_gen_matrix(kind, rows, cols, p0, p1, seed, nt, None, None, None)
    if nnz == (1 << 64) - 1:
        raise ValueError("bad generator arguments")
    ptr = np.zeros(rows + 1, np.uint64)
    col = np.zeros(max(nnz, 1), np.uint32)
    val = np.zeros(max(nnz, 1), np.float32)
    L.orc_gen_matrix(kind, rows, cols, p0, p1, seed, nt, _p(ptr, _u64p), _p(col, _u32p),
                     _p(val, _f32p))
    return ptr, col[:nnz], val[:nnz]


def two_stage_many(m: "Matrix", queries, split, ck, k, qq=QQ_NUMPY, nthreads=None):
    """Matrix.two_stage for every row of `queries` on host threads: (idx [nq, k], score [nq, k],
    n [nq]); entries past n[q] are unset (row 0xFFFFFFFF, score -inf)."""
    Q = np.ascontiguousarray(np.atleast_2d(queries), np.float32)
    nq = Q.shape[0]
    oi = np.full((nq, k), 0xFFFFFFFF, np.uint32)
    os_ = np.full((nq, k), -np.inf, np.float32)
    on = np.zeros(nq, np.uint32)
    rs = m.rowscale if m.rowscale is not None else np.zeros(1, np.float32)
    lib().orc_two_stage_many(_p(m.ptr, _u64p), _p(m.col, _u32p), _p(m.val, _f32p),
                             _p(m.qptr, _u64p), _p(m.qcol, _u32p), _p(m.qval, _i32p),
                             _p(rs, _f32p), m.rows, m.cols, m.bits, m.quant, qq, split, ck, k,
                             _p(Q, _f32p), nq, nthreads or (os.cpu_count() or 1),
                             _p(oi, _u32p), _p(os_, _f32p), _p(on, _u32p))
    return oi, os_, on


def topk_f64_many(ptr, col, val, rows, cols, queries, k, nthreads=None):
    """float64 Top-k of every row per query: (idx [nq, k], score [nq, k]), score descending,
    lower row first among equal scores."""
    Q = np.ascontiguousarray(np.atleast_2d(queries), np.float32)
    nq = Q.shape[0]
    oi = np.zeros((nq, k), np.uint32)
    os_ = np.zeros((nq, k), np.float64)
    lib().orc_topk_f64_many(_p(ptr, _u64p), _p(col, _u32p), _p(val, _f32p), rows, cols,
                            _p(Q, _f32p), nq, k, nthreads or (os.cpu_count() or 1),
                            _p(oi, _u32p), _p(os_, _f64p))
    return oi, os_


def topk_f32_many(ptr, col, val, rows, cols, queries, k, nthreads=None):
    """FP32 exact Top-k of every row per query (the reference's FP32 method, sort_tuples order):
    (idx [nq, k], score [nq, k])."""
    Q = np.ascontiguousarray(np.atleast_2d(queries), np.float32)
    nq = Q.shape[0]
    oi = np.zeros((nq, k), np.uint32)
    os_ = np.zeros((nq, k), np.float32)
    lib().orc_topk_f32_many(_p(ptr, _u64p), _p(col, _u32p), _p(val, _f32p), rows, cols,
                            _p(Q, _f32p), nq, k, nthreads or (os.cpu_count() or 1),
                            _p(oi, _u32p), _p(os_, _f32p))
    return oi, os_


def rows_f64(ptr, col, val, cols, queries, rows_sel):
    """float64 scores of rows_sel [nq, k] against queries [nq, cols] (NaN for row 0xFFFFFFFF)."""
    Q = np.ascontiguousarray(np.atleast_2d(queries), np.float32)
    R = np.ascontiguousarray(rows_sel, np.uint32)
    out = np.zeros(R.shape, np.float64)
    lib().orc_rows_f64(_p(ptr, _u64p), _p(col, _u32p), _p(val, _f32p), cols, _p(Q, _f32p),
                       R.shape[0], R.shape[1], _p(R, _u32p), _p(out, _f64p))
    return out


def bench_two_stage(m: "Matrix", queries, ck, k, nthreads=1, max_seconds=10.0):
    """Time the CPU two-stage method (symmetric quantiser) on host threads.
    Returns (seconds, queries done, result rows [done, k])."""
    Q = np.ascontiguousarray(queries, np.float32)
    done = np.zeros(1, np.uint32)
    out = np.zeros((Q.shape[0], k), np.uint32)
    el = lib().orc_bench_two_stage(_p(m.ptr, _u64p), _p(m.col, _u32p), _p(m.val, _f32p),
                                   _p(m.qptr, _u64p), _p(m.qcol, _u32p), _p(m.qval, _i32p),
                                   m.rows, m.cols, m.bits, ck, k, _p(Q, _f32p), Q.shape[0],
                                   nthreads, max_seconds, _p(done, _u32p), _p(out, _u32p))
    return el, int(done[0]), out[: int(done[0])]


def bench_fp32_topk(m: "Matrix", queries, k, nthreads=1, max_seconds=10.0):
    """Time the CPU FP32 full Top-K (spmv_coo_gold_top_k) on host threads.
    Returns (seconds, queries done)."""
    Q = np.ascontiguousarray(queries, np.float32)
    done = np.zeros(1, np.uint32)
    el = lib().orc_bench_fp32_topk(_p(m.ptr, _u64p), _p(m.col, _u32p), _p(m.val, _f32p),
                                   m.rows, m.cols, k, _p(Q, _f32p), Q.shape[0], nthreads,
                                   max_seconds, _p(done, _u32p))
    return el, int(done[0])


# ---------------------------------------------------------------------------------------------
# numpy restatements (cross-checks of the C code against the Python reference's arithmetic)
# ---------------------------------------------------------------------------------------------

def np_quantify_vector(v, B, symmetric=True):
    """quantify_util.py:31-49 on a float64 copy."""
    v = np.array(v, np.float64)
    M = 2 ** B - 1
    if symmetric:
        M = int(M / 2)
    m = max(abs(np.max(v)), abs(np.min(v)))
    v /= m
    return np.clip(np.int32(np.round(M * v)), int(-M) - 1, int(M))


# ---------------------------------------------------------------------------------------------
# ReSparse and its ratio search
# ---------------------------------------------------------------------------------------------

def resparse(ptr, col, val, rows, cols, keep):
    """orc_resparse: (ptr u64, col u32, val f32) of the kept entries."""
    ptr = np.ascontiguousarray(ptr, np.uint64)
    col = np.ascontiguousarray(col, np.uint32)
    val = np.ascontiguousarray(val, np.float32)
    n = int(ptr[rows])
    op = np.zeros(rows + 1, np.uint64)
    oc = np.zeros(max(n, 1), np.uint32)
    ov = np.zeros(max(n, 1), np.float32)
    k = lib().orc_resparse(_p(ptr, _u64p), _p(col, _u32p), _p(val, _f32p), rows, cols,
                           float(keep), _p(op, _u64p), _p(oc, _u32p), _p(ov, _f32p))
    return op, oc[:k], ov[:k]


TOP_KS = (1, 8, 16, 32, 50, 75, 100)
TOP_K_WEIGHTS = (1.0, 1 / 8, 1 / 16, 1 / 32, 1 / 50, 1 / 75, 1 / 100)


def compt_precision(ref_top_idx, cand):
    """|set(cand) & set(ref[:K])| / K for K in TOP_KS (quantify_util.py:198-219)."""
    c = set(int(x) for x in cand)
    return [len(c & set(int(x) for x in ref_top_idx[:K])) / K for K in TOP_KS]


def convergence_metric(precisions):
    """Weighted sum of the mean precisions (quantify_util.py:413-437)."""
    n = len(precisions)
    avg = [sum(p[i] for p in precisions) / n for i in range(len(TOP_KS))]
    return sum(avg[i] * TOP_K_WEIGHTS[i] for i in range(len(TOP_KS)))


def search_keep_ratio(evaluate, accuracy_threshold=0.999, max_epochs=100):
    """The reference's ReSparse bisection (search_best_resparse_ratio.py:55-117) over an
    evaluate(keep_ratio, epoch) -> convergence-metric callback.  Returns (converged keep ratio
    or None, [(epoch, ratio, metric), ...])."""
    history = []
    high, low = 1.0, 0.0
    attempted = set()
    ratio = 1.0
    threshold = None
    for epoch in range(max_epochs):
        if epoch == 0:
            ratio = 1.0
        elif epoch == 1:
            ratio = (low + high) / 2
        metric = evaluate(ratio, epoch)
        attempted.add(ratio)
        history.append((epoch, ratio, metric))
        if epoch == 0:
            threshold = metric * accuracy_threshold
            continue
        if metric >= threshold:
            high = ratio
        else:
            low = ratio
        ratio = round((low + high) / 2, 3)
        if ratio in attempted:
            return high, history
    return None, history


def ref_read_mtx(path, directed=0, read_values=True, zero_indexed=False, sort=True, cap=1 << 20):
    """readMtx of the reference (needs oracle/_ref): (rows, cols, row, col, val)."""
    R = ref_lib()
    if R is None:
        raise RuntimeError("reference library not built")
    rows, cols = ctypes.c_uint32(0), ctypes.c_uint32(0)
    r = np.zeros(cap, np.uint32)
    c = np.zeros(cap, np.uint32)
    v = np.zeros(cap, np.float32)
    n = R.ref_read_mtx(os.fsencode(path), directed, int(read_values), int(zero_indexed), int(sort),
                       ctypes.byref(rows), ctypes.byref(cols), _p(r, _u32p), _p(c, _u32p),
                       _p(v, _f32p), cap)
    return rows.value, cols.value, r[:n].copy(), c[:n].copy(), v[:n].copy()
