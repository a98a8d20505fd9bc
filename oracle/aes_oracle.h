/*
 * aes_oracle.h -- CPU restatement of the AccelES two-stage low-bit Top-K SpMV path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle: tests/, the smoke() entry point and
 * bench.py's cpu_baseline / reference arm may load it.  The product library never links it and
 * never falls back to it.
 *
 * Every function restates one piece of the reference (zhaijiaqi/AccelES); the reference
 * file:line it follows is cited beside it.  Pinning: the quantizers are checked against
 * golden vectors produced by importing src/resources/python/quantify/quantify_util.py, the
 * streaming Top-K and FP32 gold against the reference's own gold_algorithms.hpp compiled into
 * oracle/_ref (see oracle/Makefile), and the packet decoder against the x_decoder flag word
 * 0x20080200 (src/fpga/src/x_decoder/test_x_decoder.cpp:6).
 */
#ifndef AES_ORACLE_H
#define AES_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* quantiser modes (mirrors include/acceles.h) */
#define ORC_QUANT_SYM_GLOBAL 0   /* quantify_util.py:8-28 / :31-49, symmetric */
#define ORC_QUANT_UNSIGNED_ROW 1 /* per-row max-scaled unsigned (builder-defined) */
#define ORC_QUANT_UNSIGNED_GLOBAL 2 /* quantify_util.py:8-49, symmetric=False, values >= 0 */
#define ORC_QQ_NUMPY 0           /* query: quantify_vector (quantify_util.py:31-49) */
#define ORC_QQ_TRUNC 1           /* query: quantize_vec (quantize_utils.hpp:8-18), unpinned */

/* Ultra-CSR elements per 512-bit packet: types.hpp:161 with Q_AP_INT_VAL_BITWIDTH = bits. */
int orc_packet_size(int bits);

/* ---- quantisers ------------------------------------------------------------------------ */
/* max |v| over n values, in float64 (np.max / np.min of the dense matrix, zeros included). */
double orc_maxabs(const float* v, uint64_t n);
/* one element of quantify_matrix / quantify_vector, symmetric=True:
 *   M = int((2^B-1)/2); clip(int32(round(M * (v / m))), -M-1, M), round = half-to-even. */
int32_t orc_q_sym(double v, double m, int bits);
/* per-row (or per-query) unsigned: clip(round((2^B-1) * (v / m)), 0, 2^B-1). */
int32_t orc_q_unsigned(double v, double m, int bits);
/* quantize_utils.hpp:8-18: ap_fixed<32,B,AP_TRN_ZERO>(2^(B-2) * v), to_int(), ap_int<B>. */
int32_t orc_q_trunc(float v, int bits);
/* quantise one query vector.  mode: ORC_QQ_NUMPY with quant ORC_QUANT_SYM_GLOBAL or
 * ORC_QUANT_UNSIGNED_ROW, or ORC_QQ_TRUNC.  Returns 0, or -1 when an unsigned query has a
 * negative entry.  An all-zero query quantises to all zeros. */
int orc_quantize_query(const float* x, uint32_t cols, int bits, int quant, int qq, int32_t* out);

/* ---- matrix quantisation + empty-row rule --------------------------------------------- */
/* Input: CSR sorted by (row, col): ptr[rows+1], col[nnz], val[nnz].
 * quant = ORC_QUANT_SYM_GLOBAL: global max-abs scale (quantify_matrix).  Zero results are
 *   dropped, as matrix_to_coo does (quantify_util.py:461-467).
 * quant = ORC_QUANT_UNSIGNED_ROW: per-row scale, requires val >= 0; rowscale[r] =
 *   (float)(rowmax / (2^B-1)).
 * quant = ORC_QUANT_UNSIGNED_GLOBAL: quantify_matrix with symmetric=False (M = 2^B-1) on
 *   non-negative values; the result fits an unsigned B-bit field.
 * Rows left empty get one entry of value 1 (check_empty_rows, quantify_util.py:440-445) at a
 *   seeded column: the column of the row's largest |v| (first in column order), value
 *   sign(v)*1 in symmetric mode; a row with no input entries uses splitmix64(seed ^ row) % cols.
 * Output arrays must hold nnz + rows entries (qptr: rows+1).  Returns the quantised nnz, or
 * (uint64_t)-1 on invalid input (negative value in unsigned mode). */
uint64_t orc_quantize_matrix(const uint64_t* ptr, const uint32_t* col, const float* val,
                             uint32_t rows, uint32_t cols, int bits, int quant, uint64_t seed,
                             uint64_t* qptr, uint32_t* qcol, int32_t* qval, float* rowscale);

/* ---- Ultra-CSR packer / decoder --------------------------------------------------------- */
/* Packs the quantised matrix into 64-byte packets, partition by partition
 * (host_spmv_ucsr.cpp:278-319, :388-425; fpga_utils.hpp:438-503).  parts = number of row
 * partitions; partition p holds rows [p*s, (p+1)*s) with s = rows / parts and the remainder on
 * the last partition (quantify_util.py:185-189).  out == NULL counts packets only.
 * Returns the packet count. */
uint64_t orc_pack_ultracsr(const uint64_t* qptr, const uint32_t* qcol, const int32_t* qval,
                           uint32_t rows, int bits, uint32_t parts, uint8_t* out);
/* increment_array (fpga_utils.hpp:279-302; x_decoder.cpp:5-22): out[i] = base +
 * popcount(flags & ((2 << i) - 1)) for i < P. */
void orc_xdecode(uint64_t flags, int P, uint32_t base, uint32_t* out);
/* Q_read_block_x/y/val (fpga_utils.hpp:317-384): unpack one packet. */
void orc_unpack_packet(const uint8_t* pkt, int bits, int is_signed, uint64_t* flags,
                       uint32_t* cols, int32_t* vals);

/* ---- candidate pass ----------------------------------------------------------------------- */
/* integer score per row: sum_j qval * qq[qcol], int32 arithmetic (spmv_coo_gold_top_k_2 with
 * L = int32, gold_algorithms.hpp:249-308; np.dot of int32 arrays). */
void orc_int_scores(const uint64_t* qptr, const uint32_t* qcol, const int32_t* qval,
                    uint32_t rows, const int32_t* qq, int32_t* out);
/* order-preserving 32-bit keys */
uint32_t orc_key_i32(int32_t s);
uint32_t orc_key_f32(float f);
/* candidate keys: key_i32(score) or, with rowscale, key_f32((float)score * rowscale[r]). */
void orc_cand_keys(const int32_t* scores, const float* rowscale, uint32_t rows, uint32_t* keys);
/* split selection (quantify_util.py:173-196, split <= 1 = global top-CK, :260-262): per row
 * partition keep the top floor(ck/split) rows by (key desc, row desc).  Writes candidate rows
 * partition by partition, each partition in (key desc, row desc) order.  Returns the count. */
uint32_t orc_select_split(const uint32_t* keys, uint32_t rows, uint32_t split, uint32_t ck,
                          uint32_t* cand);
/* spmv_coo_gold_top_k_2 (gold_algorithms.hpp:249-308) with V = L = int32, restated with its
 * streaming rule (replace on >=, new worst = first minimum slot). */
void orc_gold_topk2(const uint32_t* coo_row, const uint32_t* coo_col, const int32_t* coo_val,
                    uint64_t nnz, const int32_t* vec, int k, uint32_t* res_idx, int32_t* res_val);
/* spmv_coo_gold_top_k (gold_algorithms.hpp:189-247) with V = float. */
void orc_gold_topk_f32(const uint32_t* coo_row, const uint32_t* coo_col, const float* coo_val,
                       uint64_t nnz, const float* vec, int k, uint32_t* res_idx, float* res_val);

/* ---- exact pass and final order ------------------------------------------------------------- */
/* FP32 rescoring of the given rows, sequential over each row's entries in column order:
 * acc = acc + val*q[col], separately rounded (gold_algorithms.hpp:211-239 with V = float). */
void orc_rescore_f32(const uint64_t* ptr, const uint32_t* col, const float* val, const float* q,
                     const uint32_t* rows, uint32_t n, float* out);
/* float64 score of every row (error reference). */
void orc_scores_f64(const uint64_t* ptr, const uint32_t* col, const float* val, const float* q,
                    uint32_t rows, double* out);
/* sort_tuples (evaluation_utils.hpp:40-62): sort (idx, val) by val desc, idx desc, in place. */
void orc_sort_tuples_f32(uint32_t n, uint32_t* idx, float* val);
void orc_sort_tuples_i32(uint32_t n, uint32_t* idx, int32_t* val);

/* ---- whole path ------------------------------------------------------------------------------ */
/* quantised candidate pass -> split Top-CK -> FP32 rescoring -> final Top-K (sort_tuples order).
 * Returns the number of results written (min(k, candidates)); cand/cand_n report the
 * candidate set (at most ck rows). */
uint32_t orc_two_stage(const uint64_t* ptr, const uint32_t* col, const float* val,
                       const uint64_t* qptr, const uint32_t* qcol, const int32_t* qval,
                       const float* rowscale, uint32_t rows, uint32_t cols, int bits, int quant,
                       int qq, uint32_t split, uint32_t ck, uint32_t k, const float* query,
                       uint32_t* out_idx, float* out_score, uint32_t* cand, uint32_t* cand_n);

/* ---- CPU timing harness ------------------------------------------------------------------- */
/* The two-stage method for up to nq queries on nthreads host threads (symmetric quantiser):
 * each thread runs the streaming Top-CK of gold_algorithms.hpp:249-308 over its row block, the
 * blocks' candidates merge to the Top-CK by (key desc, row desc), then FP32 rescoring and
 * sort_tuples.  Stops once max_seconds have passed (after at least one query).  Returns the
 * elapsed seconds, timed through the thread joins; *done = queries completed; out_idx (may be
 * NULL) receives [done][k] result rows. */
double orc_bench_two_stage(const uint64_t* ptr, const uint32_t* col, const float* val,
                           const uint64_t* qptr, const uint32_t* qcol, const int32_t* qval,
                           uint32_t rows, uint32_t cols, int bits, uint32_t ck, uint32_t k,
                           const float* queries, uint32_t nq, int nthreads, double max_seconds,
                           uint32_t* done, uint32_t* out_idx);

/* FP32 full Top-K timing (spmv_coo_gold_top_k, gold_algorithms.hpp:189-247, V = float): each of
 * nthreads threads runs the streaming Top-k over its row block, then the blocks' results merge by
 * (score desc, row desc).  Same stopping rule and return value as orc_bench_two_stage. */
double orc_bench_fp32_topk(const uint64_t* ptr, const uint32_t* col, const float* val,
                           uint32_t rows, uint32_t cols, uint32_t k, const float* queries,
                           uint32_t nq, int nthreads, double max_seconds, uint32_t* done);

/* ReSparse per-row pruning, restating resparse_spm (quantify_util.py:375-403) on a CSR sorted by
 * (row, col) without duplicates: mean |v| over rows x cols (zeros included, plain double sum in
 * entry order); a row whose smallest nonzero |v| exceeds the mean is kept whole, else its
 * ceil(n * keep) largest |v| are kept (equal |v|: higher column first, the order of the
 * reference's reversed ascending argsort for rows of up to 16 nonzeros), in column order.
 * Explicit zeros are dropped.  out_ptr[rows+1]; out_col/out_val sized ptr[rows].  Returns the
 * kept count. */
uint64_t orc_resparse(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t rows,
                      uint32_t cols, double keep, uint64_t* out_ptr, uint32_t* out_col,
                      float* out_val);

/* ---- seeded synthetic matrices and full-size checks ------------------------------------- */
#define ORC_GEN_UNIFORM_DEG 0     /* degree U{p0..p1}, distinct uniform columns, values U(0,1) */
#define ORC_GEN_FIXED_ABSNORMAL 1 /* degree p0, distinct uniform columns, values |N(0,1)| */
#define ORC_GEN_GAMMA_DEG 2       /* degree min(p1, max(1, round(Gamma(2, p0/2)))), U(0,1) */
#define ORC_GEN_FIXED_UNIFORM 3   /* degree p0, distinct uniform columns, values U(0,1) */
/* The engine's seeded generator (aes_gen_matrix), restated so that the CPU baseline needs no
 * engine library: a CSR sorted by (row, col), identical for the same arguments whatever the
 * thread count.  ptr == NULL returns the nnz only; UINT64_MAX on bad arguments. */
uint64_t orc_gen_matrix(uint32_t kind, uint32_t rows, uint32_t cols, double p0, double p1,
                        uint64_t seed, int nthreads, uint64_t* ptr, uint32_t* col, float* val);
/* orc_two_stage for nq queries [nq][cols] on nthreads threads: out_idx / out_score [nq][k],
 * out_n[q] = results written for query q. */
void orc_two_stage_many(const uint64_t* ptr, const uint32_t* col, const float* val,
                        const uint64_t* qptr, const uint32_t* qcol, const int32_t* qval,
                        const float* rowscale, uint32_t rows, uint32_t cols, int bits, int quant,
                        int qq, uint32_t split, uint32_t ck, uint32_t k, const float* queries,
                        uint32_t nq, int nthreads, uint32_t* out_idx, float* out_score,
                        uint32_t* out_n);
/* float64 Top-k of every row for nq queries (score descending, lower row first among equal
 * scores: numpy's stable argsort of -score), nthreads threads; [nq][k] outputs. */
void orc_topk_f64_many(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t rows,
                       uint32_t cols, const float* queries, uint32_t nq, uint32_t k, int nthreads,
                       uint32_t* out_idx, double* out_score);
/* FP32 exact Top-k of every row (column-order FP32 sums, sort_tuples order), nthreads threads. */
void orc_topk_f32_many(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t rows,
                       uint32_t cols, const float* queries, uint32_t nq, uint32_t k, int nthreads,
                       uint32_t* out_idx, float* out_score);
/* float64 scores of rows_sel[q][i] for query q ([nq][k]; row 0xFFFFFFFF gives NaN). */
void orc_rows_f64(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t cols,
                  const float* queries, uint32_t nq, uint32_t k, const uint32_t* rows_sel,
                  double* out);

#ifdef __cplusplus
}
#endif
#endif
