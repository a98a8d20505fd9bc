/*
 * acceles.h -- C ABI of the GB300 two-stage low-bit Top-K SpMV engine.
 *
 * The engine replaces the reference's quantised host driver `struct SpMV`
 * (zhaijiaqi/AccelES, src/fpga/src/host_spmv_ucsr.cpp:134-829) and its GPU-host twin
 * (src/gpu/host_spmv_topk_csr_gpu_int8.cu:123-314).  Every entry point takes plain pointers and
 * sizes, returns a status code (never exits), and is annotated with the reference interface it
 * stands in for.  One handle owns one device-resident matrix; a handle is used by one host
 * thread at a time.
 *
 * Method (reference README.md:5): the matrix is quantised to B bits and packed as Ultra-CSR
 * (512-bit packets, types.hpp:151-162); a query is quantised the same way; an integer candidate
 * pass scores every row and keeps the Top-CK rows per row partition (split); the candidates are
 * rescored in FP32 against the FP32 matrix and the final Top-K is returned in sort_tuples order
 * (score descending, row index descending; evaluation_utils.hpp:40-62).
 */
#ifndef ACCELES_H
#define ACCELES_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------ */
#define AES_OK 0
#define AES_ERR_INVALID (-1)     /* bad argument or malformed matrix */
#define AES_ERR_UNSUPPORTED (-2) /* bits not in {4,6,8}, cols > 1024, K > 1024, ... */
#define AES_ERR_CUDA (-3)        /* CUDA runtime failure; aes_last_error() has the text */
#define AES_ERR_NOMEM (-4)       /* device memory over the handle's limit, or allocation refused */
#define AES_ERR_QUERY (-5)       /* query rejected (negative entry under an unsigned quantiser) */
#define AES_ERR_STATE (-6)       /* call out of order (run before set_query, ...) */
#define AES_ERR_NODEV (-7)       /* no CUDA device */

/* ---- quantiser choices ---------------------------------------------------------------------- */
/* matrix + query quantiser */
#define AES_QUANT_SYM_GLOBAL 0      /* quantify_matrix/quantify_vector, symmetric=True
                                       (quantify_util.py:8-49): the reference's default */
#define AES_QUANT_UNSIGNED_ROW 1    /* per-row max-scaled unsigned B-bit matrix, per-query
                                       unsigned query; candidate key = rowscale * int score */
#define AES_QUANT_UNSIGNED_GLOBAL 2 /* quantify_matrix/quantify_vector, symmetric=False, on
                                       non-negative data */
/* query quantiser */
#define AES_QQ_NUMPY 0 /* quantify_vector (quantify_util.py:31-49) */
#define AES_QQ_TRUNC 1 /* quantize_vec (quantize_utils.hpp:8-18): trunc(2^(B-2) * v) */

typedef struct aes_handle aes_handle;

typedef struct aes_params {
  uint32_t bits;          /* B: 4, 6 or 8 (QUANTIZE_B, types.hpp:148) */
  uint32_t quant;         /* AES_QUANT_* */
  uint32_t query_quant;   /* AES_QQ_* */
  uint32_t split;         /* row partitions of the Top-CK select; <= 1 means one global
                             Top-CK (SPLIT, quantify_util.py:173-196 / SPMV_PARTITIONS) */
  uint32_t ck;            /* candidates kept (APPROXIMATE_K, types.hpp:149) */
  uint32_t k_max;         /* largest K a run may request (<= 1024) */
  uint32_t max_batch;     /* most queries per aes_set_query / aes_run_device call */
  uint32_t pack_parts;    /* Ultra-CSR packing partitions (SPMV_PARTITIONS = 32) */
  uint32_t sample_stride; /* threshold sample: one 32-packet tile in this many (0 = auto) */
  uint32_t batch_tile;    /* queries per matrix pass in the batched kernel (0 = auto) */
  int32_t device;         /* CUDA device ordinal */
  uint32_t flags;         /* AES_FLAG_* bits */
  uint64_t seed;          /* seed of the empty-row rule (check_empty_rows is unseeded) */
  uint64_t mem_limit;     /* device bytes this handle may allocate; 0 = no limit */
  uint32_t batch_warps;   /* warps per CTA of the batched dp4a pass (0 = auto: the most whose
                             element records fit in shared memory next to the query table, at
                             most 16); a larger value is lowered to that */
} aes_params;

/* params.flags bits */
#define AES_FLAG_PROFILE 1u /* time every candidate-pass launch with CUDA events on its stream */
#define AES_FLAG_GRAPHS 2u  /* replay each batch's launch sequence as a CUDA graph (captured once
                               per set of buffers, batch size and K); profiling events are
                               not recorded inside graphs */
#define AES_FLAG_POSITIVE 8u /* aes_read_candidates returns only candidates whose score is above
                               0, as Q_read_result keeps only positive slots
                               (host_spmv_ucsr.cpp:709); the final Top-K is unaffected */
#define AES_FLAG_TENSOR 4u  /* 4-bit matrices: lay the quantised entries out for the tensor
                               cores at creation (4 B per entry) and run the batched candidate
                               pass as FP8 tcgen05 products of 128-row tiles; the integers are
                               exact in FP8 and the scores exact in FP32, so results equal the
                               dp4a pass.  Ignored for 6- and 8-bit matrices, for matrices with
                               duplicate (row, col) entries and for split > 32 */

#define AES_FLAG_TEST_IDLE_MMA 16u /* failure-path tests only: the tensor-core pass's MMA role
                                     issues nothing, so the other roles' bounded waits run out
                                     (about a second); the pass gives up, frees its tensor
                                     memory and aes_run / aes_finish return AES_ERR_CUDA.  Has
                                     no effect on the other passes */

typedef struct aes_stats {
  uint64_t launches;       /* kernels launched by the engine since the last reset */
  uint64_t cand_launches;  /* full-matrix candidate-pass launches (the dominant kernel) */
  double cand_ms;          /* device time of those launches (AES_FLAG_PROFILE only) */
  uint64_t cand_timed;     /* launches included in cand_ms */
  uint64_t repaired;       /* queries sent down the exact slow path */
} aes_stats;

typedef struct aes_info {
  uint32_t rows, cols, bits, packet_elems;
  uint64_t nnz, quantized_nnz, packets, tiles;
  uint64_t packet_bytes;  /* Ultra-CSR bytes streamed by one full candidate pass */
  uint64_t device_bytes;  /* device memory held by the handle */
  uint32_t split, ck, ck_effective, sample_tiles;
  uint32_t sample_rows, max_batch, batch_tile;
  uint32_t tensor_tiles;  /* 1 when the batched candidate pass runs on the tensor cores */
  uint32_t exact_pass;    /* 1 when FP32 values are resident (the final Top-K is rescored in
                             FP32); 0 for a pre-quantised matrix created without them */
  uint32_t batch_warps;   /* warps per CTA of the batched dp4a pass (0: plain passes only) */
} aes_info;

/* Defaults: bits 6, AES_QUANT_SYM_GLOBAL, AES_QQ_NUMPY, split 32, ck 512, k_max 100
 * (types.hpp:39,148-149; options.hpp:50), max_batch 1, pack_parts 32. */
void aes_params_default(aes_params* p);

/* Build a device-resident matrix from a COO (any order; duplicates are kept as separate
 * entries and summed).  Quantises, fixes rows left empty, packs Ultra-CSR and uploads it
 * together with the FP32 CSR used by the exact pass.  Replaces the quantised constructor
 * SpMV(ConfigOpenCL&, q_x, q_y, q_val, rows, cols, nnz, q_vec, debug)
 * (host_spmv_ucsr.cpp:198-218) plus Q_packet_coo (:278) and Q_setup (:501); the caller keeps
 * ownership of its arrays. */
int aes_create(const uint32_t* row, const uint32_t* col, const float* val, uint32_t rows,
               uint32_t cols, uint64_t nnz, const aes_params* p, aes_handle** out);
/* The quantised constructor as the reference has it: SpMV(ConfigOpenCL&, q_x, q_y, q_val, rows,
 * cols, nnz, q_vec, debug) (host_spmv_ucsr.cpp:198-218) with Q_packet_coo (:278) and Q_setup
 * (:501).  q_val holds the B-bit signed values (the reference's ap_int<B> q_type) of a matrix
 * quantised by the caller, e.g. from a _quantified_B*.mtx file (:969); p->quant must be
 * AES_QUANT_SYM_GLOBAL and every value in [-2^(B-1), 2^(B-1) - 1] (else AES_ERR_INVALID).  The
 * entries are packed as given (zeros included); a row without entries gets one zero entry.
 * val (may be NULL) holds the entries' FP32 values for the exact pass: without them the final
 * Top-K ranks the candidates by their integer score and aes_run_exact is unavailable. */
int aes_create_quantized(const uint32_t* row, const uint32_t* col, const int8_t* q_val,
                         const float* val, uint32_t rows, uint32_t cols, uint64_t nnz,
                         const aes_params* p, aes_handle** out);
/* Same from a CSR already sorted by (row, col): ptr[rows+1]. */
int aes_create_csr(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t rows,
                   uint32_t cols, const aes_params* p, aes_handle** out);
/* A view: a second handle on the resident matrix of `base` (no copy of the matrix), with its own
 * stream, per-batch buffers and configuration p (NULL: base's parameters; bits, quant,
 * pack_parts, seed and device must equal base's).  Batches run on base and on its views at the
 * same time, so a server keeps several batches of one matrix in flight.  The matrix arrays are
 * freed with the last of the handle and its views; each is destroyed with aes_destroy, and each
 * is used by one host thread at a time.  aes_info.device_bytes of a view counts only its own
 * arrays.  No reference counterpart (the reference runs one query at a time, host_spmv_ucsr.cpp:
 * 1084-1113). */
int aes_create_view(const aes_handle* base, const aes_params* p, aes_handle** out);
int aes_destroy(aes_handle* h);
int aes_get_info(const aes_handle* h, aes_info* info);

/* Change ck, split, sample_stride, batch_tile, k_max, max_batch, flags, query_quant or
 * mem_limit of a resident matrix without packing it again (bits, quant, pack_parts, seed and
 * device must equal the creation's: AES_ERR_INVALID otherwise).  Waits for the device, frees
 * the per-batch buffers and allocates the new ones; loaded queries and results are dropped.
 * If the new buffers do not fit, the previous configuration is restored and the error returned.
 * No reference counterpart: the reference fixes these as compile-time constants of the
 * bitstream (APPROXIMATE_K, SPMV_PARTITIONS: types.hpp:39,149). */
int aes_retune(aes_handle* h, const aes_params* p);

/* Load nq FP32 queries (row-major [nq][cols], host memory) for the next aes_run.
 * Replaces Q_reset(q_type* vec, int debug) (host_spmv_ucsr.cpp:790-828) / reset(vec)
 * (host_spmv_topk_csr_gpu_int8.cu:288); quantisation happens on the device. */
int aes_set_query(aes_handle* h, const float* q, uint32_t nq);

/* Load nq pre-quantised queries ([nq][cols] B-bit signed values, host memory) for the next
 * aes_run: the candidate pass takes them as given, without the query quantiser.  Replaces
 * Q_reset(q_type* vec, int debug) (host_spmv_ucsr.cpp:790-828) with the reference's quantised
 * vector.  q_f32 (may be NULL) holds the same queries in FP32 for the exact pass; without it the
 * final Top-K ranks the candidates by their integer score (out_score = that score).  The
 * handle's quantiser must be AES_QUANT_SYM_GLOBAL; a value outside [-2^(B-1), 2^(B-1) - 1]
 * returns AES_ERR_QUERY. */
int aes_set_query_quantized(aes_handle* h, const int8_t* q, const float* q_f32, uint32_t nq);

/* Run the loaded queries: candidate pass, Top-CK select, FP32 rescoring, Top-K.  out_idx and
 * out_score are host arrays [nq][k]; entries past the number of candidates are row
 * 0xFFFFFFFF with score -inf.  *ns (may be NULL) receives the device time in nanoseconds.
 * Replaces operator()(bool, int debug) (host_spmv_ucsr.cpp:556-565) with Q_wait (:605) and the
 * merge of Q_read_result (:691-748). */
int aes_run(aes_handle* h, uint32_t k, uint32_t* out_idx, float* out_score, uint64_t* ns);

/* FP32-only single-stage Top-K of the loaded queries: the FP32 score of every row, sequential
 * in column order, and the exact Top-K in sort_tuples order; no quantisation, no candidates.
 * Replaces the software check of the reference (sw_test: spmv_coo_gold_top_k + sort_tuples,
 * host_spmv_ucsr.cpp:841-869; gold_algorithms.hpp:189-247).  Host outputs [nq][k]; *ns gets
 * the summed device time. */
int aes_run_exact(aes_handle* h, uint32_t k, uint32_t* out_idx, float* out_score, uint64_t* ns);

/* Candidates of query `query` of the last run in sort_tuples order (key descending, row
 * descending).  score_i32 gets the integer candidate score, key_f32 the ranking key (the
 * integer score, or rowscale * score under AES_QUANT_UNSIGNED_ROW); either may be NULL.
 * Replaces Q_read_result(res, idx, debug) (host_spmv_ucsr.cpp:691-748).  With AES_FLAG_POSITIVE
 * in the handle's flags only candidates scoring above 0 are returned, as the reference's
 * `tmp_val > 0` (:709) keeps them; otherwise every candidate is. */
int aes_read_candidates(aes_handle* h, uint32_t query, uint32_t* idx, int32_t* score_i32,
                        float* key_f32, uint32_t cap, uint32_t* n);

/* Device-resident variant: d_queries [nq][cols] FP32 and outputs [nq][k] are device pointers,
 * `stream` a cudaStream_t (NULL = the handle's stream).  Asynchronous: call aes_finish before
 * reading the outputs.  No reference counterpart (the reference always stages through host
 * buffers); it is the resident-input entry a serving loop uses. */
int aes_run_device(aes_handle* h, const float* d_queries, uint32_t nq, uint32_t k,
                   uint32_t* d_idx, float* d_score, void* stream);
/* One query through the whole path without allocating any memory.  No counterpart in the
 * reference.  For callers that must not call cudaMalloc (or anything that allocates) once they
 * are serving: allocation can block and synchronise the device, fail when a framework's caching
 * allocator already holds the free memory, or is simply forbidden on a latency-critical path.
 * The per-query scratch (quantised query, sample keys, thresholds, survivors, candidates) is a
 * fixed 16 MiB device array inside the library instead; matrices whose scratch would not fit
 * are rejected with AES_ERR_UNSUPPORTED.  d_query [cols] FP32, d_idx / d_score [k] are device
 * pointers; `stream` a cudaStream_t (NULL = the handle's stream).  Synchronous: it waits for
 * `stream` to read the query's status word before it returns (and, when the sample threshold
 * missed, runs the exact slow path).  The first call on a device looks up the array's device
 * address, so make that call before any stream capture.  All calls share the one array: calls
 * that overlap on the GPU race and must not be issued.  Its launches and repairs count in
 * aes_get_stats like those of aes_run_device. */
int aes_run_noalloc(aes_handle* h, const float* d_query, uint32_t k, uint32_t* d_idx,
                    float* d_score, void* stream);

/* Wait for the last aes_run_device and repair any query whose fast path reported a sample
 * threshold miss or a survivor-buffer overflow (exact slow path).  *repaired (may be NULL)
 * receives the number of repaired queries. */
int aes_finish(aes_handle* h, uint32_t* repaired);

/* Candidate-pass keys of every row for one host FP32 query: keys[rows] receives the
 * order-preserving key of the integer score (score ^ 0x80000000), or of rowscale * score under
 * AES_QUANT_UNSIGNED_ROW.  Synchronous.  The integer counterpart of the reference's full SpMV
 * check (spmv_coo_gold4 + sort_pr in sw_test, host_spmv_ucsr.cpp:841-869). */
int aes_score_all(aes_handle* h, const float* q, uint32_t* keys);

/* Counters since the previous call (reset = 1 clears them).  Waits for the handle's pending
 * timing events. */
int aes_get_stats(aes_handle* h, aes_stats* st, int reset);

/* Text of the last error on this thread. */
const char* aes_last_error(void);

/* Host-only (no device): quantise and pack a CSR sorted by (row, col) exactly as
 * aes_create_csr does and return the Ultra-CSR packets in reference order (partition by
 * partition, 64 bytes each, the layout Q_packet_coo_partition + Q_write_block_x/y/val write:
 * host_spmv_ucsr.cpp:388-425, fpga_utils.hpp:438-503).  Pass packets == NULL to learn
 * *n_packets.  tile_rowbase (may be NULL) receives ceil(n_packets/32)+1 prefix counts of row
 * flags per 32-packet tile. */
int aes_pack_host(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t rows,
                  uint32_t cols, const aes_params* p, uint8_t* packets, uint64_t cap_packets,
                  uint64_t* n_packets, uint32_t* tile_rowbase);

/* Host-only: the tensor-core tile layout that aes_create builds for a 4-bit matrix with
 * AES_FLAG_TENSOR in p->flags (no device needed; no reference counterpart).  Entries of each
 * 128-row tile grouped by 256-column chunk, tile-major; entry = (byte offset of (row in tile,
 * column in chunk) in the K-major FP8 operand: (k/16)*2048 + (r/8)*128 + (r%8)*16 + k%16) << 16
 * | e4m3 byte of the quantised value.  tile_ptr[t * chunks + c] is the first entry of (tile t,
 * chunk c); chunks = ceil(ceil32(cols) / 256).  Pass NULL arrays to get the sizes only;
 * *n_entries = 0 when the layout is not built (not 4-bit, flag clear, or a repeated
 * (row, col)). */
int aes_pack_tc_host(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t rows,
                     uint32_t cols, const aes_params* p, uint32_t* tile_ptr, uint64_t cap_ptr,
                     uint32_t* entries, uint64_t cap_entries, uint64_t* n_ptr,
                     uint64_t* n_entries);

/* ---- seeded synthetic matrices (the reference matrices are not shipped) ------------------ */
#define AES_GEN_UNIFORM_DEG 0 /* degree U{p0..p1}, distinct uniform columns, values U(0,1) */
#define AES_GEN_FIXED_ABSNORMAL 1 /* degree p0, distinct uniform columns, values |N(0,1)| */
#define AES_GEN_GAMMA_DEG 2   /* degree min(p1, max(1, round(Gamma(2, p0/2)))), values U(0,1) */
#define AES_GEN_FIXED_UNIFORM 3 /* degree p0, distinct uniform columns, values U(0,1) */
/* Pass ptr == NULL to get the total nnz only; then call again with arrays of that size.
 * Output is a CSR sorted by (row, col).  Deterministic for (kind, rows, cols, p0, p1, seed)
 * whatever the thread count.  Returns nnz, or (uint64_t)-1 on bad arguments. */
uint64_t aes_gen_matrix(uint32_t kind, uint32_t rows, uint32_t cols, double p0, double p1,
                        uint64_t seed, uint64_t* ptr, uint32_t* col, float* val);

/* ---- Matrix Market files ------------------------------------------------------------------ */
#define AES_MTX_ZERO_INDEXED 1u  /* indices in the file start at 0 (the reference host reads its
                                    .mtx files this way: host_spmv_ucsr.cpp:938,969) */
#define AES_MTX_SORT 2u          /* order entries by (row, col); equal keys keep file order */
#define AES_MTX_KEEP_DIRECTED 4u /* do not mirror the off-diagonal entries of a symmetric file */
/* Read a coordinate Matrix Market file (real, integer or pattern; general or symmetric) into a
 * COO whose arrays the library allocates (release each with aes_free).  Entries come in file
 * order, then the mirrored off-diagonal entries of a symmetric file; pattern entries read as
 * 1.0; values are parsed as double and rounded to FP32.  Replaces readMtx + readTuples +
 * undirect + customSort (utils.hpp:331-492, mmio.hpp), which exit() on errors where this
 * returns AES_ERR_INVALID (bad banner, entry count, index out of range). */
int aes_read_mtx(const char* path, uint32_t flags, uint32_t* rows, uint32_t* cols, uint64_t* nnz,
                 uint32_t** row, uint32_t** col, float** val);
void aes_free(void* p);
/* Write a COO as "%%MatrixMarket matrix coordinate real general", a "%" line, the size line
 * and one "row col value" line per entry (one-based unless AES_MTX_ZERO_INDEXED), values with
 * 9 significant digits (FP32 values read back exactly).  Replaces write_coo_to_mtx
 * (quantify_util.py:469-477), which takes the shape from the largest indices instead. */
int aes_write_mtx(const char* path, const uint32_t* row, const uint32_t* col, const float* val,
                  uint32_t rows, uint32_t cols, uint64_t nnz, uint32_t flags);

/* ---- ReSparse: per-row pruning before quantisation ---------------------------------------- */
/* For each row of a CSR (sorted, no duplicate (row, col)): if its smallest nonzero |v| exceeds
 * the mean |v| of the whole rows x cols matrix (zeros included), keep the row; else keep its
 * ceil(n * keep) largest |v| (equal |v|: the higher column first), in column order.  Explicit
 * zeros are dropped.  keep in (0, 1].  out_ptr[rows+1]; pass out_col = out_val = NULL to learn
 * *out_nnz.  Replaces resparse_spm (quantify_util.py:375-403), a dense-matrix loop in numpy. */
int aes_resparse(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t rows,
                 uint32_t cols, double keep, uint64_t* out_ptr, uint32_t* out_col,
                 float* out_val, uint64_t cap, uint64_t* out_nnz);

#ifdef __cplusplus
}
#endif
#endif
