/*
 * aes_oracle.c -- CPU restatement of the AccelES two-stage low-bit Top-K SpMV path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle of tests/, smoke() and bench.py's CPU legs.  The
 * product library (acceles_gb300) never links or calls this file.
 *
 * Build with -ffp-contract=off: the FP32 gold sums are separately rounded multiply-then-add,
 * which is what the GPU exact pass computes too.  References are to files of
 * zhaijiaqi/AccelES.
 */
#include "aes_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* types.hpp:151-162: ULTRACSR_PACKET_SIZE = (512 - DIM_BOOL) / (B + 10 + 1), DIM_BOOL = 1. */
int orc_packet_size(int bits) { return 511 / (bits + 11); }

/* ---------------------------------------------------------------------------------------- */
/* quantisers                                                                                */
/* ---------------------------------------------------------------------------------------- */

double orc_maxabs(const float* v, uint64_t n) {
  /* quantify_util.py:24-26: max(abs(np.max(m)), abs(np.min(m))) over the dense matrix; the
   * implicit zeros contribute |0|, so this is the max |v| over the stored values. */
  double m = 0.0;
  for (uint64_t i = 0; i < n; i++) {
    double a = fabs((double)v[i]);
    if (a > m) m = a;
  }
  return m;
}

int32_t orc_q_sym(double v, double m, int bits) {
  /* quantify_util.py:21-27 (matrix) and :45-49 (vector): M = int((2^B-1)/2),
   * clip(int32(round(M * (v / m))), -M-1, M) with numpy's round-half-to-even. */
  int32_t M = ((1 << bits) - 1) / 2;
  if (m == 0.0) return 0;
  double x = v / m;
  double y = (double)M * x;
  double r = nearbyint(y); /* default rounding mode: to nearest, ties to even */
  int32_t q = (int32_t)r;
  if (q < -M - 1) q = -M - 1;
  if (q > M) q = M;
  return q;
}

int32_t orc_q_unsigned(double v, double m, int bits) {
  int32_t M = (1 << bits) - 1;
  if (m == 0.0) return 0;
  double x = v / m;
  double y = (double)M * x;
  double r = nearbyint(y);
  int32_t q = (int32_t)r;
  if (q < 0) q = 0;
  if (q > M) q = M;
  return q;
}

int32_t orc_q_trunc(float v, int bits) {
  /* quantize_utils.hpp:8-18.  q_temp = ap_fixed<32, B, AP_TRN_ZERO> (fpga_types.hpp:235, with
   * B = QUANTIZE_B): (q_temp)(2^(B-2) * v) keeps 32-B fractional bits, truncating toward zero,
   * and wraps the integer part (default AP_WRAP); to_int() truncates toward zero; the ap_int<B>
   * cast wraps to B bits.  Parity unpinned: the ap_fixed sources are not available. */
  int F = 32 - bits;
  double x = (double)v * ldexp(1.0, bits - 2 + F); /* exact: power-of-two scaling */
  double t = trunc(x);
  /* beyond the int64 range x is a multiple of 2^32: its low 32 bits are zero */
  int64_t X = fabs(t) >= 9.2e18 ? 0 : (int64_t)t;
  int32_t X32 = (int32_t)(uint32_t)(uint64_t)X;    /* 32-bit two's-complement wrap */
  int32_t n = X32 / (int32_t)(1u << F);           /* C division truncates toward zero */
  int32_t mask = (1 << bits) - 1;
  int32_t half = 1 << (bits - 1);
  int32_t w = ((n & mask) ^ half) - half;          /* ap_int<B> wrap */
  return w;
}

int orc_quantize_query(const float* x, uint32_t cols, int bits, int quant, int qq, int32_t* out) {
  if (qq == ORC_QQ_TRUNC) {
    for (uint32_t j = 0; j < cols; j++) out[j] = orc_q_trunc(x[j], bits);
    return 0;
  }
  if (quant == ORC_QUANT_UNSIGNED_ROW || quant == ORC_QUANT_UNSIGNED_GLOBAL) {
    /* per-query unsigned scale; for UNSIGNED_GLOBAL this is quantify_vector(symmetric=False),
     * whose clip bound -M-1 never binds on non-negative input */
    double m = 0.0;
    for (uint32_t j = 0; j < cols; j++) {
      if (x[j] < 0.0f) return -1;
      if ((double)x[j] > m) m = (double)x[j];
    }
    for (uint32_t j = 0; j < cols; j++) out[j] = orc_q_unsigned((double)x[j], m, bits);
    return 0;
  }
  double m = orc_maxabs(x, cols);
  for (uint32_t j = 0; j < cols; j++) out[j] = orc_q_sym((double)x[j], m, bits);
  return 0;
}

/* ---------------------------------------------------------------------------------------- */
/* matrix quantisation + seeded empty-row rule                                               */
/* ---------------------------------------------------------------------------------------- */

static uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

uint64_t orc_quantize_matrix(const uint64_t* ptr, const uint32_t* col, const float* val,
                             uint32_t rows, uint32_t cols, int bits, int quant, uint64_t seed,
                             uint64_t* qptr, uint32_t* qcol, int32_t* qval, float* rowscale) {
  uint64_t nnz = ptr[rows];
  double gm = 0.0;
  if (quant == ORC_QUANT_SYM_GLOBAL) {
    gm = orc_maxabs(val, nnz);
  } else {
    if (quant == ORC_QUANT_UNSIGNED_GLOBAL) gm = orc_maxabs(val, nnz);
    for (uint64_t e = 0; e < nnz; e++)
      if (val[e] < 0.0f) return (uint64_t)-1;
  }
  uint64_t o = 0;
  qptr[0] = 0;
  for (uint32_t r = 0; r < rows; r++) {
    uint64_t b = ptr[r], e_end = ptr[r + 1];
    double m = gm;
    if (quant == ORC_QUANT_UNSIGNED_ROW) {
      m = 0.0;
      for (uint64_t e = b; e < e_end; e++)
        if ((double)val[e] > m) m = (double)val[e];
      rowscale[r] = (float)(m / (double)((1 << bits) - 1));
    }
    uint64_t start = o;
    for (uint64_t e = b; e < e_end; e++) {
      int32_t q = (quant == ORC_QUANT_SYM_GLOBAL) ? orc_q_sym((double)val[e], m, bits)
                                                  : orc_q_unsigned((double)val[e], m, bits);
      /* UNSIGNED_GLOBAL: quantify_matrix(symmetric=False) clips to [-M-1, M]; with values >= 0
       * that is orc_q_unsigned with the global scale */
      if (q != 0) { /* matrix_to_coo keeps value != 0 only */
        qcol[o] = col[e];
        qval[o] = q;
        o++;
      }
    }
    if (o == start) { /* empty after quantisation: check_empty_rows puts a 1 in the row */
      uint32_t c;
      int32_t v = 1;
      if (e_end > b) {
        uint64_t best = b;
        double ba = fabs((double)val[b]);
        for (uint64_t e = b + 1; e < e_end; e++) {
          double a = fabs((double)val[e]);
          if (a > ba) { ba = a; best = e; }
        }
        c = col[best];
        if (quant == ORC_QUANT_SYM_GLOBAL && val[best] < 0.0f) v = -1;
      } else {
        c = (uint32_t)(splitmix64(seed ^ (uint64_t)r) % (uint64_t)cols);
      }
      qcol[o] = c;
      qval[o] = v;
      o++;
    }
    qptr[r + 1] = o;
  }
  return o;
}

/* ---------------------------------------------------------------------------------------- */
/* Ultra-CSR packets                                                                          */
/* ---------------------------------------------------------------------------------------- */

/* ap_uint<512>.range(hi, lo): bit i lives in byte i >> 3, bit i & 7. */
static void put_bits(uint8_t* pkt, int pos, int width, uint32_t v) {
  for (int b = 0; b < width; b++) {
    int i = pos + b;
    if ((v >> b) & 1u) pkt[i >> 3] |= (uint8_t)(1u << (i & 7));
    else pkt[i >> 3] &= (uint8_t)~(1u << (i & 7));
  }
}

static uint32_t get_bits(const uint8_t* pkt, int pos, int width) {
  uint32_t v = 0;
  for (int b = 0; b < width; b++) {
    int i = pos + b;
    v |= (uint32_t)((pkt[i >> 3] >> (i & 7)) & 1u) << b;
  }
  return v;
}

uint64_t orc_pack_ultracsr(const uint64_t* qptr, const uint32_t* qcol, const int32_t* qval,
                           uint32_t rows, int bits, uint32_t parts, uint8_t* out) {
  const int P = orc_packet_size(bits);
  if (parts == 0) parts = 1;
  uint32_t slice = rows / parts;
  uint64_t npk = 0;
  uint32_t last_row = 0; /* host_spmv_ucsr.cpp:304: r_last = 0 before partition 0 */
  for (uint32_t p = 0; p < parts; p++) {
    uint32_t r0 = p * slice;
    uint32_t r1 = (p == parts - 1) ? rows : (p + 1) * slice;
    uint64_t e0 = qptr[r0], e1 = qptr[r1];
    uint64_t n = e1 - e0;
    uint64_t np = (n + (uint64_t)P - 1) / (uint64_t)P;
    if (out) {
      uint32_t r = r0;
      for (uint64_t k = 0; k < np; k++) {
        uint8_t* pkt = out + (npk + k) * 64;
        memset(pkt, 0, 64);
        for (int j = 0; j < P; j++) {
          uint64_t e = e0 + k * (uint64_t)P + (uint64_t)j;
          if (e >= e1) break; /* tail slots stay flag 0, col 0, val 0 (:407-411) */
          while (qptr[r + 1] <= e) r++;
          uint32_t flag = (r != last_row) ? 1u : 0u; /* :401-403 */
          last_row = r;
          put_bits(pkt, j, 1, flag);
          put_bits(pkt, P + 10 * j, 10, qcol[e] & 0x3FFu);
          put_bits(pkt, 11 * P + bits * j, bits, (uint32_t)qval[e] & ((1u << bits) - 1u));
        }
      }
    } else if (n) {
      /* keep last_row consistent for counting-only calls */
      uint32_t r = r1 - 1;
      while (qptr[r] == qptr[r + 1] && r > r0) r--;
      last_row = r;
    }
    npk += np;
  }
  return npk;
}

void orc_xdecode(uint64_t flags, int P, uint32_t base, uint32_t* out) {
  for (int i = 0; i < P; i++) {
    uint64_t m = (i >= 63) ? ~0ull : ((2ull << i) - 1ull);
    out[i] = base + (uint32_t)__builtin_popcountll(flags & m);
  }
}

void orc_unpack_packet(const uint8_t* pkt, int bits, int is_signed, uint64_t* flags,
                       uint32_t* cols, int32_t* vals) {
  const int P = orc_packet_size(bits);
  uint64_t f = 0;
  for (int j = 0; j < P; j++) {
    f |= (uint64_t)get_bits(pkt, j, 1) << j;
    cols[j] = get_bits(pkt, P + 10 * j, 10);
    uint32_t v = get_bits(pkt, 11 * P + bits * j, bits);
    if (is_signed && (v >> (bits - 1))) vals[j] = (int32_t)v - (1 << bits);
    else vals[j] = (int32_t)v;
  }
  *flags = f;
}

/* ---------------------------------------------------------------------------------------- */
/* candidate pass                                                                             */
/* ---------------------------------------------------------------------------------------- */

void orc_int_scores(const uint64_t* qptr, const uint32_t* qcol, const int32_t* qval,
                    uint32_t rows, const int32_t* qq, int32_t* out) {
  for (uint32_t r = 0; r < rows; r++) {
    uint32_t acc = 0; /* int32 wrap-around arithmetic, as the int32 accumulator computes */
    for (uint64_t e = qptr[r]; e < qptr[r + 1]; e++)
      acc += (uint32_t)(qval[e] * qq[qcol[e]]);
    out[r] = (int32_t)acc;
  }
}

uint32_t orc_key_i32(int32_t s) { return (uint32_t)s ^ 0x80000000u; }

uint32_t orc_key_f32(float f) {
  if (f == 0.0f) f = 0.0f; /* -0 and +0 compare equal in sort_tuples */
  uint32_t u;
  memcpy(&u, &f, 4);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

void orc_cand_keys(const int32_t* scores, const float* rowscale, uint32_t rows, uint32_t* keys) {
  for (uint32_t r = 0; r < rows; r++) {
    if (rowscale) {
      float s = (float)scores[r];
      keys[r] = orc_key_f32(s * rowscale[r]);
    } else {
      keys[r] = orc_key_i32(scores[r]);
    }
  }
}

typedef struct {
  uint64_t comp; /* key << 32 | row: (key desc, row desc) is descending comp */
} comp_t;

static int cmp_comp_desc(const void* a, const void* b) {
  uint64_t x = ((const comp_t*)a)->comp, y = ((const comp_t*)b)->comp;
  return (x > y) ? -1 : (x < y) ? 1 : 0;
}

uint32_t orc_select_split(const uint32_t* keys, uint32_t rows, uint32_t split, uint32_t ck,
                          uint32_t* cand) {
  uint32_t S = split <= 1 ? 1 : split;
  uint32_t ntop = ck / S; /* int(APPROXIMATE_K / split_size), quantify_util.py:194 */
  uint32_t slice = rows / S;
  uint32_t outn = 0;
  comp_t* buf = (comp_t*)malloc(sizeof(comp_t) * (rows ? rows : 1));
  for (uint32_t p = 0; p < S; p++) {
    uint32_t r0 = p * slice;
    uint32_t r1 = (p == S - 1) ? rows : (p + 1) * slice; /* remainder on the last slice */
    uint32_t n = r1 - r0;
    for (uint32_t i = 0; i < n; i++)
      buf[i].comp = ((uint64_t)keys[r0 + i] << 32) | (uint64_t)(r0 + i);
    qsort(buf, n, sizeof(comp_t), cmp_comp_desc);
    uint32_t take = n < ntop ? n : ntop;
    for (uint32_t i = 0; i < take; i++) cand[outn++] = (uint32_t)(buf[i].comp & 0xFFFFFFFFu);
  }
  free(buf);
  return outn;
}

void orc_gold_topk2(const uint32_t* coo_row, const uint32_t* coo_col, const int32_t* coo_val,
                    uint64_t nnz, const int32_t* vec, int k, uint32_t* res_idx, int32_t* res_val) {
  /* gold_algorithms.hpp:249-308 */
  for (int i = 0; i < k; i++) { res_idx[i] = 0; res_val[i] = 0; }
  if (nnz == 0) return;
  uint32_t curr_row = coo_row[0];
  int32_t curr_out = 0;
  int curr_worst_idx = 0;
  int32_t curr_worst_val = 0;
  for (uint64_t i = 0; i < nnz; i++) {
    uint32_t r = coo_row[i];
    int32_t p = coo_val[i] * vec[coo_col[i]];
    if (r == curr_row) {
      curr_out += p;
    } else {
      if (curr_out >= curr_worst_val) {
        res_idx[curr_worst_idx] = curr_row;
        res_val[curr_worst_idx] = curr_out;
        int wi = 0;
        int32_t wv = res_val[0];
        for (int j = 0; j < k; j++) {
          if (res_val[j] < wv) { wi = j; wv = res_val[j]; }
        }
        curr_worst_idx = wi;
        curr_worst_val = wv;
      }
      curr_row = r;
      curr_out = p;
    }
  }
  if (curr_out >= curr_worst_val) {
    res_idx[curr_worst_idx] = curr_row;
    res_val[curr_worst_idx] = curr_out;
  }
}

void orc_gold_topk_f32(const uint32_t* coo_row, const uint32_t* coo_col, const float* coo_val,
                       uint64_t nnz, const float* vec, int k, uint32_t* res_idx, float* res_val) {
  /* gold_algorithms.hpp:189-247 */
  for (int i = 0; i < k; i++) { res_idx[i] = 0; res_val[i] = 0.0f; }
  if (nnz == 0) return;
  uint32_t curr_row = coo_row[0];
  float curr_out = 0.0f;
  int curr_worst_idx = 0;
  float curr_worst_val = 0.0f;
  for (uint64_t i = 0; i < nnz; i++) {
    uint32_t r = coo_row[i];
    float p = coo_val[i] * vec[coo_col[i]];
    if (r == curr_row) {
      curr_out += p;
    } else {
      if (curr_out >= curr_worst_val) {
        res_idx[curr_worst_idx] = curr_row;
        res_val[curr_worst_idx] = curr_out;
        int wi = 0;
        float wv = res_val[0];
        for (int j = 0; j < k; j++) {
          if (res_val[j] < wv) { wi = j; wv = res_val[j]; }
        }
        curr_worst_idx = wi;
        curr_worst_val = wv;
      }
      curr_row = r;
      curr_out = p;
    }
  }
  if (curr_out >= curr_worst_val) {
    res_idx[curr_worst_idx] = curr_row;
    res_val[curr_worst_idx] = curr_out;
  }
}

/* ---------------------------------------------------------------------------------------- */
/* exact pass and final order                                                                */
/* ---------------------------------------------------------------------------------------- */

void orc_rescore_f32(const uint64_t* ptr, const uint32_t* col, const float* val, const float* q,
                     const uint32_t* rows, uint32_t n, float* out) {
  for (uint32_t i = 0; i < n; i++) {
    uint32_t r = rows[i];
    float acc = 0.0f;
    for (uint64_t e = ptr[r]; e < ptr[r + 1]; e++) {
      float p = val[e] * q[col[e]];
      acc = acc + p;
    }
    out[i] = acc;
  }
}

void orc_scores_f64(const uint64_t* ptr, const uint32_t* col, const float* val, const float* q,
                    uint32_t rows, double* out) {
  for (uint32_t r = 0; r < rows; r++) {
    double acc = 0.0;
    for (uint64_t e = ptr[r]; e < ptr[r + 1]; e++) acc += (double)val[e] * (double)q[col[e]];
    out[r] = acc;
  }
}

typedef struct {
  uint32_t idx;
  float v;
} tf_t;
typedef struct {
  uint32_t idx;
  int32_t v;
} ti_t;

static int cmp_tf(const void* a, const void* b) {
  const tf_t* x = (const tf_t*)a;
  const tf_t* y = (const tf_t*)b;
  if (x->v != y->v) return (x->v > y->v) ? -1 : 1;
  return (x->idx > y->idx) ? -1 : (x->idx < y->idx) ? 1 : 0;
}
static int cmp_ti(const void* a, const void* b) {
  const ti_t* x = (const ti_t*)a;
  const ti_t* y = (const ti_t*)b;
  if (x->v != y->v) return (x->v > y->v) ? -1 : 1;
  return (x->idx > y->idx) ? -1 : (x->idx < y->idx) ? 1 : 0;
}

void orc_sort_tuples_f32(uint32_t n, uint32_t* idx, float* val) {
  tf_t* t = (tf_t*)malloc(sizeof(tf_t) * (n ? n : 1));
  for (uint32_t i = 0; i < n; i++) { t[i].idx = idx[i]; t[i].v = val[i]; }
  qsort(t, n, sizeof(tf_t), cmp_tf);
  for (uint32_t i = 0; i < n; i++) { idx[i] = t[i].idx; val[i] = t[i].v; }
  free(t);
}

void orc_sort_tuples_i32(uint32_t n, uint32_t* idx, int32_t* val) {
  ti_t* t = (ti_t*)malloc(sizeof(ti_t) * (n ? n : 1));
  for (uint32_t i = 0; i < n; i++) { t[i].idx = idx[i]; t[i].v = val[i]; }
  qsort(t, n, sizeof(ti_t), cmp_ti);
  for (uint32_t i = 0; i < n; i++) { idx[i] = t[i].idx; val[i] = t[i].v; }
  free(t);
}

uint32_t orc_two_stage(const uint64_t* ptr, const uint32_t* col, const float* val,
                       const uint64_t* qptr, const uint32_t* qcol, const int32_t* qval,
                       const float* rowscale, uint32_t rows, uint32_t cols, int bits, int quant,
                       int qq, uint32_t split, uint32_t ck, uint32_t k, const float* query,
                       uint32_t* out_idx, float* out_score, uint32_t* cand, uint32_t* cand_n) {
  int32_t* q = (int32_t*)malloc(sizeof(int32_t) * (cols ? cols : 1));
  int32_t* s = (int32_t*)malloc(sizeof(int32_t) * (rows ? rows : 1));
  uint32_t* keys = (uint32_t*)malloc(sizeof(uint32_t) * (rows ? rows : 1));
  if (orc_quantize_query(query, cols, bits, quant, qq, q) != 0) {
    free(q); free(s); free(keys);
    *cand_n = 0;
    return 0;
  }
  orc_int_scores(qptr, qcol, qval, rows, q, s);
  orc_cand_keys(s, quant == ORC_QUANT_UNSIGNED_ROW ? rowscale : NULL, rows, keys);
  uint32_t nc = orc_select_split(keys, rows, split, ck, cand);
  *cand_n = nc;
  float* sc = (float*)malloc(sizeof(float) * (nc ? nc : 1));
  uint32_t* ix = (uint32_t*)malloc(sizeof(uint32_t) * (nc ? nc : 1));
  memcpy(ix, cand, sizeof(uint32_t) * nc);
  orc_rescore_f32(ptr, col, val, query, ix, nc, sc);
  /* final order: sort_tuples on (row, fp32 score); -0 canonicalised like the device key */
  for (uint32_t i = 0; i < nc; i++)
    if (sc[i] == 0.0f) sc[i] = 0.0f;
  orc_sort_tuples_f32(nc, ix, sc);
  uint32_t nout = nc < k ? nc : k;
  for (uint32_t i = 0; i < nout; i++) { out_idx[i] = ix[i]; out_score[i] = sc[i]; }
  free(q); free(s); free(keys); free(sc); free(ix);
  return nout;
}

/* ---------------------------------------------------------------------------------------- */
/* CPU timing harness (the reference two-stage method on host threads)                       */
/* ---------------------------------------------------------------------------------------- */
#include <pthread.h>
#include <time.h>

typedef struct {
  const uint64_t* qptr;
  const uint32_t* qcol;
  const int32_t* qval;
  const int32_t* q;
  uint32_t r0, r1;
  int k;
  uint32_t* idx;
  int32_t* val;
} orc_job_t;

/* streaming Top-k of gold_algorithms.hpp:249-308 over the rows [r0, r1) of a quantised CSR */
static void* orc_job_run(void* arg) {
  orc_job_t* j = (orc_job_t*)arg;
  for (int i = 0; i < j->k; i++) { j->idx[i] = 0; j->val[i] = 0; }
  int wi = 0;
  int32_t wv = 0;
  for (uint32_t r = j->r0; r < j->r1; r++) {
    int32_t s = 0;
    for (uint64_t e = j->qptr[r]; e < j->qptr[r + 1]; e++) s += j->qval[e] * j->q[j->qcol[e]];
    if (s >= wv) {
      j->idx[wi] = r;
      j->val[wi] = s;
      int bi = 0;
      int32_t bv = j->val[0];
      for (int t = 0; t < j->k; t++)
        if (j->val[t] < bv) { bi = t; bv = j->val[t]; }
      wi = bi;
      wv = bv;
    }
  }
  return NULL;
}

static double orc_now(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

double orc_bench_two_stage(const uint64_t* ptr, const uint32_t* col, const float* val,
                           const uint64_t* qptr, const uint32_t* qcol, const int32_t* qval,
                           uint32_t rows, uint32_t cols, int bits, uint32_t ck, uint32_t k,
                           const float* queries, uint32_t nq, int nthreads, double max_seconds,
                           uint32_t* done, uint32_t* out_idx) {
  if (nthreads < 1) nthreads = 1;
  int32_t* q = (int32_t*)malloc(sizeof(int32_t) * cols);
  orc_job_t* jobs = (orc_job_t*)malloc(sizeof(orc_job_t) * nthreads);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
  uint32_t* cidx = (uint32_t*)malloc(sizeof(uint32_t) * ck * nthreads);
  int32_t* cval = (int32_t*)malloc(sizeof(int32_t) * ck * nthreads);
  comp_t* cc = (comp_t*)malloc(sizeof(comp_t) * ck * nthreads);
  uint32_t* sel = (uint32_t*)malloc(sizeof(uint32_t) * ck);
  float* sc = (float*)malloc(sizeof(float) * ck);
  double t0 = orc_now();
  uint32_t n = 0;
  for (; n < nq; n++) {
    if (n > 0 && orc_now() - t0 > max_seconds) break;
    const float* x = queries + (size_t)n * cols;
    orc_quantize_query(x, cols, bits, ORC_QUANT_SYM_GLOBAL, ORC_QQ_NUMPY, q);
    for (int t = 0; t < nthreads; t++) {
      jobs[t].qptr = qptr; jobs[t].qcol = qcol; jobs[t].qval = qval; jobs[t].q = q;
      jobs[t].r0 = (uint32_t)((uint64_t)rows * t / nthreads);
      jobs[t].r1 = (uint32_t)((uint64_t)rows * (t + 1) / nthreads);
      jobs[t].k = (int)ck;
      jobs[t].idx = cidx + (size_t)t * ck;
      jobs[t].val = cval + (size_t)t * ck;
      if (nthreads == 1) orc_job_run(&jobs[t]);
      else pthread_create(&th[t], NULL, orc_job_run, &jobs[t]);
    }
    if (nthreads > 1)
      for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    uint32_t m = ck * (uint32_t)nthreads;
    for (uint32_t i = 0; i < m; i++)
      cc[i].comp = ((uint64_t)orc_key_i32(cval[i]) << 32) | cidx[i];
    qsort(cc, m, sizeof(comp_t), cmp_comp_desc);
    uint32_t nsel = m < ck ? m : ck;
    for (uint32_t i = 0; i < nsel; i++) sel[i] = (uint32_t)(cc[i].comp & 0xFFFFFFFFu);
    orc_rescore_f32(ptr, col, val, x, sel, nsel, sc);
    orc_sort_tuples_f32(nsel, sel, sc);
    if (out_idx)
      for (uint32_t i = 0; i < k && i < nsel; i++) out_idx[(size_t)n * k + i] = sel[i];
  }
  double el = orc_now() - t0;
  *done = n;
  free(q); free(jobs); free(th); free(cidx); free(cval); free(cc); free(sel); free(sc);
  return el;
}

typedef struct {
  const uint64_t* ptr;
  const uint32_t* col;
  const float* val;
  const float* q;
  uint32_t r0, r1;
  int k;
  uint32_t* idx;
  float* out;
} orc_fjob_t;

/* streaming FP32 Top-k of gold_algorithms.hpp:189-247 over the rows [r0, r1) of a CSR (the
 * reference walks a row-sorted COO; the rows and their entry order are the same) */
static void* orc_fjob_run(void* arg) {
  orc_fjob_t* j = (orc_fjob_t*)arg;
  for (int i = 0; i < j->k; i++) { j->idx[i] = 0; j->out[i] = 0.0f; }
  int wi = 0;
  float wv = 0.0f;
  for (uint32_t r = j->r0; r < j->r1; r++) {
    float s = 0.0f;
    for (uint64_t e = j->ptr[r]; e < j->ptr[r + 1]; e++) s = s + j->val[e] * j->q[j->col[e]];
    if (s >= wv) {
      j->idx[wi] = r;
      j->out[wi] = s;
      int bi = 0;
      float bv = j->out[0];
      for (int t = 0; t < j->k; t++)
        if (j->out[t] < bv) { bi = t; bv = j->out[t]; }
      wi = bi;
      wv = bv;
    }
  }
  return NULL;
}

double orc_bench_fp32_topk(const uint64_t* ptr, const uint32_t* col, const float* val,
                           uint32_t rows, uint32_t cols, uint32_t k, const float* queries,
                           uint32_t nq, int nthreads, double max_seconds, uint32_t* done) {
  if (nthreads < 1) nthreads = 1;
  orc_fjob_t* jobs = (orc_fjob_t*)malloc(sizeof(orc_fjob_t) * nthreads);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
  uint32_t* cidx = (uint32_t*)malloc(sizeof(uint32_t) * k * nthreads);
  float* cval = (float*)malloc(sizeof(float) * k * nthreads);
  comp_t* cc = (comp_t*)malloc(sizeof(comp_t) * k * nthreads);
  double t0 = orc_now();
  uint32_t n = 0;
  for (; n < nq; n++) {
    if (n > 0 && orc_now() - t0 > max_seconds) break;
    const float* x = queries + (size_t)n * cols;
    for (int t = 0; t < nthreads; t++) {
      jobs[t].ptr = ptr; jobs[t].col = col; jobs[t].val = val; jobs[t].q = x;
      jobs[t].r0 = (uint32_t)((uint64_t)rows * t / nthreads);
      jobs[t].r1 = (uint32_t)((uint64_t)rows * (t + 1) / nthreads);
      jobs[t].k = (int)k;
      jobs[t].idx = cidx + (size_t)t * k;
      jobs[t].out = cval + (size_t)t * k;
      if (nthreads == 1) orc_fjob_run(&jobs[t]);
      else pthread_create(&th[t], NULL, orc_fjob_run, &jobs[t]);
    }
    if (nthreads > 1)
      for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    uint32_t m = k * (uint32_t)nthreads;
    for (uint32_t i = 0; i < m; i++)
      cc[i].comp = ((uint64_t)orc_key_f32(cval[i]) << 32) | cidx[i];
    qsort(cc, m, sizeof(comp_t), cmp_comp_desc);  /* the blocks' Top-k merged */
  }
  double el = orc_now() - t0;
  *done = n;
  free(jobs); free(th); free(cidx); free(cval); free(cc);
  return el;
}

/* ---------------------------------------------------------------------------------------- */
/* ReSparse (quantify_util.py:375-403)                                                        */
/* ---------------------------------------------------------------------------------------- */

uint64_t orc_resparse(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t rows,
                      uint32_t cols, double keep, uint64_t* out_ptr, uint32_t* out_col,
                      float* out_val) {
  double sum = 0.0;
  for (uint64_t e = 0; e < ptr[rows]; e++) sum += fabs((double)val[e]);
  const double avg = sum / ((double)rows * (double)cols);  /* np.mean(np.abs(spm)) */
  uint64_t o = 0;
  out_ptr[0] = 0;
  for (uint32_t r = 0; r < rows; r++) {
    uint64_t n = 0;
    double mn = INFINITY;
    for (uint64_t e = ptr[r]; e < ptr[r + 1]; e++) {
      if (val[e] == 0.0f) continue;
      n++;
      if (fabs((double)val[e]) < mn) mn = fabs((double)val[e]);
    }
    if (n > 0 && mn > avg) {
      for (uint64_t e = ptr[r]; e < ptr[r + 1]; e++) {
        if (val[e] == 0.0f) continue;
        out_col[o] = col[e];
        out_val[o] = val[e];
        o++;
      }
    } else if (n > 0) {
      uint64_t k = (uint64_t)ceil((double)n * keep);
      if (k > n) k = n;
      /* mark the k largest |v| one at a time; among equal |v| the higher column wins */
      unsigned char* take = (unsigned char*)calloc(ptr[r + 1] - ptr[r], 1);
      for (uint64_t t = 0; t < k; t++) {
        uint64_t best = UINT64_MAX;
        for (uint64_t e = ptr[r]; e < ptr[r + 1]; e++) {
          if (val[e] == 0.0f || take[e - ptr[r]]) continue;
          if (best == UINT64_MAX) { best = e; continue; }
          const float a = fabsf(val[e]), b = fabsf(val[best]);
          if (a > b || (a == b && col[e] > col[best])) best = e;
        }
        take[best - ptr[r]] = 1;
      }
      for (uint64_t e = ptr[r]; e < ptr[r + 1]; e++) {
        if (!take[e - ptr[r]]) continue;
        out_col[o] = col[e];
        out_val[o] = val[e];
        o++;
      }
      free(take);
    }
    out_ptr[r + 1] = o;
  }
  return o;
}

/* ---------------------------------------------------------------------------------------- */
/* Seeded synthetic matrices: the same generator as the engine's aes_gen_matrix (it defines   */
/* the benchmark workloads; the reference ships no matrices).  Restated here so that the CPU  */
/* baseline builds its inputs without loading the engine library.                             */
/* ---------------------------------------------------------------------------------------- */

typedef struct { uint64_t s[4]; } orc_xo_t;

static void orc_xo_seed(orc_xo_t* g, uint64_t seed) {
  uint64_t x = seed;
  for (int i = 0; i < 4; i++) {
    x += 0x9E3779B97F4A7C15ull;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    g->s[i] = z ^ (z >> 31);
  }
}
static inline uint64_t orc_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static uint64_t orc_xo_next(orc_xo_t* g) {
  uint64_t* s = g->s;
  uint64_t r = orc_rotl(s[1] * 5, 7) * 9;
  uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = orc_rotl(s[3], 45);
  return r;
}
static double orc_xo_uniform(orc_xo_t* g) { return (double)(orc_xo_next(g) >> 11) * (1.0 / 9007199254740992.0); }
static uint32_t orc_xo_below(orc_xo_t* g, uint32_t n) {
  return (uint32_t)(((orc_xo_next(g) >> 32) * (uint64_t)n) >> 32);
}
static uint64_t orc_row_seed(uint64_t seed, uint64_t row, uint64_t stream) {
  uint64_t z = seed * 0xD1B54A32D192ED03ull + row * 0x9E3779B97F4A7C15ull + stream * 0xA0761D6478BD642Full;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static uint32_t orc_gen_degree(uint32_t kind, uint32_t cols, double p0, double p1, orc_xo_t* g) {
  uint32_t d = 0;
  switch (kind) {
    case ORC_GEN_UNIFORM_DEG: {
      uint32_t lo = (uint32_t)p0, hi = (uint32_t)p1;
      d = lo + orc_xo_below(g, hi - lo + 1);
      break;
    }
    case ORC_GEN_FIXED_ABSNORMAL:
    case ORC_GEN_FIXED_UNIFORM:
      d = (uint32_t)p0;
      break;
    case ORC_GEN_GAMMA_DEG: {
      double u1 = 1.0 - orc_xo_uniform(g), u2 = 1.0 - orc_xo_uniform(g);
      double x = -(p0 / 2.0) * log(u1 * u2);
      double r = nearbyint(x);
      if (r < 1.0) r = 1.0;
      if (r > p1) r = p1;
      d = (uint32_t)r;
      break;
    }
  }
  return d < cols ? d : cols;
}

typedef struct {
  uint32_t kind, cols, r0, r1;
  double p0, p1;
  uint64_t seed;
  const uint64_t* ptr;
  uint32_t* col;
  float* val;
  uint32_t* deg;
} orc_genjob_t;

static void* orc_gen_deg_run(void* arg) {
  orc_genjob_t* j = (orc_genjob_t*)arg;
  for (uint32_t r = j->r0; r < j->r1; r++) {
    orc_xo_t g;
    orc_xo_seed(&g, orc_row_seed(j->seed, r, 0));
    j->deg[r] = orc_gen_degree(j->kind, j->cols, j->p0, j->p1, &g);
  }
  return NULL;
}

static void* orc_gen_row_run(void* arg) {
  orc_genjob_t* j = (orc_genjob_t*)arg;
  const uint32_t cols = j->cols, nw = (cols + 63) / 64;
  uint64_t* bm = (uint64_t*)malloc(sizeof(uint64_t) * nw);
  for (uint32_t r = j->r0; r < j->r1; r++) {
    orc_xo_t g;
    orc_xo_seed(&g, orc_row_seed(j->seed, r, 1));
    const uint32_t d = (uint32_t)(j->ptr[r + 1] - j->ptr[r]);
    memset(bm, 0, sizeof(uint64_t) * nw);
    if (d * 2 <= cols) {
      uint32_t got = 0;
      while (got < d) {
        uint32_t c = orc_xo_below(&g, cols);
        uint64_t bit = 1ull << (c & 63);
        if (!(bm[c >> 6] & bit)) { bm[c >> 6] |= bit; got++; }
      }
    } else { /* dense rows: the columns to leave out are drawn */
      for (uint32_t w = 0; w < nw; w++) bm[w] = ~0ull;
      if (cols & 63) bm[nw - 1] = (1ull << (cols & 63)) - 1;
      uint32_t drop = cols - d, got = 0;
      while (got < drop) {
        uint32_t c = orc_xo_below(&g, cols);
        uint64_t bit = 1ull << (c & 63);
        if (bm[c >> 6] & bit) { bm[c >> 6] &= ~bit; got++; }
      }
    }
    uint64_t o = j->ptr[r];
    for (uint32_t w = 0; w < nw; w++) {
      uint64_t x = bm[w];
      while (x) {
        int b = __builtin_ctzll(x);
        x &= x - 1;
        j->col[o++] = w * 64 + (uint32_t)b;
      }
    }
    for (uint64_t k = j->ptr[r]; k < o; k++) {
      float v;
      if (j->kind == ORC_GEN_FIXED_ABSNORMAL) {
        double u1 = 1.0 - orc_xo_uniform(&g), u2 = orc_xo_uniform(&g);
        v = (float)fabs(sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
      } else {
        v = (float)orc_xo_uniform(&g);
      }
      j->val[k] = v;
    }
  }
  free(bm);
  return NULL;
}

static void orc_gen_pass(orc_genjob_t* base, uint32_t rows, int nthreads, void* (*fn)(void*)) {
  if (nthreads < 1) nthreads = 1;
  orc_genjob_t* jobs = (orc_genjob_t*)malloc(sizeof(orc_genjob_t) * nthreads);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
  for (int t = 0; t < nthreads; t++) {
    jobs[t] = *base;
    jobs[t].r0 = (uint32_t)((uint64_t)rows * t / nthreads);
    jobs[t].r1 = (uint32_t)((uint64_t)rows * (t + 1) / nthreads);
    if (nthreads == 1) fn(&jobs[t]);
    else pthread_create(&th[t], NULL, fn, &jobs[t]);
  }
  if (nthreads > 1)
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  free(jobs);
  free(th);
}

uint64_t orc_gen_matrix(uint32_t kind, uint32_t rows, uint32_t cols, double p0, double p1,
                        uint64_t seed, int nthreads, uint64_t* ptr, uint32_t* col, float* val) {
  if (kind > ORC_GEN_FIXED_UNIFORM || cols == 0 || rows == 0) return UINT64_MAX;
  if (kind == ORC_GEN_UNIFORM_DEG && (p1 < p0 || p0 < 0)) return UINT64_MAX;
  uint32_t* deg = (uint32_t*)malloc(sizeof(uint32_t) * rows);
  orc_genjob_t base;
  memset(&base, 0, sizeof(base));
  base.kind = kind; base.cols = cols; base.p0 = p0; base.p1 = p1; base.seed = seed;
  base.deg = deg;
  orc_gen_pass(&base, rows, nthreads, orc_gen_deg_run);
  uint64_t total = 0;
  for (uint32_t r = 0; r < rows; r++) total += deg[r];
  if (!ptr) { free(deg); return total; }
  ptr[0] = 0;
  for (uint32_t r = 0; r < rows; r++) ptr[r + 1] = ptr[r] + deg[r];
  free(deg);
  base.ptr = ptr; base.col = col; base.val = val;
  orc_gen_pass(&base, rows, nthreads, orc_gen_row_run);
  return total;
}

/* ---------------------------------------------------------------------------------------- */
/* Checks at full size, threaded                                                             */
/* ---------------------------------------------------------------------------------------- */

typedef struct {
  const uint64_t *ptr, *qptr;
  const uint32_t *col, *qcol;
  const float *val, *rowscale, *queries;
  const int32_t* qval;
  uint32_t rows, cols, split, ck, k, q0, q1;
  int bits, quant, qq;
  uint32_t *out_idx, *out_n;
  float* out_score;
} orc_tsjob_t;

static void* orc_ts_run(void* arg) {
  orc_tsjob_t* j = (orc_tsjob_t*)arg;
  uint32_t* cand = (uint32_t*)malloc(sizeof(uint32_t) * (j->ck ? j->ck : 1));
  for (uint32_t q = j->q0; q < j->q1; q++) {
    uint32_t cn = 0;
    j->out_n[q] = orc_two_stage(j->ptr, j->col, j->val, j->qptr, j->qcol, j->qval, j->rowscale,
                                j->rows, j->cols, j->bits, j->quant, j->qq, j->split, j->ck, j->k,
                                j->queries + (size_t)q * j->cols, j->out_idx + (size_t)q * j->k,
                                j->out_score + (size_t)q * j->k, cand, &cn);
  }
  free(cand);
  return NULL;
}

void orc_two_stage_many(const uint64_t* ptr, const uint32_t* col, const float* val,
                        const uint64_t* qptr, const uint32_t* qcol, const int32_t* qval,
                        const float* rowscale, uint32_t rows, uint32_t cols, int bits, int quant,
                        int qq, uint32_t split, uint32_t ck, uint32_t k, const float* queries,
                        uint32_t nq, int nthreads, uint32_t* out_idx, float* out_score,
                        uint32_t* out_n) {
  if (nthreads < 1) nthreads = 1;
  if ((uint32_t)nthreads > nq) nthreads = nq ? (int)nq : 1;
  orc_tsjob_t* jobs = (orc_tsjob_t*)malloc(sizeof(orc_tsjob_t) * nthreads);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
  for (int t = 0; t < nthreads; t++) {
    orc_tsjob_t* j = &jobs[t];
    j->ptr = ptr; j->col = col; j->val = val; j->qptr = qptr; j->qcol = qcol; j->qval = qval;
    j->rowscale = rowscale; j->queries = queries; j->rows = rows; j->cols = cols;
    j->split = split; j->ck = ck; j->k = k; j->bits = bits; j->quant = quant; j->qq = qq;
    j->q0 = (uint32_t)((uint64_t)nq * t / nthreads);
    j->q1 = (uint32_t)((uint64_t)nq * (t + 1) / nthreads);
    j->out_idx = out_idx; j->out_score = out_score; j->out_n = out_n;
    if (nthreads == 1) orc_ts_run(j);
    else pthread_create(&th[t], NULL, orc_ts_run, j);
  }
  if (nthreads > 1)
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  free(jobs);
  free(th);
}

/* float64 Top-k of one query: a size-k min-heap on (score, -row), i.e. the k best by score
 * descending with the lower row first among equal scores (numpy's stable argsort of -score). */
typedef struct { double s; uint32_t r; } orc_sd_t;
static int orc_sd_worse(orc_sd_t a, orc_sd_t b) { /* a ranks below b */
  return a.s < b.s || (a.s == b.s && a.r > b.r);
}
static void orc_heap_down(orc_sd_t* h, uint32_t n, uint32_t i) {
  for (;;) {
    uint32_t l = 2 * i + 1, r = l + 1, m = i;
    if (l < n && orc_sd_worse(h[l], h[m])) m = l;
    if (r < n && orc_sd_worse(h[r], h[m])) m = r;
    if (m == i) return;
    orc_sd_t t = h[i]; h[i] = h[m]; h[m] = t;
    i = m;
  }
}
static int orc_sd_cmp_desc(const void* a, const void* b) {
  orc_sd_t x = *(const orc_sd_t*)a, y = *(const orc_sd_t*)b;
  if (orc_sd_worse(x, y)) return 1;
  if (orc_sd_worse(y, x)) return -1;
  return 0;
}

typedef struct {
  const uint64_t* ptr;
  const uint32_t* col;
  const float *val, *queries;
  uint32_t rows, cols, k, q0, q1;
  uint32_t* out_idx;
  double* out_score;
} orc_f64job_t;

static void* orc_f64_run(void* arg) {
  orc_f64job_t* j = (orc_f64job_t*)arg;
  orc_sd_t* h = (orc_sd_t*)malloc(sizeof(orc_sd_t) * (j->k ? j->k : 1));
  for (uint32_t q = j->q0; q < j->q1; q++) {
    const float* x = j->queries + (size_t)q * j->cols;
    uint32_t n = 0;
    for (uint32_t r = 0; r < j->rows; r++) {
      double s = 0.0;
      for (uint64_t e = j->ptr[r]; e < j->ptr[r + 1]; e++) s += (double)j->val[e] * (double)x[j->col[e]];
      orc_sd_t c = {s, r};
      if (n < j->k) {
        h[n++] = c;
        if (n == j->k)
          for (int32_t i = (int32_t)n / 2 - 1; i >= 0; i--) orc_heap_down(h, n, (uint32_t)i);
      } else if (orc_sd_worse(h[0], c)) {
        h[0] = c;
        orc_heap_down(h, n, 0);
      }
    }
    qsort(h, n, sizeof(orc_sd_t), orc_sd_cmp_desc);
    for (uint32_t i = 0; i < j->k; i++) {
      j->out_idx[(size_t)q * j->k + i] = i < n ? h[i].r : 0xFFFFFFFFu;
      j->out_score[(size_t)q * j->k + i] = i < n ? h[i].s : -INFINITY;
    }
  }
  free(h);
  return NULL;
}

void orc_topk_f64_many(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t rows,
                       uint32_t cols, const float* queries, uint32_t nq, uint32_t k, int nthreads,
                       uint32_t* out_idx, double* out_score) {
  if (nthreads < 1) nthreads = 1;
  if ((uint32_t)nthreads > nq) nthreads = nq ? (int)nq : 1;
  orc_f64job_t* jobs = (orc_f64job_t*)malloc(sizeof(orc_f64job_t) * nthreads);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
  for (int t = 0; t < nthreads; t++) {
    orc_f64job_t* j = &jobs[t];
    j->ptr = ptr; j->col = col; j->val = val; j->queries = queries;
    j->rows = rows; j->cols = cols; j->k = k;
    j->q0 = (uint32_t)((uint64_t)nq * t / nthreads);
    j->q1 = (uint32_t)((uint64_t)nq * (t + 1) / nthreads);
    j->out_idx = out_idx; j->out_score = out_score;
    if (nthreads == 1) orc_f64_run(j);
    else pthread_create(&th[t], NULL, orc_f64_run, j);
  }
  if (nthreads > 1)
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  free(jobs);
  free(th);
}

/* FP32 exact Top-k of every row (spmv_coo_gold_top_k's arithmetic, gold_algorithms.hpp:211-239:
 * acc = acc + val * q[col] in column order, separately rounded), ordered as sort_tuples orders
 * (score descending, row descending; evaluation_utils.hpp:40-62). */
typedef struct { float s; uint32_t r; } orc_sf_t;
static int orc_sf_worse(orc_sf_t a, orc_sf_t b) { return a.s < b.s || (a.s == b.s && a.r < b.r); }
static void orc_heapf_down(orc_sf_t* h, uint32_t n, uint32_t i) {
  for (;;) {
    uint32_t l = 2 * i + 1, r = l + 1, m = i;
    if (l < n && orc_sf_worse(h[l], h[m])) m = l;
    if (r < n && orc_sf_worse(h[r], h[m])) m = r;
    if (m == i) return;
    orc_sf_t t = h[i]; h[i] = h[m]; h[m] = t;
    i = m;
  }
}
static int orc_sf_cmp_desc(const void* a, const void* b) {
  orc_sf_t x = *(const orc_sf_t*)a, y = *(const orc_sf_t*)b;
  if (orc_sf_worse(x, y)) return 1;
  if (orc_sf_worse(y, x)) return -1;
  return 0;
}

typedef struct {
  const uint64_t* ptr;
  const uint32_t* col;
  const float *val, *queries;
  uint32_t rows, cols, k, q0, q1;
  uint32_t* out_idx;
  float* out_score;
} orc_f32job_t;

static void* orc_f32_run(void* arg) {
  orc_f32job_t* j = (orc_f32job_t*)arg;
  orc_sf_t* h = (orc_sf_t*)malloc(sizeof(orc_sf_t) * (j->k ? j->k : 1));
  for (uint32_t q = j->q0; q < j->q1; q++) {
    const float* x = j->queries + (size_t)q * j->cols;
    uint32_t n = 0;
    for (uint32_t r = 0; r < j->rows; r++) {
      float s = 0.0f;
      for (uint64_t e = j->ptr[r]; e < j->ptr[r + 1]; e++) s = s + j->val[e] * x[j->col[e]];
      if (s == 0.0f) s = 0.0f;
      orc_sf_t c = {s, r};
      if (n < j->k) {
        h[n++] = c;
        if (n == j->k)
          for (int32_t i = (int32_t)n / 2 - 1; i >= 0; i--) orc_heapf_down(h, n, (uint32_t)i);
      } else if (orc_sf_worse(h[0], c)) {
        h[0] = c;
        orc_heapf_down(h, n, 0);
      }
    }
    qsort(h, n, sizeof(orc_sf_t), orc_sf_cmp_desc);
    for (uint32_t i = 0; i < j->k; i++) {
      j->out_idx[(size_t)q * j->k + i] = i < n ? h[i].r : 0xFFFFFFFFu;
      j->out_score[(size_t)q * j->k + i] = i < n ? h[i].s : -INFINITY;
    }
  }
  free(h);
  return NULL;
}

void orc_topk_f32_many(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t rows,
                       uint32_t cols, const float* queries, uint32_t nq, uint32_t k, int nthreads,
                       uint32_t* out_idx, float* out_score) {
  if (nthreads < 1) nthreads = 1;
  if ((uint32_t)nthreads > nq) nthreads = nq ? (int)nq : 1;
  orc_f32job_t* jobs = (orc_f32job_t*)malloc(sizeof(orc_f32job_t) * nthreads);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
  for (int t = 0; t < nthreads; t++) {
    orc_f32job_t* j = &jobs[t];
    j->ptr = ptr; j->col = col; j->val = val; j->queries = queries;
    j->rows = rows; j->cols = cols; j->k = k;
    j->q0 = (uint32_t)((uint64_t)nq * t / nthreads);
    j->q1 = (uint32_t)((uint64_t)nq * (t + 1) / nthreads);
    j->out_idx = out_idx; j->out_score = out_score;
    if (nthreads == 1) orc_f32_run(j);
    else pthread_create(&th[t], NULL, orc_f32_run, j);
  }
  if (nthreads > 1)
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  free(jobs);
  free(th);
}

/* float64 score of the given (query, row) pairs: rows[q * k + i] of query q (0xFFFFFFFF: NaN). */
void orc_rows_f64(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t cols,
                  const float* queries, uint32_t nq, uint32_t k, const uint32_t* rows_sel,
                  double* out) {
  for (uint32_t q = 0; q < nq; q++) {
    const float* x = queries + (size_t)q * cols;
    for (uint32_t i = 0; i < k; i++) {
      const uint32_t r = rows_sel[(size_t)q * k + i];
      if (r == 0xFFFFFFFFu) { out[(size_t)q * k + i] = NAN; continue; }
      double s = 0.0;
      for (uint64_t e = ptr[r]; e < ptr[r + 1]; e++) s += (double)val[e] * (double)x[col[e]];
      out[(size_t)q * k + i] = s;
    }
  }
}
