// aes_tc.cuh -- candidate pass of 4-bit matrices on the tensor cores (tcgen05).
//
// The batched candidate pass of aes_batch.cuh scores 128 queries per matrix read with dp4a and is
// bound by instruction issue.  For B = 4 every matrix value (signed [-8, 7], unsigned [0, 15]) and
// every quantised query value is an integer of magnitude <= 16, which FP8 e4m3 holds exactly, and
// every partial sum of a row score stays far below 2^24 (15 * 15 * 1024), so an FP32 accumulation
// of the products is exact in any order.  The pass is then a dense product
//
//     D[128 rows x 128 queries] = A[128 rows x cols] * Q[128 queries x cols]^T
//
// per tile of 128 consecutive rows, with the row tile A densified in shared memory:
//   - the host lays out the quantised entries per (row tile, 256-column chunk) as 32-bit words
//     holding the entry's byte offset inside the chunk's operand layout and its e4m3 byte;
//   - the CTA scatters a chunk's entries into one of two zeroed 32 KB chunk buffers, one thread
//     issues the chunk's tcgen05.mma (kind::f8f6f4, M = 128, N = 128, K = 32 each) into a
//     128-column FP32 accumulator in tensor memory, and tcgen05.commit signals an mbarrier when
//     they have read the buffer; the entries are then written back to zero (the buffer is reused
//     two chunks later);
//   - after a tile's last chunk the accumulator (one of two) is read with tcgen05.ld while the
//     next tile's MMAs run: every (row, query) score becomes the same candidate key as in the
//     other passes and is compared with the query's threshold; hits are appended exactly as
//     the dp4a pass appends them.
// Both operands are K-major without swizzle (layout in aes_tc_layout.h).
// Reference counterpart: the candidate pass spmv_ucsr_top_k_multicore.hpp:195-413 (one query per
// pass on the FPGA); scores equal those of gold_algorithms.hpp:249-308 on the same integers.
#pragma once

#include "aes_kernels.cuh"
#include "aes_tc_layout.h"

namespace aes {
namespace dev {

constexpr int kTcThreads = 256;
constexpr uint32_t kTcTmemCols = 2 * kTcQ;  // two FP32 accumulators

__host__ inline size_t tc_smem_bytes(uint32_t cols, uint32_t split) {
  const uint32_t S = split <= 1 ? 1 : split;
  return tc_qtab_bytes(cols) + 2 * (size_t)kTcChunkBytes + (size_t)S * kTcQ * 4 + 64;
}

// e4m3 query operand of queries q0 .. q0 + nq - 1 (zero past nq and past cols)
__global__ void k_qtable_tc(const int8_t* __restrict__ q8, uint32_t ld8, uint32_t cols, uint32_t q0,
                            uint32_t nq, uint8_t* __restrict__ qt) {
  const uint32_t kp = tc_kpad(cols);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kTcQ * kp) return;
  const uint32_t n = i / kp, k = i % kp;
  const int v = (n < nq && k < cols) ? (int)q8[(size_t)(q0 + n) * ld8 + k] : 0;
  qt[tc_off(n, k)] = e4m3_small(v);
}

struct TcArgs {
  const uint32_t* ent;   // per entry: byte offset in its chunk operand | e4m3 value << 16
  const uint32_t* ptr;   // [n_rtiles * nch + 1] first entry of (row tile, chunk)
  uint32_t n_rtiles, nch, kpad, n_rows;
  const uint8_t* qt;     // e4m3 query operand of this launch, tc_qtab_bytes(cols)
  uint32_t q0, nq;       // this launch scores queries q0 .. q0 + nq - 1 (nq <= 128)
  const float* rowscale;
  uint32_t split, slice; // split >= 1
  const uint32_t* thr;   // [nq_total][split]
  uint32_t* cnt;         // [nq_total][split]
  uint2* surv;           // [nq_total][split][cap]
  uint32_t cap;
  uint32_t* status;      // [nq_total]
};

__device__ __forceinline__ uint32_t tc_smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
// shared-memory operand descriptor: start address, K-adjacent core matrices 2048 B apart
// (leading byte offset), 8-row groups 128 B apart (stride byte offset), descriptor version 1,
// no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(2048u >> 4) << 16) |
         ((uint64_t)(128u >> 4) << 32) | ((uint64_t)1 << 46);
}
// waits for the phase of the given parity to complete; gives up after about a second
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  uint32_t done = 0;
  while (!done) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done) : "r"(bar), "r"(parity) : "memory");
    if (!done && clock64() - t0 > (1ll << 31)) return false;
  }
  return true;
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t da, uint64_t db, uint32_t idesc,
                                       uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n"
      :: "r"(d), "l"(da), "l"(db), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               :: "r"(bar) : "memory");
}
// 32 consecutive accumulator columns of this warp's 32 lanes (one row per thread)
__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
        "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
        "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Reads accumulator `dbuf` of row tile T and appends every (row, query) key at or above the
// query's threshold.  Warp w holds rows 32 (w % 4) .. + 31 of the tile (its tensor-memory lane
// quarter) and queries 64 (w / 4) .. + 63.
__device__ __forceinline__ bool tc_epilogue(const TcArgs& a, uint32_t T, uint32_t tmem,
                                            uint32_t dbuf, uint32_t bar, uint32_t parity,
                                            const uint32_t* thr_s, uint32_t S) {
  const bool ok = tc_wait(bar, parity);
  tc_fence_after();
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  const uint32_t g = warp & 3u, h = warp >> 2;
  const uint32_t row = T * kTcRows + g * 32u + lane;
  const bool valid = row < a.n_rows;
  uint32_t p = 0;
  float rs = 0.0f;
  if (valid) {
    p = part_of(row, S, a.slice);
    if (a.rowscale) rs = __ldg(a.rowscale + row);
  }
  const float* thf = reinterpret_cast<const float*>(thr_s) + p * kTcQ;
#pragma unroll 1
  for (uint32_t cc = 0; cc < 2; cc++) {
    const uint32_t col0 = h * 64u + cc * 32u;
    uint32_t v[32];
    tc_ld32(tmem + dbuf * kTcQ + col0 + ((g * 32u) << 16), v);
    if (valid) {
#pragma unroll
      for (int j = 0; j < 32; j++) {
        const uint32_t q = col0 + j;
        const float f = __uint_as_float(v[j]);  // an exact integer score
        const float x = a.rowscale ? __fmul_rn(f, rs) : f;
        if (x >= thf[q] && q < a.nq) {
          const uint32_t key = a.rowscale ? key_f32(x) : key_i32(__float2int_rn(f));
          const size_t qp = (size_t)(a.q0 + q) * S + p;
          const uint32_t i = atomicAdd(a.cnt + qp, 1u);
          if (i < a.cap) a.surv[qp * a.cap + i] = make_uint2(key, row);
        }
      }
    }
  }
  tc_fence_before();
  return ok;
}

constexpr int kTcPer = 8;  // entries of a chunk a thread holds in registers (2048 per chunk)

// A thread's share of one chunk's entries: v[u] = entry b + tid + 256 u for tid + 256 u < n
struct TcEnt {
  uint32_t v[kTcPer];
  uint32_t b = 0, n = 0;
  __device__ __forceinline__ void load(const uint32_t* ent, uint32_t b_, uint32_t n_, uint32_t tid) {
    b = b_;
    n = n_;
#pragma unroll
    for (int u = 0; u < kTcPer; u++) {
      const uint32_t i = tid + (uint32_t)u * kTcThreads;
      v[u] = i < n ? __ldg(ent + b + i) : 0u;
    }
  }
  // writes the entries' e4m3 bytes (or zeros) into a chunk buffer
  __device__ __forceinline__ void stage(unsigned char* ab, const uint32_t* ent, uint32_t tid,
                                        bool clear) const {
#pragma unroll
    for (int u = 0; u < kTcPer; u++) {
      const uint32_t i = tid + (uint32_t)u * kTcThreads;
      if (i < n) ab[v[u] & 0xFFFFu] = clear ? (uint8_t)0 : (uint8_t)(v[u] >> 16);
    }
    for (uint32_t i = tid + kTcPer * kTcThreads; i < n; i += kTcThreads) {
      const uint32_t e = __ldg(ent + b + i);
      ab[e & 0xFFFFu] = clear ? (uint8_t)0 : (uint8_t)(e >> 16);
    }
  }
};

// One CTA per SM, persistent over row tiles T = blockIdx.x, + gridDim.x, ...
__global__ void __launch_bounds__(kTcThreads, 1) k_cand_tc(TcArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t qbytes = (a.kpad / 16u) * 2048u;
  unsigned char* sq = smem;                     // query operand
  unsigned char* sa = smem + qbytes;            // two chunk buffers of the row tile
  uint32_t* thr_s = reinterpret_cast<uint32_t*>(sa + 2 * kTcChunkBytes);
  const uint32_t S = a.split <= 1 ? 1u : a.split;
  uint64_t* bars = reinterpret_cast<uint64_t*>(thr_s + S * kTcQ);  // 2 chunk, 2 accumulator
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 4);
  const uint32_t tid = threadIdx.x, warp = tid >> 5;
  {
    const uint4* src = reinterpret_cast<const uint4*>(a.qt);
    uint4* dst = reinterpret_cast<uint4*>(sq);
    for (uint32_t i = tid; i < qbytes / 16u; i += blockDim.x) dst[i] = src[i];
    uint4* z = reinterpret_cast<uint4*>(sa);
    for (uint32_t i = tid; i < 2 * kTcChunkBytes / 16u; i += blockDim.x) z[i] = make_uint4(0, 0, 0, 0);
    // thresholds as FP32 bounds on the score (int keys) or on rowscale * score, so that the
    // comparison needs no conversion: key >= th  <=>  bound <= x for every x the pass produces
    for (uint32_t i = tid; i < S * kTcQ; i += blockDim.x) {
      const uint32_t p = i / kTcQ, q = i % kTcQ;
      const uint32_t th = q < a.nq ? a.thr[(size_t)(a.q0 + q) * S + p] : 0xFFFFFFFFu;
      float fb;
      if (a.rowscale) {  // x >= +0, key(x) = bits(x) | 2^31; NaN bits: never
        fb = th <= 0x80000000u ? -__int_as_float(0x7f800000) : __uint_as_float(th & 0x7FFFFFFFu);
      } else {           // |score| < 2^24, exact in FP32
        const int32_t b = (int32_t)(th ^ 0x80000000u);
        fb = b > (1 << 24) ? __int_as_float(0x7f800000)
                           : (b < -(1 << 24) ? -__int_as_float(0x7f800000) : __int2float_rn(b));
      }
      thr_s[i] = __float_as_uint(fb);
    }
  }
  if (tid == 0) {
    for (int b = 0; b < 4; b++)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(tc_smem_u32(bars + b)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(tc_smem_u32(tslot)), "n"(kTcTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  // instruction descriptor: FP32 accumulator, e4m3 x e4m3, both K-major, N = 128, M = 128
  const uint32_t idesc = (1u << 4) | ((kTcQ >> 3) << 17) | ((kTcRows >> 4) << 24);
  const uint32_t bar_chunk = tc_smem_u32(bars), bar_acc = tc_smem_u32(bars + 2);
  const uint32_t sq_addr = tc_smem_u32(sq), sa_addr = tc_smem_u32(sa);
  const uint32_t ep_chunk = a.nch > 1 ? 1u : 0u;  // the chunk after which the previous tile's
                                                  // accumulator is read
  // Entries move through registers: a thread holds entries tid + 256 u (u < kTcPer) of a chunk,
  // chunk i in ring set E[i % 4].  Step i clears chunk i - 2 from E[(i + 2) % 4], then loads
  // chunk i + 2 into it, and stages chunk i (loaded two steps earlier); the row offsets of a
  // chunk are read four steps before its entries.  The ring has static names (the step is
  // unrolled four times), so no register copy waits on a load in flight.  Chunks of more than
  // 256 kTcPer entries read the rest from global memory.
  const uint32_t ntl = a.n_rtiles > blockIdx.x ? (a.n_rtiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0u;
  const uint32_t total = ntl * a.nch;  // chunks of this CTA
  auto chunk_id = [&](uint32_t i) -> uint32_t {
    return i < total ? (blockIdx.x + (i / a.nch) * gridDim.x) * a.nch + i % a.nch : 0xFFFFFFFFu;
  };
  auto ptr_of = [&](uint32_t i, uint32_t& b, uint32_t& e) {
    const uint32_t j = chunk_id(i);
    b = j != 0xFFFFFFFFu ? __ldg(a.ptr + j) : 0u;
    e = j != 0xFFFFFFFFu ? __ldg(a.ptr + j + 1) : 0u;
  };
  TcEnt E0, E1, E2, E3;
  uint32_t P0b, P0e, P1b, P1e, P2b, P2e, P3b, P3e;  // row offsets of chunk i + 2 in P[(i + 2) % 4]
  {
    uint32_t b, e;
    ptr_of(0, b, e);
    E0.load(a.ent, b, e - b, tid);
    ptr_of(1, b, e);
    E1.load(a.ent, b, e - b, tid);
    ptr_of(2, P2b, P2e);
    ptr_of(3, P3b, P3e);
    ptr_of(4, P0b, P0e);
    ptr_of(5, P1b, P1e);
  }
  // ok: every bounded wait of this thread succeeded.  The CTA leaves the loop together (the
  // barrier's AND) at the first failure, so a stalled tensor pipe costs one wait, not one per chunk.
  bool ok = true, live = true;
  auto step = [&](uint32_t i, TcEnt& cur, TcEnt& old, uint32_t& pb, uint32_t& pe) {
    const uint32_t tl = i / a.nch, c = i % a.nch;
    const uint32_t buf = i & 1u;
    unsigned char* ab = sa + buf * kTcChunkBytes;
    if (i >= 2) {  // the MMAs of chunk i - 2 have read this buffer: clear its entries
      ok &= tc_wait(bar_chunk + 8u * buf, ((i - 2) >> 1) & 1u);
      old.stage(ab, a.ent, tid, true);
    }
    // every clear lands before any write of this chunk (they may share a byte)
    if (!__syncthreads_and(ok)) {
      live = false;
      return;
    }
    old.load(a.ent, pb, pe - pb, tid);  // chunk i + 2
    ptr_of(i + 6, pb, pe);
    cur.stage(ab, a.ent, tid, false);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint32_t nk = min(kTcChunkK, a.kpad - c * kTcChunkK) / 32u;
      const uint32_t d = tmem + (tl & 1u) * kTcQ;
      for (uint32_t kk = 0; kk < nk; kk++)
        tc_mma(d, tc_desc(sa_addr + buf * kTcChunkBytes + kk * 4096u),
               tc_desc(sq_addr + (c * 16u + 2u * kk) * 2048u), idesc, (c | kk) != 0);
      tc_commit(bar_chunk + 8u * buf);
      if (c == a.nch - 1) tc_commit(bar_acc + 8u * (tl & 1u));
    }
  };
  for (uint32_t i = 0; i < total; i++) {
    switch (i & 3u) {  // static ring names: four inlined copies of the step
      case 0: step(i, E0, E2, P2b, P2e); break;
      case 1: step(i, E1, E3, P3b, P3e); break;
      case 2: step(i, E2, E0, P0b, P0e); break;
      default: step(i, E3, E1, P1b, P1e); break;
    }
    if (!live) break;
    const uint32_t tl = i / a.nch;
    if (tl > 0 && i % a.nch == ep_chunk)  // the previous tile's accumulator
      ok &= tc_epilogue(a, blockIdx.x + (tl - 1) * gridDim.x, tmem, (tl - 1) & 1u,
                        bar_acc + 8u * ((tl - 1) & 1u), ((tl - 1) >> 1) & 1u, thr_s, S);
  }
  const uint32_t it = total;
  if (__syncthreads_and(ok && live) && ntl > 0) {
    const uint32_t tl = ntl - 1;
    ok &= tc_epilogue(a, blockIdx.x + tl * gridDim.x, tmem, tl & 1u, bar_acc + 8u * (tl & 1u),
                      (tl >> 1) & 1u, thr_s, S);
  }
  // the chunk barriers' last arrivals land before the CTA (and its shared memory) goes away
  if (__syncthreads_and(ok && live)) {
    if (it >= 1) ok &= tc_wait(bar_chunk + 8u * ((it - 1) & 1u), ((it - 1) >> 1) & 1u);
    if (it >= 2) ok &= tc_wait(bar_chunk + 8u * ((it - 2) & 1u), ((it - 2) >> 1) & 1u);
  }
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "n"(kTcTmemCols));
  }
  if (!ok) {
    for (uint32_t q = tid; q < a.nq; q += blockDim.x) atomicOr(a.status + a.q0 + q, ST_DEVICE);
  }
}

}  // namespace dev
}  // namespace aes
