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
//   - producer warps write a chunk's entries into one of two or three zeroed 32 KB chunk buffers
//     (and write them back to zero once the MMAs of that chunk have read the buffer);
//   - one thread issues the chunk's tcgen05.mma (kind::f8f6f4, M = 128, N = 128, K = 32 each)
//     into one of four 128-column FP32 accumulators in tensor memory; tcgen05.commit signals
//     mbarriers when a chunk buffer is read and when a tile's accumulator is complete;
//   - epilogue warps read a complete accumulator with tcgen05.ld while the next tiles' MMAs run:
//     every (row, query) score becomes the same candidate key as in the other passes and is
//     compared with the query's threshold; hits are appended exactly as the dp4a pass appends
//     them.
// Two blocks of 128 queries run together on CTA pairs (cta_group::2, M = 256 over the pair's two
// row tiles, N = 256 queries): the same roles in each CTA, the even CTA's thread issuing the MMAs
// (see k_cand_tc).
// The roles hand work over through mbarriers only.
// Both operands are K-major without swizzle (layout in aes_tc_layout.h).
// Reference counterpart: the candidate pass spmv_ucsr_top_k_multicore.hpp:195-413 (one query per
// pass on the FPGA); scores equal those of gold_algorithms.hpp:249-308 on the same integers.
#pragma once

#include "aes_kernels.cuh"
#include "aes_tc_layout.h"

namespace aes {
namespace dev {

// Warp roles: warps 0-7 stage the chunks (producers), warps 8-15 read the accumulators (warp w
// may only read tensor-memory lanes 32 (w % 4) .. + 31; warps 8-11 take the first half of the
// queries, warps 12-15 the second), warp 16 allocates tensor memory and its lane 0 issues the
// MMAs (on a pair: the even CTA's; lanes 0 and 1 of the odd CTA's forward barrier phases).
// They hand work over through mbarriers only.
constexpr int kTcProducers = 256;
constexpr int kTcEpiWarp = 8;
constexpr int kTcEpilogue = 256;
constexpr int kTcMmaWarp = 16;
constexpr int kTcThreads = 17 * 32;
constexpr uint32_t kTcTmemCols = 512;  // all of tensor memory, in FP32 accumulators
// Queries per launch and accumulators.  One CTA: 128 queries (N = 128, M = 128), four
// accumulators of 128 columns.  A CTA pair (cta_group::2): 256 queries (N = 256, each CTA
// holding 128 of them in its operand) and M = 256 (each CTA's 128-row tile), two accumulators
// of 256 columns in each CTA's tensor memory.
template <bool PAIR>
struct TcShape {
  static constexpr uint32_t Q = PAIR ? 2 * kTcQ : kTcQ;
  static constexpr uint32_t ACC = kTcTmemCols / Q;
};
// mbarriers of a kernel with nb chunk buffers and acc accumulators: staged[nb] (producers ->
// MMA), done[nb] (MMA -> producers), full[acc] (MMA -> epilogue), empty[acc] (epilogue -> MMA),
// drain (the MMA thread's own MMAs complete); then the tensor-memory address and the give-up
// flag
__host__ __device__ constexpr uint32_t tc_nbars(uint32_t nb, uint32_t acc) { return 2 * nb + 2 * acc + 1; }

// shared memory of one CTA of the pass with nb chunk buffers (2 or 3)
__host__ inline size_t tc_smem_bytes(uint32_t cols, uint32_t split, uint32_t nb, bool pair) {
  const uint32_t S = split <= 1 ? 1 : split;
  const uint32_t q = pair ? 2 * kTcQ : kTcQ;
  return tc_qtab_bytes(cols) + nb * (size_t)kTcChunkBytes + (size_t)S * q * 4 +
         ((tc_nbars(nb, kTcTmemCols / q) * 8 + 8 + 15) & ~15u);
}
// chunk buffers for a configuration: three where they fit next to the query operand and the
// thresholds (the producers then run two chunks ahead of the MMAs), else two
__host__ inline uint32_t tc_bufs(uint32_t cols, uint32_t split, size_t smem_limit, bool pair) {
  return tc_smem_bytes(cols, split, 3, pair) <= smem_limit ? 3u : 2u;
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
  const uint32_t* ent;   // per entry: byte offset in its chunk operand << 16 | e4m3 value
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
  uint32_t mma_idle;     // failure-path test: the MMA role issues nothing, so every hand-over
                         // wait of the other roles runs out and the CTA gives up
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
// Waits for the phase of the given parity to complete, for about a second at most, whether or
// not another role has given up: the MMA thread's wait for its own MMAs in flight before the CTA
// frees its tensor memory and leaves.
// CL: acquire at cluster scope (a barrier that the peer CTA of a pair arrives on, or whose
// phase orders work of the peer).
template <bool CL>
__device__ __forceinline__ uint32_t tc_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  if constexpr (CL) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done) : "r"(bar), "r"(parity) : "memory");
  } else {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done) : "r"(bar), "r"(parity) : "memory");
  }
  return done;
}
template <bool CL = false>
__device__ __forceinline__ bool tc_wait_own(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  uint32_t done = 0;
  while (!done) {
    done = tc_try<CL>(bar, parity);
    if (!done && clock64() - t0 > (1ll << 31)) return false;
  }
  return true;
}
// Waits for the phase of the given parity to complete.  Gives up after about a second, or as
// soon as another thread of the CTA has given up (*gave_up set), so that every role leaves its
// loop instead of waiting on a partner that has left.
template <bool CL = false>
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity, volatile uint32_t* gave_up) {
  const long long t0 = clock64();
  uint32_t done = 0;
  while (!done) {
    done = tc_try<CL>(bar, parity);
    if (done) break;
    if (*gave_up) return false;
    if (clock64() - t0 > (1ll << 31)) {
      *gave_up = 1u;
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ void tc_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Arrives on a barrier of the pair's even CTA (the one whose thread issues the MMAs): through
// its shared::cluster address, with release at cluster scope.  One CTA: a local arrive.
template <bool PAIR>
__device__ __forceinline__ void tc_arrive_leader(uint32_t bar) {
  if constexpr (PAIR) {
    uint32_t ra;
    asm volatile("mapa.shared::cluster.u32 %0, %1, 0;" : "=r"(ra) : "r"(bar));
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" :: "r"(ra) : "memory");
  } else {
    tc_arrive(bar);
  }
}
template <bool PAIR>
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t da, uint64_t db, uint32_t idesc,
                                       uint32_t acc) {
  if constexpr (PAIR) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n"
        :: "r"(d), "l"(da), "l"(db), "r"(idesc), "r"(acc));
  } else {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n"
        :: "r"(d), "l"(da), "l"(db), "r"(idesc), "r"(acc));
  }
}
// Arrives on `bar` once the MMAs issued so far complete.  PAIR: on the barrier at the same
// offset in each CTA of ctamask (bit r: the pair's CTA of rank r).
template <bool PAIR>
__device__ __forceinline__ void tc_commit(uint32_t bar, uint16_t ctamask = 3) {
  if constexpr (PAIR) {
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
        :: "r"(bar), "h"(ctamask) : "memory");
  } else {
    (void)ctamask;
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(bar) : "memory");
  }
}
// Tensor memory of the CTA (PAIR: of both CTAs, the same columns, by one warp of each)
template <bool PAIR>
__device__ __forceinline__ void tc_alloc(uint32_t slot) {
  if constexpr (PAIR) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(slot), "n"(kTcTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
  } else {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(slot), "n"(kTcTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
}
template <bool PAIR>
__device__ __forceinline__ void tc_dealloc(uint32_t tmem) {
  if constexpr (PAIR)
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" :: "r"(tmem), "n"(kTcTmemCols));
  else
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "n"(kTcTmemCols));
}
__device__ __forceinline__ void tc_cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
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

// Epilogue warps: reads accumulator `dbuf` of row tile T (thread = row, half the queries) and
// appends every (row, query) key at or above the query's threshold.  thf holds the thresholds as
// FP32 bounds on rs * score: rs is the row's scale, or 1 without row scales (the score is an
// exact integer in FP32, and times 1 it stays itself).
// A block of 32 queries is compared without branches into a bit mask of hits.  The hits of a
// thread then take their survivor slots with atomics issued back to back (none waits for
// another's result) before any survivor is written, so a block costs one atomic round trip
// however many of its queries hit; the eight epilogue warps all work on the same tile, so a
// round trip per hit would leave nothing to hide it behind.
// The thread's row of tile T, and its row scale (loaded before the accumulator wait, so that the
// load's latency passes while the MMAs finish)
__device__ __forceinline__ uint32_t tc_epi_row(uint32_t T) {
  return T * kTcRows + ((threadIdx.x >> 5) & 3u) * 32u + (threadIdx.x & 31u);
}
// The accumulator goes back to the MMA role (an arrive on `empty`) as soon as the thread's last
// load from it has completed, so the compares of the last block overlap the next MMAs.
template <bool PAIR>
__device__ __forceinline__ void tc_epilogue(const TcArgs& a, uint32_t T, uint32_t tmem,
                                            uint32_t dbuf, const float* thf_all, uint32_t S,
                                            float rs, uint32_t empty) {
  constexpr uint32_t Q = TcShape<PAIR>::Q, HALF = Q / 2;
  const uint32_t warp = threadIdx.x >> 5;
  const uint32_t g = warp & 3u, h = (warp - kTcEpiWarp) >> 2;
  const uint32_t row = tc_epi_row(T);
  const bool valid = row < a.n_rows;
  const uint32_t p = valid ? part_of(row, S, a.slice) : 0u;
  const float* thf = thf_all + p * Q;
#pragma unroll 1
  for (uint32_t col0 = h * HALF; col0 < h * HALF + HALF; col0 += 32u) {
    uint32_t v[32];
    tc_ld32(tmem + dbuf * Q + col0 + ((g * 32u) << 16), v);
    if (col0 + 32u == h * HALF + HALF) {  // the last load of this unit has completed
      tc_fence_before();
      tc_arrive(empty);
    }
    uint32_t hit = 0;
#pragma unroll
    for (int j4 = 0; j4 < 8; j4++) {  // the same 32 thresholds for every lane: 16-byte broadcasts
      const float4 x = reinterpret_cast<const float4*>(thf + col0)[j4];
      const float tj[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const float f = __uint_as_float(v[4 * j4 + u]);
        hit |= (__fmul_rn(f, rs) >= tj[u] ? 1u : 0u) << (4 * j4 + u);
      }
    }
    if (!valid || col0 >= a.nq) hit = 0;
    else if (a.nq - col0 < 32u) hit &= (1u << (a.nq - col0)) - 1u;
    const size_t qp0 = (size_t)(a.q0 + col0) * S + p;
#pragma unroll
    for (int j0 = 0; j0 < 32; j0 += 16) {  // 16 slots at a time keeps the slot indices in registers
      if (!((hit >> j0) & 0xFFFFu)) continue;
      uint32_t ix[16];
#pragma unroll
      for (int j = j0; j < j0 + 16; j++)
        if ((hit >> j) & 1u) ix[j - j0] = atomicAdd(a.cnt + qp0 + (size_t)j * S, 1u);
#pragma unroll
      for (int j = j0; j < j0 + 16; j++) {
        if (((hit >> j) & 1u) && ix[j - j0] < a.cap) {
          const float f = __uint_as_float(v[j]);
          const uint32_t key = a.rowscale ? key_f32(__fmul_rn(f, rs)) : key_i32(__float2int_rn(f));
          a.surv[(qp0 + (size_t)j * S) * a.cap + ix[j - j0]] = make_uint2(key, row);
        }
      }
    }
  }
}

constexpr int kTcPer = 8;  // entries of a chunk a producer thread holds (2048 per chunk)

// A producer's share of one chunk's entries: v[u] = entry b + tid + 256 u for tid + 256 u < n
struct TcEnt {
  uint32_t v[kTcPer];
  uint32_t b = 0, n = 0;
  __device__ __forceinline__ void load(const uint32_t* ent, uint32_t b_, uint32_t n_, uint32_t tid) {
    b = b_;
    n = n_;
#pragma unroll
    for (int u = 0; u < kTcPer; u++) {
      const uint32_t i = tid + (uint32_t)u * kTcProducers;
      v[u] = i < n ? __ldg(ent + b + i) : 0u;
    }
  }
  // writes the entries' e4m3 bytes (or zeros) into a chunk buffer
  __device__ __forceinline__ void stage(unsigned char* ab, const uint32_t* ent, uint32_t tid,
                                        bool clear) const {
#pragma unroll
    for (int u = 0; u < kTcPer; u++) {
      const uint32_t i = tid + (uint32_t)u * kTcProducers;
      if (i < n) ab[v[u] >> 16] = clear ? (uint8_t)0 : (uint8_t)v[u];
    }
    for (uint32_t i = tid + kTcPer * kTcProducers; i < n; i += kTcProducers) {
      const uint32_t e = __ldg(ent + b + i);
      ab[e >> 16] = clear ? (uint8_t)0 : (uint8_t)e;
    }
  }
};

// OR of `fail` over the producer threads (named barrier 1)
__device__ __forceinline__ bool tc_producers_any(bool fail) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred f, r;\n setp.ne.u32 f, %1, 0;\n bar.red.or.pred r, 1, %2, f;\n"
      " selp.u32 %0, 1, 0, r;\n}\n"
      : "=r"(r) : "r"((uint32_t)fail), "n"(kTcProducers) : "memory");
  return r != 0;
}


// One CTA per SM (PAIR: one CTA pair, a cluster of two, per two SMs), persistent over units of
// work U = unit, unit + units, ...: a 128-row tile (one CTA), or two consecutive tiles, 2U for
// the even CTA and 2U + 1 for the odd one (PAIR).  Chunk i of the CTA is chunk i % nch of its
// unit i / nch; chunk buffer i % NB; accumulator (unit t) t % ACC.
// PAIR: the even CTA's MMA thread issues cta_group::2 MMAs with M = 256 (the two CTAs' row tiles
// from their own chunk buffers) and N = 256 (the two CTAs' 128-query operands), and commits them
// to the barriers of both CTAs; both CTAs' producers and epilogues hand their buffers and
// accumulators back to the even CTA's barriers.  The two CTAs keep identical shared-memory
// layouts, since an operand descriptor addresses the same offset in both.
template <uint32_t NB, bool PAIR>
__global__ void __launch_bounds__(kTcThreads, 1) k_cand_tc(TcArgs a) {
  static_assert(NB == 2 || NB == 3, "two or three chunk buffers");
  constexpr uint32_t Q = TcShape<PAIR>::Q, ACC = TcShape<PAIR>::ACC;
  constexpr uint32_t kDone = NB, kFull = 2 * NB, kEmpty = 2 * NB + ACC;
  constexpr uint32_t kDrain = kEmpty + ACC, kBars = tc_nbars(NB, ACC);
  constexpr uint32_t R = NB + 2;  // producer ring: the chunks of every buffer and two ahead
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t qbytes = (a.kpad / 16u) * 2048u;
  unsigned char* sq = smem;                     // query operand (PAIR: this CTA's 128 queries)
  unsigned char* sa = smem + qbytes;            // NB chunk buffers of the row tile
  float* thf = reinterpret_cast<float*>(sa + NB * kTcChunkBytes);
  const uint32_t S = a.split <= 1 ? 1u : a.split;
  uint64_t* bars = reinterpret_cast<uint64_t*>(thf + S * Q);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + kBars);
  volatile uint32_t* gave_up = tslot + 1;
  const uint32_t tid = threadIdx.x, warp = tid >> 5;
  uint32_t rank = 0;  // the CTA's rank in its pair
  if constexpr (PAIR) asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
  const uint32_t unit = PAIR ? (blockIdx.x >> 1) : blockIdx.x;
  const uint32_t units = PAIR ? (gridDim.x >> 1) : gridDim.x;
  const uint32_t n_units = PAIR ? (a.n_rtiles + 1u) / 2u : a.n_rtiles;
  auto tile_of = [&](uint32_t u) { return PAIR ? 2u * u + rank : u; };  // this CTA's row tile
  {
    const uint4* src = reinterpret_cast<const uint4*>(a.qt + (PAIR ? rank * qbytes : 0u));
    uint4* dst = reinterpret_cast<uint4*>(sq);
    for (uint32_t i = tid; i < qbytes / 16u; i += blockDim.x) dst[i] = src[i];
    uint4* z = reinterpret_cast<uint4*>(sa);
    for (uint32_t i = tid; i < NB * kTcChunkBytes / 16u; i += blockDim.x) z[i] = make_uint4(0, 0, 0, 0);
    // thresholds as FP32 bounds on the score (int keys) or on rowscale * score:
    // key >= th  <=>  x >= bound for every x the pass produces
    for (uint32_t i = tid; i < S * Q; i += blockDim.x) {
      const uint32_t p = i / Q, q = i % Q;
      const uint32_t th = q < a.nq ? a.thr[(size_t)(a.q0 + q) * S + p] : 0xFFFFFFFFu;
      float fb;
      if (a.rowscale) {  // x >= +0, key(x) = bits(x) | 2^31; NaN bits: never
        fb = th <= 0x80000000u ? -__int_as_float(0x7f800000) : __uint_as_float(th & 0x7FFFFFFFu);
      } else {           // |score| < 2^24, exact in FP32
        const int32_t b = (int32_t)(th ^ 0x80000000u);
        fb = b > (1 << 24) ? __int_as_float(0x7f800000)
                           : (b < -(1 << 24) ? -__int_as_float(0x7f800000) : __int2float_rn(b));
      }
      thf[i] = fb;
    }
  }
  if (tid == 0) {
    for (uint32_t b = 0; b < kBars; b++) {
      // The roles arrive on their own CTA's staged and empty barriers.  PAIR: a thread of the
      // odd CTA forwards each completed phase of those to the even CTA's, which therefore take
      // one arrival more (a release at cluster scope costs about a thousand cycles: forwarded,
      // it stays off the producers' and the epilogue's paths)
      const uint32_t fwd = (PAIR && rank == 0) ? 1u : 0u;
      const uint32_t cnt = (b < kDone) ? (uint32_t)kTcProducers + fwd
                                       : ((b >= kEmpty && b < kDrain) ? (uint32_t)kTcEpilogue + fwd : 1u);
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(tc_smem_u32(bars + b)), "r"(cnt));
    }
    *gave_up = 0u;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kTcMmaWarp) tc_alloc<PAIR>(tc_smem_u32(tslot));
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  if constexpr (PAIR) tc_cluster_sync();  // both CTAs' barriers exist before any remote arrive
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t b_staged = tc_smem_u32(bars), b_done = tc_smem_u32(bars + kDone);
  const uint32_t b_full = tc_smem_u32(bars + kFull), b_empty = tc_smem_u32(bars + kEmpty);
  const uint32_t ntl = n_units > unit ? (n_units - unit + units - 1) / units : 0u;
  const uint32_t total = ntl * a.nch;  // chunks of this CTA (PAIR: the same in both CTAs)
  bool ok = true;

  if (warp < kTcProducers / 32) {
    // ---- producers ----------------------------------------------------------------------------
    // Chunk i lives in ring set E[i % R], R = NB + 2 (indices fixed at compile time: the loop
    // below is unrolled R ways).  Step i clears chunk i - NB, the last chunk of buffer i % NB,
    // from E[(i + 2) % R], loads chunk i + 2 into that set and stages chunk i (loaded two steps
    // earlier); a chunk's row offsets are read R steps before its entries.  So no register a
    // store or a copy reads waits on a load in flight.
    // chunk id of chunk i: tile tile_of(unit + (i / nch) units), chunk i % nch; kept
    // incrementally for the look-ahead chunk (no division per step).  PAIR: the odd CTA's tile
    // of the last unit may lie past the matrix; its chunks are empty.
    uint32_t la_i = 0, la_t = tile_of(unit), la_c = 0;
    auto ptr_next = [&](uint32_t& b, uint32_t& e) {  // offsets of chunk la_i, then advance it
      const bool in = la_i < total && la_t < a.n_rtiles;
      const uint32_t j = la_t * a.nch + la_c;
      b = in ? __ldg(a.ptr + j) : 0u;
      e = in ? __ldg(a.ptr + j + 1) : 0u;
      la_i++;
      if (++la_c == a.nch) {
        la_c = 0;
        la_t += (PAIR ? 2u : 1u) * units;
      }
    };
    TcEnt E[R];
    uint32_t Pb[R], Pe[R];  // P[j % R]: row offsets of chunk j, for j = i + 2 .. i + R + 1
    {
      uint32_t b, e;
      ptr_next(b, e);
      E[0].load(a.ent, b, e - b, tid);
      ptr_next(b, e);
      E[1].load(a.ent, b, e - b, tid);
#pragma unroll
      for (uint32_t j = 2; j < R + 2; j++) ptr_next(Pb[j % R], Pe[j % R]);
    }
    uint32_t buf = 0;  // i % NB
    auto step = [&](uint32_t i, TcEnt& cur, TcEnt& old, uint32_t& pb, uint32_t& pe) -> bool {
      unsigned char* ab = sa + buf * kTcChunkBytes;
      if (i >= NB) {  // the MMAs of chunk i - NB have read this buffer: clear its entries
        ok &= tc_wait<PAIR>(b_done + 8u * buf, ((i - NB) / NB) & 1u, gave_up);
        if (ok) old.stage(ab, a.ent, tid, true);
      }
      // every clear lands before any write of this chunk (they may share a byte); the
      // producers leave together at the first failure
      if (tc_producers_any(!ok)) return false;
      old.load(a.ent, pb, pe - pb, tid);  // chunk i + 2
      ptr_next(pb, pe);                   // chunk i + R + 2
      cur.stage(ab, a.ent, tid, false);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tc_arrive(b_staged + 8u * buf);
      buf = buf + 1 == NB ? 0u : buf + 1;
      return true;
    };
    bool go = true;
    for (uint32_t i0 = 0; go && i0 < total; i0 += R) {
#pragma unroll
      for (uint32_t k = 0; k < R; k++) {
        if (i0 + k >= total) break;
        go = step(i0 + k, E[k], E[(k + 2) % R], Pb[(k + 2) % R], Pe[(k + 2) % R]);
        if (!go) break;
      }
    }
  } else if (warp < kTcEpiWarp + kTcEpilogue / 32) {
    // ---- epilogue -----------------------------------------------------------------------------
    for (uint32_t tl = 0; tl < ntl; tl++) {
      const uint32_t d = tl % ACC;
      const uint32_t T = tile_of(unit + tl * units), row = tc_epi_row(T);
      // without row scales rs = 1: f * 1 is f exactly, so every score takes one path
      const float rs = a.rowscale ? (row < a.n_rows ? __ldg(a.rowscale + row) : 0.0f) : 1.0f;
      ok &= tc_wait<PAIR>(b_full + 8u * d, (tl / ACC) & 1u, gave_up);
      ok = __all_sync(0xFFFFFFFFu, ok);  // tcgen05.ld needs the whole warp
      if (!ok) break;
      tc_fence_after();
      tc_epilogue<PAIR>(a, T, tmem, d, thf, S, rs, b_empty + 8u * d);
    }
  } else if ((tid & 31u) == 0 && rank == 0) {
    // ---- MMA issue (one thread; PAIR: of the even CTA) ----------------------------------------
    // instruction descriptor: FP32 accumulator, e4m3 x e4m3, both K-major, N = Q, M = 128 (256
    // over a pair)
    const uint32_t idesc = (1u << 4) | ((Q >> 3) << 17) | (((PAIR ? 2u : 1u) * kTcRows >> 4) << 24);
    const uint32_t sq_addr = tc_smem_u32(sq), sa_addr = tc_smem_u32(sa);
    uint32_t tl = 0, c = 0, issued = 0;
    for (uint32_t i = 0; i < total && !a.mma_idle; i++) {
      const uint32_t buf = i % NB, d = tl % ACC;
      if (c == 0 && tl >= ACC) ok &= tc_wait<PAIR>(b_empty + 8u * d, ((tl - ACC) / ACC) & 1u, gave_up);
      if (ok) ok &= tc_wait<PAIR>(b_staged + 8u * buf, (i / NB) & 1u, gave_up);
      if (!ok) break;
      tc_fence_after();
      const uint32_t nk = min(kTcChunkK, a.kpad - c * kTcChunkK) / 32u;
      for (uint32_t kk = 0; kk < nk; kk++)
        tc_mma<PAIR>(tmem + d * Q, tc_desc(sa_addr + buf * kTcChunkBytes + kk * 4096u),
                     tc_desc(sq_addr + (c * 16u + 2u * kk) * 2048u), idesc, (c | kk) != 0);
      tc_commit<PAIR>(b_done + 8u * buf);
      if (c == a.nch - 1) tc_commit<PAIR>(b_full + 8u * d);
      issued = i + 1;
      if (++c == a.nch) {
        c = 0;
        tl++;
      }
    }
    // Before the CTA frees its tensor memory and its shared memory goes away, every MMA this
    // thread issued has completed and the arrivals of its commits have landed, whether the
    // roles finished or gave up: the last commit of each chunk buffer and of each accumulator,
    // and a final commit on the drain barrier (each waited for at most about a second).
    if (issued >= 1) {
      bool drained = true;
      for (uint32_t j = 1; j <= NB && j <= issued; j++)  // the last use of each chunk buffer
        drained &= tc_wait_own<PAIR>(b_done + 8u * ((issued - j) % NB), ((issued - j) / NB) & 1u);
      const uint32_t tiles_full = issued / a.nch;  // units whose accumulator commit was issued
      for (uint32_t j = 1; j <= ACC && j <= tiles_full; j++)  // the last use of each accumulator
        drained &= tc_wait_own<PAIR>(b_full + 8u * ((tiles_full - j) % ACC), ((tiles_full - j) / ACC) & 1u);
      tc_commit<PAIR>(tc_smem_u32(bars + kDrain), 1);
      drained &= tc_wait_own<PAIR>(tc_smem_u32(bars + kDrain), 0u);
      if (!drained) *gave_up = 1u;
    }
  } else if (PAIR && rank == 1 && (tid & 31u) == 1) {
    // ---- the odd CTA: forwards each completed phase of its empty barriers (its epilogue has
    // read the accumulator) to the even CTA's
    for (uint32_t tl = 0; tl < ntl; tl++) {
      const uint32_t d = tl % ACC;
      if (!tc_wait(b_empty + 8u * d, (tl / ACC) & 1u, gave_up)) break;
      tc_arrive_leader<PAIR>(b_empty + 8u * d);
    }
  } else if (PAIR && rank == 1 && (tid & 31u) == 0) {
    // ---- the odd CTA: forwards each completed phase of its staged barriers (its producers have
    // staged the chunk) to the even CTA's
    for (uint32_t i = 0; i < total; i++) {
      const uint32_t buf = i % NB;
      if (!tc_wait(b_staged + 8u * buf, (i / NB) & 1u, gave_up)) break;
      tc_arrive_leader<PAIR>(b_staged + 8u * buf);
    }
    // before the CTA leaves, the even CTA's commits to its barriers have landed (the last use of
    // each chunk buffer and accumulator; skipped once it gave up)
    bool drained = true;
    for (uint32_t j = 1; j <= NB && j <= total && drained && !*gave_up; j++)
      drained = tc_wait_own<PAIR>(b_done + 8u * ((total - j) % NB), ((total - j) / NB) & 1u);
    for (uint32_t j = 1; j <= ACC && j <= ntl && drained && !*gave_up; j++)
      drained = tc_wait_own<PAIR>(b_full + 8u * ((ntl - j) % ACC), ((ntl - j) / ACC) & 1u);
    if (!drained) *gave_up = 1u;
  }
  tc_fence_before();
  __syncthreads();
  // PAIR: neither CTA frees its tensor memory or leaves while the even CTA's MMAs may still read
  // the odd CTA's shared memory or the odd CTA's roles still arrive on the even CTA's barriers
  if constexpr (PAIR) tc_cluster_sync();
  if (warp == kTcMmaWarp) {
    __syncwarp();
    tc_fence_after();
    tc_dealloc<PAIR>(tmem);
  }
  if (*gave_up && tid == 0) {
    for (uint32_t q = 0; q < a.nq; q++) atomicOr(a.status + a.q0 + q, ST_DEVICE);
  }
}

}  // namespace dev
}  // namespace aes
