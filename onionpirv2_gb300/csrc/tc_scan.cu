// tc_scan.cu -- first dimension of a batch of queries on the tcgen05 tensor cores.
//
// Per NTT slot c the first dimension of B queries is the integer product
// (n_rest x n1) . (n1 x 2B) of 60-bit residues, accumulated exactly
// (matrix.cpp:79-97, 220-235 compute it with 64x64->128-bit multiply-adds,
// server.cpp:178-293 reduce the 128-bit sums mod q).  Here every residue is
// split into balanced limbs that are exact in bf16: a database residue into
// eight 8-bit limbs, v = sum_i d_i 2^(8i) with d_i in [-128, 127] (the top
// limb in [0, 16]), a query residue into eight such limbs or into seven
// 9-bit limbs, v = sum_j e_j 2^(9j) with e_j in [-256, 255] (the top limb in
// [0, 64]).  A limb product is at most 2^15 in magnitude and a sum of 512 of
// them at most 2^24, so the fp32 accumulation of tcgen05.mma kind::f16 is
// exact.  Longer first dimensions run as segments of at most 512 k inside
// one launch: the MMAs of each segment fill an accumulator of their own, the
// epilogue reduces it mod q and keeps the running sum in registers, and a
// tile's result is stored once, after its last segment.
//
// MMA shape per tile: M = 16 database rows x 8 limbs = 128 (TMEM lanes),
// N = 2B query polynomials x QL limbs (QL = 8 or 7; two MMAs of <= 256
// columns), K = n1.  Cell (row r, limb i ; query poly b', limb j) holds
// x_ij = sum_k d_i(A[r,k]) e_j(Q[k,b']); the result is
// sum_s Y_s 2^(8s), Y_s = sum_{i+j=s} x_ij w^j, with w = 1 for 8-bit query
// limbs (weight 2^(8i+8j)) and w = 2 for 9-bit ones (2^(8i+9j) =
// 2^(8(i+j)) 2^j).  The epilogue gathers the anti-diagonal sums Y_s across
// the 8 lanes of a row with one skewed shuffle pass, rebuilds the exact
// (<= 2^130) integer from them and reduces it mod q -- the same value the
// 128-bit accumulation of the reference reduces, without its wrap-around
// (the sum is exact here).  Seven query limbs do 56 limb products per
// modular multiply-add instead of 64; the row side keeps eight limbs because
// a tile's 128 TMEM lanes must hold whole rows of limbs.
//
// Data layout in HBM (bf16 limbs, "core matrices" of 8 rows x 8 k):
//   database  dbl[c][rb][k/8][r%16][i][k%8]      (rb = r / 16)
//   queries   ql [c][h][k/8][b'][j][k%8]         (b' = 2 b + poly - 32 h)
// (h: column half of at most 32 query polynomials, <= 256 TMEM columns), so
// the slice of a pipeline stage (32 or 64 k) of either operand is contiguous
// and lands in shared memory in the K-major, no-swizzle canonical layout
// that the tcgen05 shared-memory descriptors below describe (leading byte
// offset = stride between core matrices along k, stride byte offset = 128
// between 8-row groups).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <cstdlib>
#include <cstring>

#include "async.cuh"
#include "common.cuh"
#include "kernels.h"

namespace opir {
namespace {

constexpr int kTcRows = 16;                 // database rows per tile
constexpr int kTcKC = 32;                   // k granularity of the first dimension
constexpr int kTcMaxNB = 128;               // query polynomials per pass (64 queries)
constexpr int kTcHalfNB = 32;               // query polynomials per tile (<= 256 TMEM columns)
static_assert(kTcHalfNB / 8 <= 4, "the epilogue holds two groups per warp part");
// pipeline stages: KC k per stage (64, or 32 when the segment length is an
// odd multiple of 32), STAGES stages; the 64-k ring (4 x 48 KB) measured
// 25 % faster than the 32-k ring (8 x 24 KB) and 5 % faster than 2 x 96 KB.
// A CTA pair (PAIR) holds half of the query tile per CTA: 32 KB stages.
template <int KC>
__host__ __device__ constexpr uint32_t tc_a_bytes() { return KC / 8 * kTcRows * 128; }
template <int KC, bool PAIR = false>
__host__ __device__ constexpr uint32_t tc_stage_bytes() {
  return tc_a_bytes<KC>() + KC / 8 * (PAIR ? kTcHalfNB / 2 : kTcHalfNB) * 128;
}
// ring depth: the stages that fit beside the epilogue's staging
template <int KC, bool PAIR>
constexpr int tc_stages() { return PAIR ? (KC == 64 ? 6 : 12) : (KC == 64 ? 4 : 8); }
constexpr int kTcYStride = 168;             // int32 words per (warp, row) block of Y staging
constexpr int kTcEpiWarps = 8;              // two per TMEM lane quadrant
constexpr int kTcThreads = (kTcEpiWarps + 2) * 32;  // epilogue warps, producer, MMA
constexpr int kTcProducer = kTcEpiWarps, kTcMma = kTcEpiWarps + 1;
constexpr uint32_t kTcTmemCols = 512;       // two 256-column accumulators

constexpr uint32_t kErrTcWaitFull = 8u;
constexpr uint32_t kErrTcWaitEmpty = 16u;
constexpr uint32_t kErrTcWaitAcc = 32u;
constexpr uint32_t kErrTcDrain = 64u;
constexpr uint32_t kErrTcRange = 128u;

constexpr int kTcMaxSegment = 512;  // k per exact fp32 accumulation
int g_tc_ring = -1;                 // OPIR_TC_RING: force a ring shape (tests, sweeps)
int g_tc_pass = kTcMaxNB / 2;       // OPIR_TC_PASS: queries per pass (16, 32, 48 or 64)
int pass_max() { return g_tc_pass; }

struct TcGeom {
  int n1, n_rest, batch;      // batch: queries of the pass
  int nh, nbh;                // column halves, query polynomials per half (multiple of 8;
                              // of 16 with 7 query limbs, so that N is a multiple of 16)
  int ql;                     // limbs per query residue: 8 (8-bit) or 7 (9-bit)
  int n_rb;                   // row tiles of 16 rows
  int nseg;                   // k segments of at most kTcMaxSegment
  bool pair;                  // CTA pairs: M = 256 (two row tiles), half the query tile each
  long long units;            // N * (n_rb or n_rb / 2) * nh tiles (or tile pairs)
  uint32_t b_bytes;           // query bytes per stage and CTA
  uint32_t idesc;             // instruction descriptor (M = 128 or 256, N = ql nbh)
};

// pipeline stages (of KC k) in segment s
template <int KC>
__device__ __forceinline__ int seg_chunks(const TcGeom &G, int s) {
  const int len = G.n1 - s * kTcMaxSegment;
  return (len < kTcMaxSegment ? len : kTcMaxSegment) / KC;
}

// Shared-memory matrix descriptor (tcgen05): start address, leading byte
// offset (k direction), stride byte offset (8-row groups), version 1, no
// swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t addr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(addr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
// 8 columns; the caller waits (tmem_ld_wait) before it reads r
__device__ __forceinline__ void tmem_ld8(uint32_t addr, uint32_t *r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                 "=r"(r[6]), "=r"(r[7])
               : "r"(addr));
}
// wait for the loads issued so far; the empty asm per register keeps every
// read of r after the wait
template <int NR>
__device__ __forceinline__ void tmem_ld_wait(uint32_t (&r)[NR]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < NR; ++i) asm volatile("" : "+r"(r[i]));
}

// ---- CTA pairs (tcgen05 cta_group::2): the even CTA of a two-CTA cluster
// issues M = 256 MMAs that read A (128 rows) and half of B from each CTA's
// shared memory and write each CTA's own tensor memory.
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_id_x() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_count_x() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::
                   : "memory");
}
// shared::cluster address of the variable at p in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t cluster_addr(const void *p, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t addr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(addr)
               : "memory");
}
// try_wait with cluster-scope acquire (arrivals from the other CTA), with or
// without a suspend-time hint
template <bool kHint>
__device__ __forceinline__ bool mbar_try_wait_cl(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  if constexpr (kHint)
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(kSuspendHintNs)
        : "memory");
  else
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
  return ok != 0;
}
// bounded waits of the tensor kernel: cluster scope in the pair form
template <bool PAIR, bool kHint = false>
__device__ __forceinline__ bool tc_wait(uint64_t *bar, uint32_t parity) {
  for (uint32_t i = 0; i < kSpinLimit; ++i) {
    if constexpr (PAIR) {
      if (mbar_try_wait_cl<kHint>(bar, parity)) return true;
    } else if constexpr (kHint) {
      if (mbar_try_wait_hint(bar, parity)) return true;
    } else {
      if (mbar_try_wait(bar, parity)) return true;
    }
  }
  return false;
}
__device__ __forceinline__ void tc_mma2(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
// arrive on the barrier at bar's offset in both CTAs of the pair once the
// pair MMAs issued so far complete
__device__ __forceinline__ void tc_commit2_both(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 "
      "[%0], %1;" ::"r"(smem_u32(bar)),
      "h"((unsigned short)3)
      : "memory");
}
// Tensor copy of the box at rows [y, y + box) of a [rows][128 bytes] view,
// issued by CTA 1 of a pair into its own shared memory, completing on the
// barrier of CTA 0 (cluster address bar): the pair's copies of a stage all
// count on CTA 0's barrier, with no thread in between.
__device__ __forceinline__ void tma_rows_pair(void *dst, const CUtensorMap *map, int y,
                                              uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(y), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tc_commit2(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// sum_s y_s 2^(8s) (exact, >= 0 and < 2^132) mod q
__device__ __forceinline__ uint64_t tc_combine(const int (&y)[16], uint64_t q, uint64_t mu_lo,
                                               uint64_t mu_hi, uint64_t r64, uint64_t r128,
                                               bool &range_ok) {
  uint32_t w[4];
  long long carry = 0;
#pragma unroll
  for (int g = 0; g < 4; ++g) {
    const long long s = carry + (long long)y[4 * g] + (long long)y[4 * g + 1] * 256 +
                        (long long)y[4 * g + 2] * 65536 + (long long)y[4 * g + 3] * 16777216;
    w[g] = (uint32_t)s;
    carry = s >> 32;  // arithmetic: floor division
  }
  range_ok = carry >= 0 && carry < 16;
  const uint64_t lo = ((uint64_t)w[1] << 32) | w[0];
  const uint64_t hi = ((uint64_t)w[3] << 32) | w[2];
  // hi 2^64 + lo + carry 2^128 == hi r64 + lo + carry r128 (mod q); < 2^125
  U128 acc = mul_wide(hi, r64);
  add_to(acc, U128{lo, 0});
  add_to(acc, U128{(uint64_t)(carry & 15) * r128, 0});
  return barrett128(acc, q, mu_lo, mu_hi);
}

// PAIR: a two-CTA cluster shares each MMA (cta_group::2, M = 256): CTA r
// of the pair loads row tile 2 t + r of tile pair t and query polynomials
// [r nbh/2, (r+1) nbh/2) of the column half.  CTA 1 loads with tensor copies
// (tm_a, tm_b: [rows][128 bytes] views of the limb planes) that complete on
// CTA 0's stage barrier, so CTA 0 issues the MMAs as soon as both CTAs'
// bytes have landed; the MMAs' completion frees the stage in both CTAs
// (multicast commit), both CTAs' epilogues read their own tensor memory and
// report back to CTA 0.  Every wait is bounded and cluster-scoped.
template <int KC, int STAGES, int QL, bool PAIR>
__global__ void __launch_bounds__(kTcThreads, 1)
    tc_scan_kernel(const uint16_t *__restrict__ dbl, const uint16_t *__restrict__ ql, uint64_t *out,
                   size_t out_stride, int b_base, TcGeom G, uint64_t q, uint64_t mu_lo,
                   uint64_t mu_hi, uint64_t r64, uint64_t r128, uint32_t *status,
                   const __grid_constant__ CUtensorMap tm_a,
                   const __grid_constant__ CUtensorMap tm_b) {
  constexpr int kTcKB = KC / 8;  // core matrices along k per stage
  constexpr uint32_t kTcABytes = tc_a_bytes<KC>(), kTcStageBytes = tc_stage_bytes<KC, PAIR>();
  extern __shared__ __align__(1024) unsigned char smem[];
  // the epilogue's staging follows the ring, so that no MMA operand read
  // can leave the allocation
  int *ysm = reinterpret_cast<int *>(smem + STAGES * kTcStageBytes);
  uint64_t *bars = reinterpret_cast<uint64_t *>(ysm + kTcEpiWarps * 4 * kTcYStride);
  uint64_t *full = bars, *empty = bars + STAGES;
  uint64_t *acc_full = bars + 2 * STAGES;  // [2]
  uint64_t *acc_empty = acc_full + 2;      // [2]
  uint64_t *drained = acc_full + 4;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * STAGES + 5);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = PAIR ? cluster_rank() : 0;
  // this CTA's (or pair's) share of the tiles
  const long long first_unit = PAIR ? (long long)cluster_id_x() : (long long)blockIdx.x;
  const long long unit_step = PAIR ? (long long)cluster_count_x() : (long long)gridDim.x;
  const int n_ut = PAIR ? G.n_rb / 2 : G.n_rb;  // row tiles (pairs) per slot
  const int nbc = PAIR ? G.nbh / 2 : G.nbh;     // query polynomials in this CTA's B tile

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], PAIR ? 2 * kTcEpiWarps : kTcEpiWarps);
    }
    mbar_init(drained, 1);
    mbar_fence_init();
  }
  if (warp == kTcMma) {
    if constexpr (PAIR) {
      asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                       smem_u32(tmem_slot)),
                   "r"(kTcTmemCols)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
    } else {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                       smem_u32(tmem_slot)),
                   "r"(kTcTmemCols)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
  }
  tc_fence_before();
  // both CTAs' barriers are initialised before either signals the other
  if constexpr (PAIR)
    cluster_sync_all();
  else
    __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t smem_base = smem_u32(smem);
  const int kblk = G.n1 / 8;
  const long long per_c = (long long)n_ut * G.nh;

  if (warp == kTcProducer) {
    // ------------------------------ producer ------------------------------
    if (lane == 0) {
      long long it = 0;
      bool ok = true;
      // CTA 0 of a pair expects both CTAs' bytes; CTA 1's copies land on it
      const uint32_t stage_tx = (PAIR ? 2u : 1u) * (kTcABytes + G.b_bytes);
      const uint32_t full0 = PAIR ? cluster_addr(full, 0) : 0u;
      for (long long u = first_unit; u < G.units && ok; u += unit_step) {
        const long long c = u / per_c, rem = u % per_c;
        const long long rt = rem / G.nh, hf = rem % G.nh;
        const long long rb = PAIR ? 2 * rt + rank : rt;
        const long long hb = PAIR ? 2 * hf + rank : hf;  // B tile in the query limb layout
        const int nhc = PAIR ? 2 * G.nh : G.nh;
        const uint16_t *a_src = dbl + (size_t)(c * G.n_rb + rb) * kblk * (kTcRows * 64);
        const uint16_t *b_src = ql + (size_t)(c * nhc + hb) * kblk * nbc * (QL * 8);
        for (int kc = 0; kc < G.n1 / KC; ++kc, ++it) {
          const int s = (int)(it % STAGES);
          const long long round = it / STAGES;
          if (round > 0 && !tc_wait<PAIR>(&empty[s], (uint32_t)((round - 1) & 1))) {
            report_error(status, kErrTcWaitEmpty);
            ok = false;
            break;
          }
          unsigned char *st = smem + (size_t)s * kTcStageBytes;
          const uint16_t *a_k = a_src + (size_t)kc * kTcKB * (kTcRows * 64);
          const uint16_t *b_k = b_src + (size_t)kc * kTcKB * nbc * (QL * 8);
          if (PAIR && rank == 1) {
            // rows of 128 bytes (64 limbs) from the start of each plane
            tma_rows_pair(st, &tm_a, (int)((a_k - dbl) / 64), full0 + (uint32_t)s * 8u);
            tma_rows_pair(st + kTcABytes, &tm_b, (int)((b_k - ql) / 64),
                          full0 + (uint32_t)s * 8u);
          } else {
            mbar_arrive_expect_tx(&full[s], stage_tx);
            bulk_g2s(st, a_k, kTcABytes, &full[s]);
            bulk_g2s(st + kTcABytes, b_k, G.b_bytes, &full[s]);
          }
        }
      }
      // never leave the CTA with copies still landing in its shared memory
      // (CTA 1's land on CTA 0's barriers, which CTA 0 drains before the
      // pair's final cluster barrier)
      const long long first = it > STAGES ? it - STAGES : 0;
      if (!(PAIR && rank == 1))
        for (long long j = first; j < it; ++j)
          if (!mbar_wait(&full[j % STAGES], (uint32_t)((j / STAGES) & 1))) {
            report_error(status, kErrTcDrain);
            break;
          }
    }
  } else if (warp == kTcMma && rank == 1) {
    // CTA 1 of a pair: its MMA warp only holds the tensor memory allocation
  } else if (warp == kTcMma) {
    // ------------------------------ MMA issue ------------------------------
    if (lane == 0) {
      const uint32_t lbo_a = kTcRows * 128, lbo_b = (uint32_t)nbc * (QL * 16);
      long long it = 0, j = 0;  // j: accumulators filled, one per (tile, segment)
      bool ok = true;
      for (long long u = first_unit; u < G.units && ok; u += unit_step) {
        for (int sg = 0; sg < G.nseg && ok; ++sg, ++j) {
          const int buf = (int)(j & 1);
          // accumulator buf was last used by accumulator j - 2
          if (j >= 2 && !tc_wait<PAIR>(&acc_empty[buf], (uint32_t)(((j >> 1) - 1) & 1))) {
            report_error(status, kErrTcWaitAcc);
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d = tmem + (uint32_t)buf * 256;
          const int nkc = seg_chunks<KC>(G, sg);
          for (int kc = 0; kc < nkc; ++kc, ++it) {
            const int s = (int)(it % STAGES);
            const uint32_t par = (uint32_t)((it / STAGES) & 1);
            if (!tc_wait<PAIR>(&full[s], par)) {
              report_error(status, kErrTcWaitFull);
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t sa = smem_base + (uint32_t)s * kTcStageBytes, sb = sa + kTcABytes;
#pragma unroll
            for (int ks = 0; ks < KC / 16; ++ks) {
              const uint64_t da = smem_desc(sa + ks * 2 * lbo_a, lbo_a, 128);
              const uint64_t db = smem_desc(sb + ks * 2 * lbo_b, lbo_b, 128);
              const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
              if constexpr (PAIR)
                tc_mma2(d, da, db, G.idesc, acc);
              else
                tc_mma(d, da, db, G.idesc, acc);
            }
            // the stage is free (in both CTAs) once these MMAs have read it
            if constexpr (PAIR)
              tc_commit2_both(&empty[s]);
            else
              tc_commit(&empty[s]);
          }
          if (ok) {
            if constexpr (PAIR)
              tc_commit2_both(&acc_full[buf]);
            else
              tc_commit(&acc_full[buf]);
          }
        }
      }
      // wait for every MMA issued so far before the columns are released
      if constexpr (PAIR)
        tc_commit2(drained);
      else
        tc_commit(drained);
      if (!mbar_wait(drained, 0)) report_error(status, kErrTcDrain);
    }
  } else {
    // ------------------------------ epilogue ------------------------------
    // warp: TMEM lane quadrant qd (rows 4 qd .. 4 qd + 3 of the tile), and
    // every other group of 8 query polynomials starting at part
    const int qd = warp & 3, part = warp >> 2;
    const int t8 = lane & 7, rsub = lane >> 3;
    int *yw = ysm + (warp * 4 + rsub) * kTcYStride;
    const uint32_t lane_bits = (uint32_t)(qd * 32) << 16;
    const int groups = G.nbh / 8;
    // the MMA issuer's accumulator-free barriers
    const uint32_t acc_empty0 = PAIR ? cluster_addr(acc_empty, 0) : 0u;
    long long j = 0;
    bool range_ok = true, alive = true;
    for (long long u = first_unit; u < G.units && alive; u += unit_step) {
      const long long c = u / per_c, rem = u % per_c;
      const long long rt = rem / G.nh, hf = rem % G.nh;
      const long long rb = PAIR ? 2 * rt + rank : rt;
      const size_t row = (size_t)rb * kTcRows + qd * 4 + rsub;
      // this lane's cell of groups part and part + 2 (a tile has kTcHalfNB / 8
      // <= 4 groups of 8 query polynomials over two warp parts)
      uint64_t sum[2] = {0, 0};
      for (int sg = 0; sg < G.nseg; ++sg, ++j) {
        const int buf = (int)(j & 1);
        bool got = true;
        if (lane == 0) got = tc_wait<PAIR, true>(&acc_full[buf], (uint32_t)((j >> 1) & 1));
        got = __shfl_sync(0xffffffffu, got, 0);
        if (!got) {
          if (lane == 0) report_error(status, kErrTcWaitAcc);
          alive = false;
          break;
        }
        tc_fence_after();
        const uint32_t acc_addr = tmem + lane_bits + (uint32_t)buf * 256;
#pragma unroll
        for (int gi = 0; gi < 2; ++gi) {
          const int grp = part + 2 * gi;
          if (grp >= groups) break;
          if constexpr (QL == 8) {
#pragma unroll
            for (int hc = 0; hc < 2; ++hc) {
              uint32_t r[32];
              tmem_ld32(acc_addr + (uint32_t)((grp * 2 + hc) * 32), r);
#pragma unroll
              for (int bl = 0; bl < 4; ++bl) {
                int x[8];
#pragma unroll
                for (int d = 0; d < 8; ++d) x[d] = __float2int_rn(__uint_as_float(r[bl * 8 + d]));
                // skewed exchange: lane t8 collects Y_t8 and Y_(t8+8) of its row
                int ylo = x[0], yhi = 0;
#pragma unroll
                for (int d = 1; d < 8; ++d) {
                  const int v = __shfl_sync(0xffffffffu, x[d], (lane & ~7) | ((lane - d) & 7));
                  if (d <= t8)
                    ylo += v;
                  else
                    yhi += v;
                }
                int *yb = yw + (hc * 4 + bl) * 20;
                yb[t8] = ylo;
                yb[t8 + 8] = yhi;
              }
            }
          } else {
            // 8 polynomials x 7 limbs = 56 columns from column 56 grp
            uint32_t r[56];
#pragma unroll
            for (int m = 0; m < 7; ++m) tmem_ld8(acc_addr + (uint32_t)(grp * 56 + m * 8), r + m * 8);
            tmem_ld_wait(r);
#pragma unroll
            for (int bl = 0; bl < 8; ++bl) {
              // x_ij 2^j: |x_ij| <= 2^24, so |Y_s| <= 127 * 2^24 < 2^31
              int x[7];
#pragma unroll
              for (int d = 0; d < 7; ++d)
                x[d] = __float2int_rn(__uint_as_float(r[bl * 7 + d])) * (1 << d);
              int ylo = x[0], yhi = 0;
#pragma unroll
              for (int d = 1; d < 7; ++d) {
                const int v = __shfl_sync(0xffffffffu, x[d], (lane & ~7) | ((lane - d) & 7));
                if (d <= t8)
                  ylo += v;
                else
                  yhi += v;
              }
              int *yb = yw + bl * 20;
              yb[t8] = ylo;
              yb[t8 + 8] = yhi;  // Y_14 = Y_15 = 0
            }
          }
          __syncwarp();
          int y[16];
          const int4 *src = reinterpret_cast<const int4 *>(yw + t8 * 20);
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            const int4 t = src[v];
            y[4 * v] = t.x;
            y[4 * v + 1] = t.y;
            y[4 * v + 2] = t.z;
            y[4 * v + 3] = t.w;
          }
          __syncwarp();
          bool ok_one = true;
          const uint64_t val = tc_combine(y, q, mu_lo, mu_hi, r64, r128, ok_one);
          range_ok &= ok_one;
          sum[gi] = sg == 0 ? val : add_mod(sum[gi], val, q);
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) {
          if constexpr (PAIR)
            mbar_arrive_cluster(acc_empty0 + (uint32_t)buf * 8u);
          else
            mbar_arrive(&acc_empty[buf]);
        }
      }
      if (!alive) break;
      // the tile's results, once
#pragma unroll
      for (int gi = 0; gi < 2; ++gi) {
        const int grp = part + 2 * gi;
        if (grp >= groups) break;
        const int bq = (int)hf * G.nbh + grp * 8 + t8;  // query polynomial in the pass
        const int b = bq >> 1;
        if (b < G.batch)
          out[(size_t)(b_base + b) * out_stride + (row * 2 + (bq & 1)) * kN + c] = sum[gi];
      }
    }
    if (!range_ok) report_error(status, kErrTcRange);
  }
  tc_fence_before();
  if constexpr (PAIR)
    cluster_sync_all();  // the pair's copies, MMAs and epilogues are done
  else
    __syncthreads();
  if (warp == kTcMma) {
    tc_fence_after();
    if constexpr (PAIR)
      asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                   "r"(kTcTmemCols)
                   : "memory");
    else
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                   "r"(kTcTmemCols)
                   : "memory");
  }
}

// balanced 8-bit limbs of a residue < 2^60, as bf16 bit patterns
__device__ __forceinline__ void limbs8(uint64_t v, uint16_t (&d)[8]) {
  int carry = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    int x = (int)(v & 255u) + carry;
    v >>= 8;
    carry = x >= 128;
    x -= carry << 8;
    d[i] = __bfloat16_as_ushort(__float2bfloat16_rn((float)x));
  }
}

// balanced 9-bit limbs of a residue < 2^60 (the top one in [0, 64]), as bf16
// bit patterns; every |limb| <= 256 is exact in bf16
__device__ __forceinline__ void limbs9(uint64_t v, uint16_t (&d)[7]) {
  int carry = 0;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    int x = (int)(v & 511u) + carry;
    v >>= 9;
    carry = x >= 256;
    x -= carry << 9;
    d[i] = __bfloat16_as_ushort(__float2bfloat16_rn((float)x));
  }
  d[6] = __bfloat16_as_ushort(__float2bfloat16_rn((float)((int)v + carry)));
}
template <int QL>
__device__ __forceinline__ void query_limbs(uint64_t v, uint16_t (&d)[QL]) {
  if constexpr (QL == 8)
    limbs8(v, d);
  else
    limbs9(v, d);
}

// one thread: 8 consecutive k of one (slot, row) -> one 128-byte core matrix
__global__ void db_limb_kernel(const uint64_t *__restrict__ dbs, uint16_t *__restrict__ dbl,
                               int n1, int n_rest) {
  const int kblk = n1 / 8, n_rb = n_rest / kTcRows;
  const long long total = (long long)kN * n_rb * kblk * kTcRows;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int r16 = (int)(t % kTcRows);
    long long rest = t / kTcRows;
    const int kb = (int)(rest % kblk);
    rest /= kblk;
    const int rb = (int)(rest % n_rb);
    const long long c = rest / n_rb;
    const uint64_t *src = dbs + (size_t)c * n1 * n_rest + (size_t)kb * 8 * n_rest +
                          (size_t)rb * kTcRows + r16;
    uint16_t d[8][8];  // [kk][limb]
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
      const uint64_t w = src[(size_t)kk * n_rest];
      limbs8((w & 0x3FFFFFFFull) + ((w >> 32) << 30), d[kk]);
    }
    uint4 *dst = reinterpret_cast<uint4 *>(dbl + (size_t)t * 64);
#pragma unroll
    for (int i = 0; i < 8; ++i)
      dst[i] = make_uint4(d[0][i] | (uint32_t)d[1][i] << 16, d[2][i] | (uint32_t)d[3][i] << 16,
                          d[4][i] | (uint32_t)d[5][i] << 16, d[6][i] | (uint32_t)d[7][i] << 16);
  }
}

// one thread: 8 consecutive k of one (slot, query polynomial) of the pass,
// from plane[b][k][poly][c] (consecutive threads read consecutive slots) to
// ql[c][h][k/8][b' - nbh h][j][k%8] (h: a block of nbh polynomials, half of
// a pass's columns, or a quarter for CTA pairs, which load half a column
// block each).  A warp covers 8 slots x 4 query
// polynomials: its output is 8 runs of QL x 64 bytes, which it writes
// through a shared-memory transpose so that every store instruction fills
// one run.
template <int QL>
__global__ void __launch_bounds__(256) query_limb_kernel(const uint64_t *__restrict__ plane,
                                                         uint16_t *__restrict__ ql, int n1,
                                                         int b_base, int nh, int nbh,
                                                         int pass_batch) {
  __shared__ uint4 stage[8][8 * 4 * QL];  // [warp][slot][polynomial][limb]
  const int kblk = n1 / 8;
  const long long total = (long long)kN * nh * kblk * nbh;  // a multiple of 32
  uint4 *st = stage[threadIdx.x >> 5];
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int lane = (int)(t & 31);
    long long rest = t >> 5;
    const int c0 = (int)(rest % (kN / 8)) * 8;
    const int c = c0 + (lane & 7);
    rest /= kN / 8;
    const int bl0 = (int)(rest % (nbh / 4)) * 4;
    const int bl = bl0 + (lane >> 3);
    rest /= nbh / 4;
    const int kb = (int)(rest % kblk);
    const int hf = (int)(rest / kblk);
    const int bq = hf * nbh + bl;
    const int b = bq >> 1;
    uint16_t d[8][QL];
    const uint64_t *src =
        plane + (((size_t)(b_base + b) * n1 + kb * 8) * 2 + (bq & 1)) * kN + c;
#pragma unroll
    for (int kk = 0; kk < 8; ++kk)
      query_limbs<QL>(b < pass_batch ? src[(size_t)kk * 2 * kN] : 0, d[kk]);
    __syncwarp();  // the previous iteration's reads of the staging buffer are done
#pragma unroll
    for (int i = 0; i < QL; ++i)
      st[((lane & 7) * 4 + (lane >> 3)) * QL + i] =
          make_uint4(d[0][i] | (uint32_t)d[1][i] << 16, d[2][i] | (uint32_t)d[3][i] << 16,
                     d[4][i] | (uint32_t)d[5][i] << 16, d[6][i] | (uint32_t)d[7][i] << 16);
    __syncwarp();
#pragma unroll
    for (int cs = 0; cs < 8; ++cs) {
      uint4 *dst = reinterpret_cast<uint4 *>(
          ql + ((((size_t)(c0 + cs) * nh + hf) * kblk + kb) * nbh + bl0) * (QL * 8));
      // polynomial bl0 + lane / QL, limb lane % QL
      if (lane < 4 * QL) dst[lane] = st[cs * 4 * QL + lane];
    }
  }
}

template <int KC, int STAGES, bool PAIR>
constexpr size_t tc_smem() {
  return STAGES * tc_stage_bytes<KC, PAIR>() + kTcEpiWarps * 4 * kTcYStride * sizeof(int) +
         (2 * STAGES + 6) * 8;
}
static_assert(tc_smem<64, tc_stages<64, false>(), false>() <= 227 * 1024, "shared memory per CTA");
static_assert(tc_smem<32, tc_stages<32, false>(), false>() <= 227 * 1024, "shared memory per CTA");
static_assert(tc_smem<64, tc_stages<64, true>(), true>() <= 227 * 1024, "shared memory per CTA");
static_assert(tc_smem<32, tc_stages<32, true>(), true>() <= 227 * 1024, "shared memory per CTA");
// an MMA operand read of a full query tile from the last stage of a pair's
// ring would still end inside the staging that follows it
static_assert(kTcEpiWarps * 4 * kTcYStride * sizeof(int) >= 64 / 8 * kTcHalfNB / 2 * 128,
              "staging after the ring");

int g_tc_sms = 0;

uint32_t make_idesc(int n, int m) {
  // D f32 (bits 4-5 = 1), A and B bf16 (bits 7-9, 10-12 = 1), both K-major,
  // N >> 3 at bits 17-22, M >> 4 at bits 24-28 (M = 128, or 256 for a CTA pair)
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

}  // namespace

bool tc_scan_supported(int n1, int n_rest) {
  return n1 % kTcKC == 0 && n1 > 0 && n_rest % kTcRows == 0 && n_rest >= kTcRows;
}

size_t tc_db_limb_bytes(int n1, int n_rest) { return (size_t)kN * n1 * n_rest * 16; }
namespace {
int g_tc_limbs = -1;  // OPIR_TC_LIMBS: force the query limb width (tests, sweeps)

// query polynomials per column block of a pass of pb queries with ql limbs:
// 8-polynomial epilogue groups, N = ql nbh a multiple of 16; above 16
// queries, blocks of 32 polynomials (16 queries), up to four per pass -- a
// pass of 64 queries streams each database tile once from DRAM and three
// times from L2, where two passes of 32 would stream it twice from DRAM
int pass_nbh(int pb, int ql, int *nh) {
  if (pb > kTcHalfNB / 2) {
    *nh = (pb + kTcHalfNB / 2 - 1) / (kTcHalfNB / 2);
    return kTcHalfNB;
  }
  const int gran = ql == 7 ? 8 : 4;
  *nh = 1;
  return 2 * ((pb + gran - 1) / gran * gran);
}
// limbs per query residue of a pass: the forced or requested width, else the
// one with fewer MMA columns (ties: 9-bit)
int pass_ql(int pb, int limbs) {
  if (g_tc_limbs >= 0) limbs = g_tc_limbs;
  if (limbs == kTcLimbs8) return 8;
  if (limbs == kTcLimbs9) return 7;
  int h8, h9;
  const int n8 = pass_nbh(pb, 8, &h8) * 8 * h8, n9 = pass_nbh(pb, 7, &h9) * 7 * h9;
  return n9 <= n8 ? 7 : 8;
}
int g_tc_pair = -1;  // OPIR_TC_PAIR: force the one-CTA (0) or CTA-pair (1) form

// Geometry of the pass of `pb` queries with ql limbs per query residue, in
// the one-CTA or the CTA-pair form.
TcGeom pass_geom(int n1, int n_rest, int pb, int ql, bool pair = false) {
  TcGeom G;
  G.n1 = n1;
  G.n_rest = n_rest;
  G.batch = pb;
  G.ql = ql;
  G.nbh = pass_nbh(pb, ql, &G.nh);
  G.n_rb = n_rest / kTcRows;
  G.pair = pair;
  G.units = (long long)kN * (pair ? G.n_rb / 2 : G.n_rb) * G.nh;
  G.nseg = (n1 + kTcMaxSegment - 1) / kTcMaxSegment;
  G.b_bytes = 0;  // per stage: set by the launcher for its stage size
  G.idesc = make_idesc(G.nbh * ql, pair ? 256 : 128);
  return G;
}
// query limbs of one pass (elements; the same in both forms); passes follow
// each other in ql
size_t pass_limb_elems(int n1, int pb, int ql) {
  const TcGeom G = pass_geom(n1, kTcRows, pb, ql);
  return (size_t)kN * G.nh * (n1 / 8) * G.nbh * ql * 8;
}
// The form of a pass: the forced or requested one where it applies (a pair
// needs an even number of row tiles, a B half of whole core matrices and
// N >= 32); without a request, one CTA per tile.  Pairs halve the bytes
// each SM streams per MMA, but the second CTA's copies complete on the first
// CTA's barriers about 2.7 us after issue (1.3 us within one CTA), and the
// six 32 KB stages that fit cannot hide that at 0.3 us of MMA per stage:
// 3.56 ms against 3.0 ms for 32 queries on 512 x 512, so the autotuner
// keeps pairs only where they measure faster.
bool pass_pair(int n_rest, int pb, int ql, int pair) {
  if (g_tc_pair >= 0) pair = g_tc_pair;
  int nh;
  const int nbh = pass_nbh(pb, ql, &nh);
  const bool ok = (n_rest / kTcRows) % 2 == 0 && (nbh / 2) % 4 == 0 && (nbh / 2 * ql) % 8 == 0 &&
                  nbh * ql >= 32;
  return ok && pair == 1;
}
}  // namespace

size_t tc_query_limb_bytes(int n1, int batch) {
  size_t e8 = 0, e9 = 0;
  for (int b0 = 0; b0 < batch; b0 += pass_max()) {
    const int pb = batch - b0 < pass_max() ? batch - b0 : pass_max();
    e8 += pass_limb_elems(n1, pb, 8);
    e9 += pass_limb_elems(n1, pb, 7);
  }
  return (e8 > e9 ? e8 : e9) * sizeof(uint16_t);
}

int tc_pass_count(int batch) { return (batch + pass_max() - 1) / pass_max(); }

int tc_query_limb_width(int batch, int limbs) {
  return pass_ql(batch < pass_max() ? batch : pass_max(), limbs) == 7 ? 9 : 8;
}

namespace {
template <int KC, int QL, bool PAIR>
cudaError_t set_tc_smem() {
  constexpr int S = tc_stages<KC, PAIR>();
  return cudaFuncSetAttribute(tc_scan_kernel<KC, S, QL, PAIR>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)tc_smem<KC, S, PAIR>());
}
}  // namespace

cudaError_t init_tc_attributes() {
  g_tc_ring = -1;
  if (const char *v = getenv("OPIR_TC_RING")) g_tc_ring = atoi(v);
  g_tc_limbs = -1;
  if (const char *v = getenv("OPIR_TC_LIMBS")) g_tc_limbs = atoi(v);
  g_tc_pair = -1;
  if (const char *v = getenv("OPIR_TC_PAIR")) g_tc_pair = atoi(v);
  g_tc_pass = kTcMaxNB / 2;
  if (const char *v = getenv("OPIR_TC_PASS")) {
    const int q = atoi(v);
    if (q >= 16 && q <= kTcMaxNB / 2 && q % 16 == 0) g_tc_pass = q;
  }
  int dev;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&g_tc_sms, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e = set_tc_smem<64, 8, false>();
  if (e == cudaSuccess) e = set_tc_smem<32, 8, false>();
  if (e == cudaSuccess) e = set_tc_smem<64, 7, false>();
  if (e == cudaSuccess) e = set_tc_smem<32, 7, false>();
  if (e == cudaSuccess) e = set_tc_smem<64, 8, true>();
  if (e == cudaSuccess) e = set_tc_smem<32, 8, true>();
  if (e == cudaSuccess) e = set_tc_smem<64, 7, true>();
  if (e == cudaSuccess) e = set_tc_smem<32, 7, true>();
  return e;
}

void launch_db_limbs(const uint64_t *dbs, uint16_t *dbl, int n1, int n_rest, cudaStream_t s) {
  const long long total = (long long)kN * (n_rest / kTcRows) * (n1 / 8) * kTcRows;
  const long long blocks = (total + 255) / 256;
  db_limb_kernel<<<(unsigned)(blocks < 65536 ? blocks : 65536), 256, 0, s>>>(dbs, dbl, n1, n_rest);
}

void launch_tc_query_limbs(const uint64_t *plane, uint16_t *ql, int n1, int n_rest, int batch,
                           cudaStream_t s, int limbs, int pair) {
  size_t off = 0;
  for (int b0 = 0; b0 < batch; b0 += pass_max()) {
    const int pb = batch - b0 < pass_max() ? batch - b0 : pass_max();
    const int qlc = pass_ql(pb, limbs);
    const TcGeom G = pass_geom(n1, kTcRows, pb, qlc);
    // a pair's CTAs each load half of a column block: blocks of nbh / 2
    const bool pr = pass_pair(n_rest, pb, qlc, pair);
    const int nh = pr ? 2 * G.nh : G.nh, nbh = pr ? G.nbh / 2 : G.nbh;
    const long long qtotal = (long long)kN * nh * (n1 / 8) * nbh;
    const long long qblocks = (qtotal + 255) / 256;
    const unsigned grid = (unsigned)(qblocks < 65536 ? qblocks : 65536);
    if (qlc == 7)
      query_limb_kernel<7><<<grid, 256, 0, s>>>(plane, ql + off, n1, b0, nh, nbh, pb);
    else
      query_limb_kernel<8><<<grid, 256, 0, s>>>(plane, ql + off, n1, b0, nh, nbh, pb);
    off += pass_limb_elems(n1, pb, qlc);
  }
}

bool tc_ring_valid(int ring, int n1) { return ring == kTcRing32x8 || (ring == kTcRing64x4 && n1 % 64 == 0); }

namespace {
// A [rows][64 x u16] (128-byte rows) view of `bytes` of a pre-tiled limb
// plane with boxes of box_rows rows: the tensor copies of a CTA pair's
// second CTA.  cuTensorMapEncodeTiled comes from the driver entry point.
bool make_row_map(CUtensorMap *m, const void *base, size_t bytes, uint32_t box_rows) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult qr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &qr) != cudaSuccess ||
        qr != cudaDriverEntryPointSuccess || !fn)
      return false;
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  const cuuint64_t dims[2] = {64, (cuuint64_t)(bytes / 128)};
  const cuuint64_t strides[1] = {128};
  const cuuint32_t box[2] = {64, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return encode(m, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<void *>(base), dims, strides, box,
                estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int KC, int QL, bool PAIR>
bool launch_tc_pass(TcGeom G, const uint16_t *dbl, const uint16_t *ql, uint64_t *out,
                    size_t out_stride, int b0, uint64_t q, uint64_t mu_lo, uint64_t mu_hi,
                    uint64_t r64, uint64_t r128, uint32_t *status, cudaStream_t s) {
  constexpr int S = tc_stages<KC, PAIR>();
  const int sms = g_tc_sms > 0 ? g_tc_sms : 152;
  G.b_bytes = (uint32_t)(KC / 8 * (PAIR ? G.nbh / 2 : G.nbh) * QL * 16);
  CUtensorMap tm_a, tm_b;
  std::memset(&tm_a, 0, sizeof tm_a);
  std::memset(&tm_b, 0, sizeof tm_b);
  if constexpr (PAIR) {
    const size_t a_bytes = (size_t)kN * G.n1 * G.n_rest * 16;
    const size_t b_bytes = (size_t)kN * G.nh * (G.n1 / 8) * G.nbh * QL * 16;
    if (!make_row_map(&tm_a, dbl, a_bytes, tc_a_bytes<KC>() / 128) ||
        !make_row_map(&tm_b, ql, b_bytes, G.b_bytes / 128))
      return false;
    // one pair per two SMs, each pair a two-CTA cluster
    const long long pairs = G.units < sms / 2 ? G.units : sms / 2;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(2 * pairs));
    cfg.blockDim = dim3(kTcThreads);
    cfg.dynamicSmemBytes = tc_smem<KC, S, PAIR>();
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, tc_scan_kernel<KC, S, QL, PAIR>, dbl, ql, out, out_stride, b0, G, q,
                       mu_lo, mu_hi, r64, r128, status, tm_a, tm_b);
  } else {
    const long long grid = G.units < sms ? G.units : sms;
    tc_scan_kernel<KC, S, QL, PAIR><<<(unsigned)grid, kTcThreads, tc_smem<KC, S, PAIR>(), s>>>(
        dbl, ql, out, out_stride, b0, G, q, mu_lo, mu_hi, r64, r128, status, tm_a, tm_b);
  }
  return true;
}
template <int KC, bool PAIR>
bool launch_tc_ql(const TcGeom &G, const uint16_t *dbl, const uint16_t *ql, uint64_t *out,
                  size_t out_stride, int b0, uint64_t q, uint64_t mu_lo, uint64_t mu_hi,
                  uint64_t r64, uint64_t r128, uint32_t *status, cudaStream_t s) {
  if (G.ql == 7)
    return launch_tc_pass<KC, 7, PAIR>(G, dbl, ql, out, out_stride, b0, q, mu_lo, mu_hi, r64,
                                       r128, status, s);
  return launch_tc_pass<KC, 8, PAIR>(G, dbl, ql, out, out_stride, b0, q, mu_lo, mu_hi, r64, r128,
                                     status, s);
}
}  // namespace

int launch_tc_scan(const uint16_t *dbl, const uint16_t *ql, uint64_t *out, size_t out_stride,
                   int n1, int n_rest, int batch, uint64_t q, uint64_t mu_lo, uint64_t mu_hi,
                   uint64_t r64, uint64_t r128, uint32_t *status, cudaStream_t s, int ring,
                   int limbs, int pair) {
  if (g_tc_ring >= 0) ring = g_tc_ring;
  // every segment length is a multiple of 64 when n1 is (segments of 512)
  if (!tc_ring_valid(ring, n1)) ring = n1 % 64 == 0 ? kTcRing64x4 : kTcRing32x8;
  int launches = 0;
  size_t off = 0;
  for (int b0 = 0; b0 < batch; b0 += pass_max()) {
    const int pb = batch - b0 < pass_max() ? batch - b0 : pass_max();
    const int qlc = pass_ql(pb, limbs);
    const bool pr = pass_pair(n_rest, pb, qlc, pair);
    const TcGeom G = pass_geom(n1, n_rest, pb, qlc, pr);
    const uint16_t *qp = ql + off;
    bool ok;
    if (ring == kTcRing64x4)
      ok = pr ? launch_tc_ql<64, true>(G, dbl, qp, out, out_stride, b0, q, mu_lo, mu_hi, r64,
                                       r128, status, s)
              : launch_tc_ql<64, false>(G, dbl, qp, out, out_stride, b0, q, mu_lo, mu_hi, r64,
                                        r128, status, s);
    else
      ok = pr ? launch_tc_ql<32, true>(G, dbl, qp, out, out_stride, b0, q, mu_lo, mu_hi, r64,
                                       r128, status, s)
              : launch_tc_ql<32, false>(G, dbl, qp, out, out_stride, b0, q, mu_lo, mu_hi, r64,
                                        r128, status, s);
    if (!ok) return -1;
    launches++;
    off += pass_limb_elems(n1, pb, qlc);
  }
  return launches;
}

bool tc_pair_form(int n_rest, int batch, int limbs, int pair) {
  const int pb = batch < pass_max() ? batch : pass_max();
  return pass_pair(n_rest, pb, pass_ql(pb, limbs), pair);
}

}  // namespace opir
