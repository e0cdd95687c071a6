// scan.cu -- first-dimension database x query product on sm_103a.
//
// Restates naive_level_mat_mat_128 / mat_mat_128 (matrix.cpp:79-97,220-235)
// and delay_modulus's reduction (server.cpp:178-243): for every NTT slot c,
//   out[row][poly][c] = sum_k DB[c][k][row] * Q[c][k][poly]  mod q,
// summed exactly (the reference sums in a wrapping uint128; for the shipped
// shapes its sums never wrap, so the results agree bit for bit).
//
// The database lives in HBM as dbs[c][k][row], each 60-bit residue stored as
// lo30 | hi30 << 32, so one 8-byte load yields both 30-bit halves.  Products
// are formed from 30x30-bit halves (IMAD.WIDE.U32), accumulated in 64-bit
// partial sums and folded into 128-bit totals every 8 k-steps.
//
// scan_bulk_kernel (the production path) is a persistent, warp-specialised
// kernel: one producer warp streams [k-block][rows] tiles of the database and
// the matching query words into a ring of shared-memory stages with
// cp.async.bulk (completion on mbarriers); eight consumer warps multiply out
// of shared memory.  All waits are bounded (async.cuh).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>

#include "async.cuh"
#include "common.cuh"
#include "kernels.h"

namespace opir {

namespace {

// acc += x * y, 32x32 -> 64 (IMAD.WIDE.U32).  Two spellings: ptxas fuses the
// 64-bit add into the multiply differently depending on the context, so the
// kernels pick the one measured faster.
__device__ __forceinline__ void mad_wide(uint64_t &acc, uint32_t x, uint32_t y) {
  asm("mad.wide.u32 %0, %1, %2, %0;" : "+l"(acc) : "r"(x), "r"(y));
}
__device__ __forceinline__ void mad_wide_c(uint64_t &acc, uint32_t x, uint32_t y) {
  acc += (uint64_t)x * y;
}
// acc += x * y as two 32-bit multiply-adds chained through the carry flag
__device__ __forceinline__ void mad_cc(uint64_t &acc, uint32_t x, uint32_t y) {
  uint32_t lo = (uint32_t)acc, hi = (uint32_t)(acc >> 32);
  asm("mad.lo.cc.u32 %0, %2, %3, %0;\n\tmadc.hi.u32 %1, %2, %3, %1;"
      : "+r"(lo), "+r"(hi)
      : "r"(x), "r"(y));
  acc = ((uint64_t)hi << 32) | lo;
}
struct Acc3 {
  uint64_t ll, mid, hh;
  U128 LL, MID, HH;
};

__device__ __forceinline__ void acc3_zero(Acc3 &a) {
  a.ll = a.mid = a.hh = 0;
  a.LL = a.MID = a.HH = U128{0, 0};
}
// a = a1 2^30 + a0, b = b1 2^30 + b0 (all halves < 2^30):
// a b = a0 b0 + (a0 b1 + a1 b0) 2^30 + a1 b1 2^60.  Each half product is
// < 2^60, so the 64-bit partials absorb 16, 8 and 16 k-steps.
template <int kForm>
__device__ __forceinline__ void madw(uint64_t &acc, uint32_t x, uint32_t y) {
  if constexpr (kForm == 1)
    mad_wide(acc, x, y);
  else if constexpr (kForm == 3)
    mad_cc(acc, x, y);
  else
    mad_wide_c(acc, x, y);
}
__device__ __forceinline__ void acc3_mac(Acc3 &a, uint32_t a0, uint32_t a1, uint32_t b0,
                                         uint32_t b1) {
  mad_cc(a.ll, a0, b0);
  mad_cc(a.mid, a0, b1);
  mad_cc(a.mid, a1, b0);
  mad_cc(a.hh, a1, b1);
}
__device__ __forceinline__ void acc3_flush(Acc3 &a) {
  add_to(a.LL, U128{a.ll, 0});
  add_to(a.MID, U128{a.mid, 0});
  add_to(a.HH, U128{a.hh, 0});
  a.ll = a.mid = a.hh = 0;
}
// the middle partial takes two products per step: flush it every 8 steps,
// the outer two every 16
__device__ __forceinline__ void acc3_flush_mid(Acc3 &a) {
  add_to(a.MID, U128{a.mid, 0});
  a.mid = 0;
}
// Karatsuba form of the same sums: `mid` takes (a0 + a1)(b0 + b1) (< 2^62,
// so it is flushed every 4 k-steps) and the cross terms are recovered at the
// end as MID - LL - HH (exact, >= 0): three products per step instead of four.
__device__ __forceinline__ void acc3_mac_k(Acc3 &a, uint32_t a0, uint32_t a1, uint32_t sa,
                                           uint32_t b0, uint32_t b1, uint32_t sb) {
  mad_cc(a.ll, a0, b0);
  mad_cc(a.mid, sa, sb);
  mad_cc(a.hh, a1, b1);
}
__device__ __forceinline__ void acc3_unkaratsuba(Acc3 &a) {
  asm("sub.cc.u64 %0, %0, %2;\n\tsubc.u64 %1, %1, %3;"
      : "+l"(a.MID.lo), "+l"(a.MID.hi)
      : "l"(a.LL.lo), "l"(a.LL.hi));
  asm("sub.cc.u64 %0, %0, %2;\n\tsubc.u64 %1, %1, %3;"
      : "+l"(a.MID.lo), "+l"(a.MID.hi)
      : "l"(a.HH.lo), "l"(a.HH.hi));
}
// the reduction constants of one modulus (a second one rides in ScanGeom)
struct ScanMod {
  uint64_t q, two30, two30_s, two60, two60_s, mu_lo, mu_hi;
};
__device__ __forceinline__ uint64_t acc3_reduce(Acc3 &a, const ScanMod &m, bool karatsuba) {
  acc3_flush(a);
  if (karatsuba) acc3_unkaratsuba(a);
  const uint64_t q = m.q;
  const uint64_t rl = barrett128(a.LL, q, m.mu_lo, m.mu_hi);
  const uint64_t rm = barrett128(a.MID, q, m.mu_lo, m.mu_hi);
  const uint64_t rh = barrett128(a.HH, q, m.mu_lo, m.mu_hi);
  uint64_t r = add_mod(rl, mul_shoup(rm, m.two30, m.two30_s, q), q);
  return add_mod(r, mul_shoup(rh, m.two60, m.two60_s, q), q);
}
__device__ __forceinline__ uint64_t acc3_reduce(Acc3 &a, const Consts &C, uint64_t mu_lo,
                                                uint64_t mu_hi, bool karatsuba = false) {
  return acc3_reduce(a, ScanMod{C.q, C.two30, C.two30_s, C.two60, C.two60_s, mu_lo, mu_hi},
                     karatsuba);
}

// ---------------------------------------------------------------------------
// generic kernel (any shape): thread owns R rows of one plane, loads straight
// from global memory
// ---------------------------------------------------------------------------
template <int R>
__global__ void __launch_bounds__(256) scan_kernel(const uint64_t *__restrict__ dbs,
                                                   const uint4 *__restrict__ qs,
                                                   size_t qs_stride, uint64_t *out,
                                                   size_t out_stride, int n1, int n_rest,
                                                   Consts C, uint64_t mu_lo, uint64_t mu_hi) {
  const int b = blockIdx.y;
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int groups = n_rest / R;
  const size_t c = g / groups;
  if (c >= (size_t)kN) return;
  const int row0 = (int)(g % groups) * R;
  const uint64_t *plane = dbs + c * (size_t)n1 * n_rest + row0;
  const uint4 *qv = qs + b * qs_stride + c * (size_t)n1;

  Acc3 acc[R][2];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    acc3_zero(acc[r][0]);
    acc3_zero(acc[r][1]);
  }
  constexpr int U = 8;
  int k = 0;
  for (; k + U <= n1; k += U) {
    uint64_t a[U][R];
    uint4 bq[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint64_t *src = plane + (size_t)(k + u) * n_rest;
      if constexpr (R == 2) {
        const ulonglong2 v = __ldcs(reinterpret_cast<const ulonglong2 *>(src));
        a[u][0] = v.x;
        a[u][R - 1] = v.y;
      } else {
        a[u][0] = __ldcs(src);
      }
      bq[u] = __ldg(qv + k + u);
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const uint32_t a0 = (uint32_t)a[u][r], a1 = (uint32_t)(a[u][r] >> 32);
        acc3_mac(acc[r][0], a0, a1, bq[u].x, bq[u].y);
        acc3_mac(acc[r][1], a0, a1, bq[u].z, bq[u].w);
      }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      acc3_flush(acc[r][0]);
      acc3_flush(acc[r][1]);
    }
  }
  for (; k < n1; ++k) {
    const uint64_t *src = plane + (size_t)k * n_rest;
    const uint4 bq = __ldg(qv + k);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const uint64_t av = src[r];
      const uint32_t a0 = (uint32_t)av, a1 = (uint32_t)(av >> 32);
      acc3_mac(acc[r][0], a0, a1, bq.x, bq.y);
      acc3_mac(acc[r][1], a0, a1, bq.z, bq.w);
    }
  }
  uint64_t *o = out + b * out_stride;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const size_t row = (size_t)row0 + r;
    o[row * 2 * kN + c] = acc3_reduce(acc[r][0], C, mu_lo, mu_hi);
    o[row * 2 * kN + kN + c] = acc3_reduce(acc[r][1], C, mu_lo, mu_hi);
  }
}

// ---------------------------------------------------------------------------
// bulk-copy pipelined kernel
// ---------------------------------------------------------------------------

struct ScanGeom {
  int n1, n_rest;
  int rt;       // rows of a plane per tile  (min(n_rest, 512))
  int pc;       // planes per tile           (512 / rt)
  int row_tiles;  // n_rest / rt
  int nkb;      // n1 / kStepK
  long long items;  // batch * (planes / pc) * row_tiles
  int q_bytes;      // pc * kStepK * 16
  int planes;       // NTT slots (kN; R N for the multi-modulus path)
  size_t o_row, o_poly;  // output strides of a row and of the second polynomial
  int mod_planes;   // slots of the first modulus; the rest reduce mod m1
  ScanMod m1;
};

// kRows rows per consumer thread, kWarps consumer warps (kRows * kWarps * 32
// == 512), kStepK k-steps per stage, kStages stages, kMinBlocks CTAs per SM;
// kKara: Karatsuba products (acc3_mac_k).
template <int kRows, int kWarps, int kStepK, int kStages, int kMinBlocks, int kKara,
          bool kTwoMods = false>
__global__ void __launch_bounds__(kWarps * 32 + 32, kMinBlocks)
    scan_bulk_kernel(const uint64_t *__restrict__ dbs, const uint4 *__restrict__ qs,
                     size_t qs_stride, uint64_t *out, size_t out_stride, ScanGeom G, Consts C,
                     uint64_t mu_lo, uint64_t mu_hi, uint32_t *status) {
  constexpr int kTileRows = kRows * kWarps * 32;  // rows (of one or more planes) per tile
  static_assert(kStepK == 1 || kStepK == 2 || kStepK == 4 || kStepK == 8 || kStepK % 16 == 0,
                "flush cadence: middle partial every 8 k-steps, outer ones every 16");
  static_assert(!kKara || kStepK % 16 == 0, "Karatsuba form: middle partial every 4 k-steps");
  constexpr int kStageDbBytes = kStepK * kTileRows * 8;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int stage_bytes = kStageDbBytes + G.q_bytes;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw + kStages * stage_bytes);
  uint64_t *full = bars, *empty = bars + kStages;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kWarps);
    }
    mbar_fence_init();
  }
  __syncthreads();

  const size_t plane_words = (size_t)G.n1 * G.n_rest;
  const long long per_b = (long long)(G.planes / G.pc) * G.row_tiles;
  // test hook (async.cuh): CTA 0 withholds its first stage, and its waits
  // for stages give up after `limit` polls; the drain below keeps the
  // production limit, since every copy it waits for was issued
  const uint32_t hook = status ? status[1] : 0u;
  const bool withhold = hook != 0 && blockIdx.x == 0;
  const uint32_t limit = withhold ? hook : kSpinLimit;

  if (warp == kWarps) {
    // ------------------------------ producer ------------------------------
    long long it = 0;
    int ps = 0;           // stage to fill next
    uint32_t pphase = 0;  // round parity of that stage
    bool ok = true;
    for (long long item = blockIdx.x; item < G.items && ok; item += gridDim.x) {
      const int b = (int)(item / per_b);
      const long long rem = item % per_b;
      const int g = (int)(rem / G.row_tiles), rt = (int)(rem % G.row_tiles);
      const int c0 = g * G.pc;
      for (int kb = 0; kb < G.nkb; ++kb, ++it) {
        const int s = ps;
        const bool reuse = it >= kStages;
        const uint32_t ephase = pphase ^ 1u;  // phase of the consumers' release of the last use
        if (++ps == kStages) {
          ps = 0;
          pphase ^= 1u;
        }
        if (reuse) {
          bool w = true;
          if (lane == 0) w = mbar_wait(&empty[s], ephase, limit);
          w = __shfl_sync(0xffffffffu, w, 0);
          if (!w) {
            if (lane == 0) report_error(status, kErrWaitEmpty);
            ok = false;
            break;
          }
        }
        if (withhold && it == 0) continue;  // stage 0 never arrives (test hook)
        unsigned char *st = smem_raw + (size_t)s * stage_bytes;
        uint64_t *sdb = reinterpret_cast<uint64_t *>(st);
        uint4 *sq = reinterpret_cast<uint4 *>(st + kStageDbBytes);
        if (lane == 0) mbar_arrive_expect_tx(&full[s], (uint32_t)stage_bytes);
        __syncwarp();
        const int k0 = kb * kStepK;
        if (G.rt == G.n_rest) {
          // one contiguous [k-block][rows] run per plane
          for (int p = lane; p < G.pc; p += 32) {
            const uint64_t *src = dbs + (size_t)(c0 + p) * plane_words + (size_t)k0 * G.n_rest;
            bulk_g2s(sdb + (size_t)p * kStepK * G.rt, src, kStepK * G.rt * 8, &full[s]);
          }
        } else {
          // one plane, a row tile of it: one run per k
          for (int k = lane; k < kStepK; k += 32) {
            const uint64_t *src = dbs + (size_t)c0 * plane_words + (size_t)(k0 + k) * G.n_rest +
                                  (size_t)rt * G.rt;
            bulk_g2s(sdb + (size_t)k * G.rt, src, G.rt * 8, &full[s]);
          }
        }
        for (int p = lane; p < G.pc; p += 32) {
          const uint4 *src = qs + b * qs_stride + (size_t)(c0 + p) * G.n1 + k0;
          bulk_g2s(sq + p * kStepK, src, kStepK * 16, &full[s]);
        }
      }
    }
    // drain: never leave the CTA with copies still landing in its shared memory
    if (lane == 0) {
      const long long first = it > kStages ? it - kStages : 0;
      for (long long j = first; j < it; ++j) {
        if (withhold && j == 0) continue;  // issued nothing
        if (!mbar_wait(&full[j % kStages], (uint32_t)((j / kStages) & 1))) {
          report_error(status, kErrDrain);
          break;
        }
      }
    }
    return;
  }

  // ------------------------------ consumers ------------------------------
  const int slot = kRows * threadIdx.x;
  const int p = slot / G.rt, r = slot % G.rt;
  int s = 0;
  uint32_t phase = 0;
  for (long long item = blockIdx.x; item < G.items; item += gridDim.x) {
    const int b = (int)(item / per_b);
    const long long rem = item % per_b;
    const int g = (int)(rem / G.row_tiles), rt = (int)(rem % G.row_tiles);
    Acc3 acc[kRows][2];
#pragma unroll
    for (int rr = 0; rr < kRows; ++rr) {
      acc3_zero(acc[rr][0]);
      acc3_zero(acc[rr][1]);
    }
    for (int kb = 0; kb < G.nkb; ++kb) {
      if (!mbar_wait_sleep(&full[s], phase, limit)) {
        report_error(status, kErrWaitFull);
        return;
      }
      const unsigned char *st = smem_raw + (size_t)s * stage_bytes;
      const uint64_t *sdb = reinterpret_cast<const uint64_t *>(st) + (size_t)p * kStepK * G.rt + r;
      const uint4 *sq = reinterpret_cast<const uint4 *>(st + kStageDbBytes) + p * kStepK;
#pragma unroll
      for (int k = 0; k < kStepK; ++k) {
        uint64_t a[kRows];
        if constexpr (kRows == 2) {
          const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(sdb + (size_t)k * G.rt);
          a[0] = v.x;
          a[kRows - 1] = v.y;
        } else {
          a[0] = sdb[(size_t)k * G.rt];
        }
        const uint4 bq = sq[k];
        if constexpr (kKara) {
          const uint32_t sb0 = bq.x + bq.y, sb1 = bq.z + bq.w;
#pragma unroll
          for (int rr = 0; rr < kRows; ++rr) {
            const uint32_t a0 = (uint32_t)a[rr], a1 = (uint32_t)(a[rr] >> 32);
            const uint32_t sa = a0 + a1;
            acc3_mac_k(acc[rr][0], a0, a1, sa, bq.x, bq.y, sb0);
            acc3_mac_k(acc[rr][1], a0, a1, sa, bq.z, bq.w, sb1);
          }
          if ((k & 15) == 15) {
#pragma unroll
            for (int rr = 0; rr < kRows; ++rr) {
              acc3_flush(acc[rr][0]);
              acc3_flush(acc[rr][1]);
            }
          } else if ((k & 3) == 3) {
#pragma unroll
            for (int rr = 0; rr < kRows; ++rr) {
              acc3_flush_mid(acc[rr][0]);
              acc3_flush_mid(acc[rr][1]);
            }
          }
          continue;
        }
#pragma unroll
        for (int rr = 0; rr < kRows; ++rr) {
          const uint32_t a0 = (uint32_t)a[rr], a1 = (uint32_t)(a[rr] >> 32);
          acc3_mac(acc[rr][0], a0, a1, bq.x, bq.y);
          acc3_mac(acc[rr][1], a0, a1, bq.z, bq.w);
        }
        if constexpr (kStepK >= 8) {
          // global step kb * kStepK + k; kStepK is 8 or a multiple of 16
          const int gk = (kStepK % 16 == 0) ? k : (kb & 1) * 8 + k;
          if ((gk & 15) == 15) {
#pragma unroll
            for (int rr = 0; rr < kRows; ++rr) {
              acc3_flush(acc[rr][0]);
              acc3_flush(acc[rr][1]);
            }
          } else if ((gk & 7) == 7) {
#pragma unroll
            for (int rr = 0; rr < kRows; ++rr) {
              acc3_flush_mid(acc[rr][0]);
              acc3_flush_mid(acc[rr][1]);
            }
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      if (++s == kStages) {
        s = 0;
        phase ^= 1u;
      }
      if constexpr (kStepK < 8) {
        constexpr int kEvery = 8 / kStepK;  // stages per 8 k-steps
        if (kb % kEvery == kEvery - 1) {
#pragma unroll
          for (int rr = 0; rr < kRows; ++rr) {
            acc3_flush(acc[rr][0]);
            acc3_flush(acc[rr][1]);
          }
        }
      }
    }
    const size_t c = (size_t)g * G.pc + p;
    uint64_t *o = out + b * out_stride;
    if constexpr (kTwoMods) {
      // slots from mod_planes on belong to the second modulus
      const ScanMod m = c < (size_t)G.mod_planes
                            ? ScanMod{C.q, C.two30, C.two30_s, C.two60, C.two60_s, mu_lo, mu_hi}
                            : G.m1;
#pragma unroll
      for (int rr = 0; rr < kRows; ++rr) {
        const size_t row = (size_t)rt * G.rt + r + rr;
        o[row * G.o_row + c] = acc3_reduce(acc[rr][0], m, kKara != 0);
        o[row * G.o_row + G.o_poly + c] = acc3_reduce(acc[rr][1], m, kKara != 0);
      }
    } else {
#pragma unroll
      for (int rr = 0; rr < kRows; ++rr) {
        const size_t row = (size_t)rt * G.rt + r + rr;
        o[row * G.o_row + c] = acc3_reduce(acc[rr][0], C, mu_lo, mu_hi, kKara != 0);
        o[row * G.o_row + G.o_poly + c] = acc3_reduce(acc[rr][1], C, mu_lo, mu_hi, kKara != 0);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// batched product (many queries, one pass over the database)
//
// Per NTT slot c the first dimension of B queries is the integer GEMM
// (n_rest x n1) . (n1 x 2B).  A CTA computes a 32-row x 32-query tile (64
// output columns) of one slot; each consumer thread owns two rows and two
// queries (8 outputs).  A 60x60-bit product uses Karatsuba on the 30-bit
// halves: a b = a0 b0 + ((a0 + a1)(b0 + b1) - a0 b0 - a1 b1) 2^30 + a1 b1 2^60,
// three IMAD.WIDE per MAC.  The (a0+a1)(b0+b1) partial (< 2^62) is folded into
// its 96-bit total every 4 k-steps, the outer ones every 16.
// ---------------------------------------------------------------------------
constexpr int kBQ = 32;       // queries per tile
constexpr int kBRows = 32;    // rows per tile
constexpr int kBWarps = 8;    // consumer warps (256 threads: 16 row pairs x 16 query pairs)
constexpr int kBK = 16;       // k-steps per stage
constexpr int kBStages = 6;

struct A96 {
  uint64_t lo;
  uint32_t hi;
};
__device__ __forceinline__ void add96(A96 &a, uint64_t v) {
  asm("add.cc.u64 %0, %0, %2;\n\taddc.u32 %1, %1, 0;" : "+l"(a.lo), "+r"(a.hi) : "l"(v));
}
struct KAcc {
  uint64_t ll, hh, ss;
  A96 LL, HH, SS;
};
__device__ __forceinline__ void kacc_zero(KAcc &a) {
  a.ll = a.hh = a.ss = 0;
  a.LL = a.HH = a.SS = A96{0, 0};
}
// kKaratsuba: SS holds (a0+a1)(b0+b1) (mid = SS - LL - HH); otherwise SS
// already holds the cross terms a0 b1 + a1 b0.
template <bool kKaratsuba>
__device__ __forceinline__ uint64_t kacc_reduce(KAcc &a, const Consts &C, uint64_t mu_lo,
                                                uint64_t mu_hi) {
  add96(a.LL, a.ll);
  add96(a.HH, a.hh);
  add96(a.SS, a.ss);
  // mid = SS - LL - HH  (exact, >= 0)
  U128 mid{a.SS.lo, a.SS.hi};
  if (kKaratsuba) {
    asm("sub.cc.u64 %0, %0, %2;\n\tsubc.u64 %1, %1, %3;" : "+l"(mid.lo), "+l"(mid.hi)
        : "l"(a.LL.lo), "l"((uint64_t)a.LL.hi));
    asm("sub.cc.u64 %0, %0, %2;\n\tsubc.u64 %1, %1, %3;" : "+l"(mid.lo), "+l"(mid.hi)
        : "l"(a.HH.lo), "l"((uint64_t)a.HH.hi));
  }
  const uint64_t q = C.q;
  const uint64_t rl = barrett128(U128{a.LL.lo, a.LL.hi}, q, mu_lo, mu_hi);
  const uint64_t rm = barrett128(mid, q, mu_lo, mu_hi);
  const uint64_t rh = barrett128(U128{a.HH.lo, a.HH.hi}, q, mu_lo, mu_hi);
  uint64_t r = add_mod(rl, mul_shoup(rm, C.two30, C.two30_s, q), q);
  return add_mod(r, mul_shoup(rh, C.two60, C.two60_s, q), q);
}

struct BatchGeom {
  int n1, n_rest, batch;
  int row_tiles;     // n_rest / 32
  int groups;        // ceil(batch / 32)
  int nkb;           // n1 / kBK
  long long items;   // groups * kN * row_tiles
};

template <int kForm>
__global__ void __launch_bounds__(kBWarps * 32 + 32, 1)
    scan_batch_kernel(const uint64_t *__restrict__ dbs, const uint4 *__restrict__ qsb,
                      uint64_t *out, size_t out_stride, BatchGeom G, Consts C, uint64_t mu_lo,
                      uint64_t mu_hi, uint32_t *status) {
  constexpr int kDbBytes = kBK * kBRows * 8;  // 4 KB
  constexpr int kQBytes = kBK * kBQ * 16;     // 8 KB
  constexpr int kStage = kDbBytes + kQBytes;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw + kBStages * kStage);
  uint64_t *empty = full + kBStages;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kBStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kBWarps);
    }
    mbar_fence_init();
  }
  __syncthreads();
  const size_t plane_words = (size_t)G.n1 * G.n_rest;
  const long long per_group = (long long)kN * G.row_tiles;

  if (warp == kBWarps) {
    // ------------------------------ producer ------------------------------
    int ps = 0;
    uint32_t pphase = 0;
    long long it = 0;
    bool ok = true;
    for (long long item = blockIdx.x; item < G.items && ok; item += gridDim.x) {
      const int grp = (int)(item / per_group);
      const long long rem = item % per_group;
      const int c = (int)(rem / G.row_tiles), rt = (int)(rem % G.row_tiles);
      const int b0 = grp * kBQ;
      const int nq = G.batch - b0 < kBQ ? G.batch - b0 : kBQ;
      for (int kb = 0; kb < G.nkb; ++kb, ++it) {
        const int s = ps;
        const bool reuse = it >= kBStages;
        const uint32_t ephase = pphase ^ 1u;
        if (++ps == kBStages) {
          ps = 0;
          pphase ^= 1u;
        }
        if (reuse) {
          bool w = true;
          if (lane == 0) w = mbar_wait(&empty[s], ephase);
          w = __shfl_sync(0xffffffffu, w, 0);
          if (!w) {
            if (lane == 0) report_error(status, kErrWaitEmpty);
            ok = false;
            break;
          }
        }
        unsigned char *st = smem_raw + (size_t)s * kStage;
        uint64_t *sdb = reinterpret_cast<uint64_t *>(st);
        uint4 *sq = reinterpret_cast<uint4 *>(st + kDbBytes);
        const uint32_t bytes = (uint32_t)(kDbBytes + kBK * nq * 16);
        if (lane == 0) mbar_arrive_expect_tx(&full[s], bytes);
        __syncwarp();
        const int k0 = kb * kBK;
        const uint64_t *plane = dbs + (size_t)c * plane_words + (size_t)rt * kBRows;
        if (G.n_rest == kBRows) {
          if (lane == 0) bulk_g2s(sdb, plane + (size_t)k0 * G.n_rest, kDbBytes, &full[s]);
        } else if (lane < kBK) {
          bulk_g2s(sdb + lane * kBRows, plane + (size_t)(k0 + lane) * G.n_rest, kBRows * 8,
                   &full[s]);
        }
        const uint4 *qsrc = qsb + ((size_t)c * G.n1 + k0) * G.batch + b0;
        if (nq == G.batch && nq == kBQ) {
          if (lane == 0) bulk_g2s(sq, qsrc, kQBytes, &full[s]);
        } else if (lane < kBK) {
          bulk_g2s(sq + lane * kBQ, qsrc + (size_t)lane * G.batch, nq * 16, &full[s]);
        }
      }
    }
    if (lane == 0) {
      const long long first = it > kBStages ? it - kBStages : 0;
      for (long long j = first; j < it; ++j)
        if (!mbar_wait(&full[j % kBStages], (uint32_t)((j / kBStages) & 1))) {
          report_error(status, kErrDrain);
          break;
        }
    }
    return;
  }

  // ------------------------------ consumers ------------------------------
  const int r = (threadIdx.x >> 4) * 2;  // first of the thread's two rows
  const int jq = (threadIdx.x & 15) * 2; // first of the thread's two queries
  int s = 0;
  uint32_t phase = 0;
  for (long long item = blockIdx.x; item < G.items; item += gridDim.x) {
    const int grp = (int)(item / per_group);
    const long long rem = item % per_group;
    const int c = (int)(rem / G.row_tiles), rt = (int)(rem % G.row_tiles);
    KAcc acc[2][2][2];  // [row][query][poly]
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        kacc_zero(acc[i][j][0]);
        kacc_zero(acc[i][j][1]);
      }
    for (int kb = 0; kb < G.nkb; ++kb) {
      if (!mbar_wait_sleep(&full[s], phase)) {
        report_error(status, kErrWaitFull);
        return;
      }
      const unsigned char *st = smem_raw + (size_t)s * kStage;
      const uint64_t *sdb = reinterpret_cast<const uint64_t *>(st) + r;
      const uint4 *sq = reinterpret_cast<const uint4 *>(st + kDbBytes) + jq;
#pragma unroll 1
      for (int k4 = 0; k4 < kBK; k4 += 4) {
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const int k = k4 + kk;
          const ulonglong2 av = *reinterpret_cast<const ulonglong2 *>(sdb + k * kBRows);
          const uint4 q0 = sq[k * kBQ], q1 = sq[k * kBQ + 1];
          const uint32_t bs[2][2] = {{q0.x + q0.y, q0.z + q0.w}, {q1.x + q1.y, q1.z + q1.w}};
          const uint4 bq[2] = {q0, q1};
#pragma unroll
          for (int i = 0; i < 2; ++i) {
            const uint64_t a = i ? av.y : av.x;
            const uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32), sa = a0 + a1;
#pragma unroll
            for (int j = 0; j < 2; ++j) {
              if constexpr (kForm == 2) {
                // four products: ss holds the cross terms a0 b1 + a1 b0 (flushed every 4 steps)
                madw<kForm>(acc[i][j][0].ll, a0, bq[j].x);
                madw<kForm>(acc[i][j][0].ss, a0, bq[j].y);
                madw<kForm>(acc[i][j][0].ss, a1, bq[j].x);
                madw<kForm>(acc[i][j][0].hh, a1, bq[j].y);
                madw<kForm>(acc[i][j][1].ll, a0, bq[j].z);
                madw<kForm>(acc[i][j][1].ss, a0, bq[j].w);
                madw<kForm>(acc[i][j][1].ss, a1, bq[j].z);
                madw<kForm>(acc[i][j][1].hh, a1, bq[j].w);
              } else {
                madw<kForm>(acc[i][j][0].ll, a0, bq[j].x);
                madw<kForm>(acc[i][j][0].hh, a1, bq[j].y);
                madw<kForm>(acc[i][j][0].ss, sa, bs[j][0]);
                madw<kForm>(acc[i][j][1].ll, a0, bq[j].z);
                madw<kForm>(acc[i][j][1].hh, a1, bq[j].w);
                madw<kForm>(acc[i][j][1].ss, sa, bs[j][1]);
              }
            }
          }
        }
        // the (a0+a1)(b0+b1) partial holds 4 steps
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int pl = 0; pl < 2; ++pl) {
              add96(acc[i][j][pl].SS, acc[i][j][pl].ss);
              acc[i][j][pl].ss = 0;
            }
      }
      // the outer partials hold 16 steps: one stage
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
          for (int pl = 0; pl < 2; ++pl) {
            add96(acc[i][j][pl].LL, acc[i][j][pl].ll);
            add96(acc[i][j][pl].HH, acc[i][j][pl].hh);
            acc[i][j][pl].ll = acc[i][j][pl].hh = 0;
          }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      if (++s == kBStages) {
        s = 0;
        phase ^= 1u;
      }
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const size_t row = (size_t)rt * kBRows + r + i;
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int b = grp * kBQ + jq + j;
        if (b < G.batch) {
          uint64_t *o = out + (size_t)b * out_stride + row * 2 * kN + c;
          o[0] = kacc_reduce<kForm != 2>(acc[i][j][0], C, mu_lo, mu_hi);
          o[kN] = kacc_reduce<kForm != 2>(acc[i][j][1], C, mu_lo, mu_hi);
        }
      }
    }
  }
}

int g_num_sms = 0;
// default tiles before (or without) the autotuner: configuration 8, the
// fastest on the 262,144-plaintext database (0.655 against 0.674 ms)
constexpr int kDefaultCfg = 8;
int g_cfg = kDefaultCfg;
bool g_balance_rounds = true;  // OPIR_SCAN_BALANCE=0: one CTA per resident slot
int g_batch_form = 3;  // accumulate spelling of scan_batch_kernel (OPIR_BATCH_MAC)

template <int R, int W, int K, int S, int B, int KA, bool TWO = false>
cudaError_t set_attr() {
  constexpr int kTileRows = R * W * 32;
  const int max_smem = S * (K * kTileRows * 8 + (kTileRows / 2) * K * 16) + 2 * S * 8;
  return cudaFuncSetAttribute(scan_bulk_kernel<R, W, K, S, B, KA, TWO>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              max_smem > 227 * 1024 ? 227 * 1024 : max_smem);
}

template <int R, int W, int K, int S, int B, int KA, bool TWO = false>
bool launch_bulk(const uint64_t *dbs, const uint4 *qs, size_t qs_stride, uint64_t *out,
                 size_t out_stride, int n1, int n_rest, int batch, const Consts &C,
                 uint64_t mu_lo, uint64_t mu_hi, uint32_t *status, cudaStream_t s,
                 int planes = kN, size_t o_row = 2 * (size_t)kN, size_t o_poly = kN,
                 int mod_planes = kN, const ScanMod *m1 = nullptr) {
  if (n1 % K != 0) return false;
  constexpr int kTileRows = R * W * 32;
  ScanGeom G;
  G.n1 = n1;
  G.n_rest = n_rest;
  G.rt = n_rest < kTileRows ? n_rest : kTileRows;
  G.pc = kTileRows / G.rt;
  if (G.rt < R) return false;
  G.row_tiles = n_rest / G.rt;
  G.nkb = n1 / K;
  if (planes % G.pc != 0) return false;
  G.planes = planes;
  G.o_row = o_row;
  G.o_poly = o_poly;
  G.mod_planes = mod_planes;
  G.m1 = m1 ? *m1 : ScanMod{C.q, C.two30, C.two30_s, C.two60, C.two60_s, mu_lo, mu_hi};
  G.items = (long long)batch * (planes / G.pc) * G.row_tiles;
  G.q_bytes = G.pc * K * 16;
  const int smem = S * (K * kTileRows * 8 + G.q_bytes) + 2 * S * 8;
  if (smem > 227 * 1024) return false;  // tiny planes: many query runs per stage
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, scan_bulk_kernel<R, W, K, S, B, KA, TWO>,
                                                W * 32 + 32, smem);
  if (per_sm < 1) per_sm = 1;
  const int sms = g_num_sms > 0 ? g_num_sms : 152;
  long long grid = (long long)per_sm * sms;
  if (grid > G.items) grid = G.items;
  if (g_balance_rounds) {
    // as many CTAs as the rounds need: the last round then keeps them all
    // busy (2048 tiles: 147 CTAs of 14 rounds instead of 152 ending with 72)
    const long long rounds = (G.items + grid - 1) / grid;
    grid = (G.items + rounds - 1) / rounds;
  }
  scan_bulk_kernel<R, W, K, S, B, KA, TWO><<<(unsigned)grid, W * 32 + 32, smem, s>>>(
      dbs, qs, qs_stride, out, out_stride, G, C, mu_lo, mu_hi, status);
  return true;
}

// compiled configurations {rows, warps, k-steps, stages, CTAs/SM, Karatsuba};
// OPIR_SCAN_CFG selects one by index (tuning sweeps)
#define OPIR_SCAN_CONFIGS(X) \
  X(0, 1, 16, 16, 3, 1, 0)   \
  X(1, 1, 16, 8, 6, 1, 0)    \
  X(2, 1, 16, 16, 2, 1, 0)   \
  X(3, 1, 16, 8, 5, 1, 0)    \
  X(4, 1, 16, 4, 12, 1, 0)   \
  X(5, 2, 8, 16, 3, 1, 0)    \
  X(6, 1, 8, 16, 3, 2, 0)    \
  X(7, 1, 16, 16, 3, 1, 1)   \
  X(8, 2, 8, 16, 3, 1, 1)
constexpr int kNumCfgs = 9;
static_assert(kDefaultCfg < kNumCfgs, "default scan configuration");
// the default configuration's template arguments (kDefaultCfg = 8 above):
// the two-modulus instantiation of the multi-modulus path
constexpr int kPlanesCfg[6] = {2, 8, 16, 3, 1, 1};

}  // namespace

cudaError_t init_scan_attributes() {
  cudaError_t e = cudaSuccess;
#define OPIR_SET(i, R, W, K, S, B, KA) \
  if (e == cudaSuccess) e = set_attr<R, W, K, S, B, KA>();
  OPIR_SCAN_CONFIGS(OPIR_SET)
#undef OPIR_SET
  if (e == cudaSuccess)
    e = set_attr<kPlanesCfg[0], kPlanesCfg[1], kPlanesCfg[2], kPlanesCfg[3], kPlanesCfg[4],
                 kPlanesCfg[5], true>();
  if (e != cudaSuccess) return e;
  int dev;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
  {
    const int smem = kBStages * (kBK * kBRows * 8 + kBK * kBQ * 16) + 2 * kBStages * 8;
    const void *fns[] = {(const void *)scan_batch_kernel<0>, (const void *)scan_batch_kernel<1>,
                         (const void *)scan_batch_kernel<2>, (const void *)scan_batch_kernel<3>};
    for (const void *f : fns) {
      e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      if (e != cudaSuccess) return e;
    }
    g_batch_form = 3;  // measured fastest: carry-chained 32-bit multiply-adds
    if (const char *v = getenv("OPIR_BATCH_MAC")) g_batch_form = atoi(v) & 3;
  }
  g_balance_rounds = true;
  if (const char *v = getenv("OPIR_SCAN_BALANCE")) g_balance_rounds = atoi(v) != 0;
  g_cfg = kDefaultCfg;
  if (const char *v = getenv("OPIR_SCAN_CFG")) {
    const int i = atoi(v);
    if (i >= 0 && i < kNumCfgs) g_cfg = i;
  }
  return cudaSuccess;
}

bool launch_scan_batched(const uint64_t *dbs, const uint4 *qsb, uint64_t *out, size_t out_stride,
                         int n1, int n_rest, int batch, const Consts &C, uint64_t mu_lo,
                         uint64_t mu_hi, uint32_t *status, cudaStream_t s) {
  if (n_rest % kBRows != 0 || n1 % kBK != 0 || batch < 1) return false;
  BatchGeom G;
  G.n1 = n1;
  G.n_rest = n_rest;
  G.batch = batch;
  G.row_tiles = n_rest / kBRows;
  G.groups = (batch + kBQ - 1) / kBQ;
  G.nkb = n1 / kBK;
  G.items = (long long)G.groups * kN * G.row_tiles;
  const int smem = kBStages * (kBK * kBRows * 8 + kBK * kBQ * 16) + 2 * kBStages * 8;
  const int sms = g_num_sms > 0 ? g_num_sms : 152;
  long long grid = sms;
  if (grid > G.items) grid = G.items;
  switch (g_batch_form) {
#define OPIR_BATCH(F)                                                        \
  case F:                                                                    \
    scan_batch_kernel<F><<<(unsigned)grid, kBWarps * 32 + 32, smem, s>>>(   \
        dbs, qsb, out, out_stride, G, C, mu_lo, mu_hi, status);             \
    break;
    OPIR_BATCH(0)
    OPIR_BATCH(1)
    OPIR_BATCH(2)
    OPIR_BATCH(3)
#undef OPIR_BATCH
  }
  return true;
}

int launch_scan_planes(const uint64_t *dbs, const uint4 *qs, size_t qs_stride, uint64_t *out,
                       size_t out_stride, int n1, int n_rest, int batch, int planes,
                       size_t o_row, size_t o_poly, int mod_planes, const Consts &C0,
                       const uint64_t mu0[2], const Consts &C1, const uint64_t mu1[2],
                       uint32_t *status, cudaStream_t s) {
  if (n_rest < 2 || n1 % 8 != 0) return -1;
  const ScanMod m1{C1.q, C1.two30, C1.two30_s, C1.two60, C1.two60_s, mu1[0], mu1[1]};
  // the default tile configuration, with the per-slot choice of modulus
  return launch_bulk<kPlanesCfg[0], kPlanesCfg[1], kPlanesCfg[2], kPlanesCfg[3], kPlanesCfg[4],
                     kPlanesCfg[5], true>(dbs, qs, qs_stride, out, out_stride, n1, n_rest, batch,
                                          C0, mu0[0], mu0[1], status, s, planes, o_row, o_poly,
                                          mod_planes, &m1)
             ? kDefaultCfg
             : -1;
}

int scan_config_count() { return kNumCfgs; }

void scan_config_desc(int i, uint32_t out[6]) {
  uint32_t d[kNumCfgs][6] = {
#define OPIR_DESC(i, R, W, K, S, B, KA) {R, W, K, S, B, KA},
      OPIR_SCAN_CONFIGS(OPIR_DESC)
#undef OPIR_DESC
  };
  for (int k = 0; k < 6; k++) out[k] = (i >= 0 && i < kNumCfgs) ? d[i][k] : 0;
}

int launch_scan(const uint64_t *dbs, const uint4 *qs, size_t qs_stride, uint64_t *out,
                size_t out_stride, int n1, int n_rest, int batch, const Consts &C,
                uint64_t mu_lo, uint64_t mu_hi, uint32_t *status, cudaStream_t s, int cfg) {
  if (cfg < 0 || cfg >= kNumCfgs) cfg = g_cfg;
  if (n_rest >= 2 && n1 % 8 == 0) {
    bool done = false;
    switch (cfg) {
#define OPIR_CASE(i, R, W, K, S, B, KA)                                                      \
  case i:                                                                                    \
    done = launch_bulk<R, W, K, S, B, KA>(dbs, qs, qs_stride, out, out_stride, n1, n_rest,   \
                                          batch, C, mu_lo, mu_hi, status, s);                \
    break;
      OPIR_SCAN_CONFIGS(OPIR_CASE)
#undef OPIR_CASE
    }
    if (done) return cfg;
  }
  if (n_rest % 2 == 0) {
    const size_t threads = (size_t)kN * (n_rest / 2);
    const unsigned blocks = (unsigned)((threads + 255) / 256);
    scan_kernel<2><<<dim3(blocks, batch), 256, 0, s>>>(dbs, qs, qs_stride, out, out_stride, n1,
                                                      n_rest, C, mu_lo, mu_hi);
  } else {
    const size_t threads = (size_t)kN * n_rest;
    const unsigned blocks = (unsigned)((threads + 255) / 256);
    scan_kernel<1><<<dim3(blocks, batch), 256, 0, s>>>(dbs, qs, qs_stride, out, out_stride, n1,
                                                      n_rest, C, mu_lo, mu_hi);
  }
  return -1;
}

}  // namespace opir
