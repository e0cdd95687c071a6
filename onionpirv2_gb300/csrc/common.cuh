// common.cuh -- device-side modular arithmetic and negacyclic NTT for the
// OnionPIRv2 query path on GB300 (sm_103a).
//
// All arithmetic is exact integer arithmetic modulo ~60-bit primes.  Every
// value stored to memory is fully reduced to [0, q), which is what makes the
// GPU path bit-identical to the reference (SEAL's non-lazy NTTs and
// add/sub/multiply all return fully reduced residues).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace opir {

constexpr int kN = 2048;       // polynomial degree (DatabaseConstants::PolyDegree)
constexpr int kLogN = 11;
constexpr int kNttThreads = 256;  // one CTA transforms one polynomial, 8 coeffs/thread
constexpr int kPerThread = kN / kNttThreads;

// Per-modulus constants passed by value to kernels.
struct ModTab {
  const ulonglong2 *fwd;  // {psi^brv(i), Shoup companion}     (forward twiddles)
  const ulonglong2 *inv;  // {psi^-brv(i), Shoup companion}    (inverse twiddles)
  uint64_t q;
  uint64_t n_inv, n_inv_s;  // N^-1 mod q and companion
  uint64_t mu_lo, mu_hi;    // floor(2^128 / q)
};

struct U128 {
  uint64_t lo, hi;
};

__device__ __forceinline__ U128 mul_wide(uint64_t a, uint64_t b) {
  U128 r;
  r.lo = a * b;
  r.hi = __umul64hi(a, b);
  return r;
}

__device__ __forceinline__ void add_to(U128 &acc, U128 v) {
  asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;"
      : "+l"(acc.lo), "+l"(acc.hi)
      : "l"(v.lo), "l"(v.hi));
}

__device__ __forceinline__ void mac_to(U128 &acc, uint64_t a, uint64_t b) {
  add_to(acc, mul_wide(a, b));
}

__device__ __forceinline__ uint64_t add_mod(uint64_t a, uint64_t b, uint64_t q) {
  uint64_t s = a + b;
  return s >= q ? s - q : s;
}
__device__ __forceinline__ uint64_t sub_mod(uint64_t a, uint64_t b, uint64_t q) {
  return a >= b ? a - b : a + q - b;
}
__device__ __forceinline__ uint64_t neg_mod(uint64_t a, uint64_t q) { return a ? q - a : 0; }

// w * x mod q with the Shoup companion ws = floor(w 2^64 / q); x < 2^64, w < q.
__device__ __forceinline__ uint64_t mul_shoup(uint64_t x, uint64_t w, uint64_t ws, uint64_t q) {
  uint64_t hq = __umul64hi(x, ws);
  uint64_t r = x * w - hq * q;
  return r >= q ? r - q : r;
}

// Exact x mod q for x < 2^125.  q_hat = floor(x * mu / 2^128) exactly, and
// that is >= floor(x/q) - 1 when x < 2^125, so one subtraction finishes.
__device__ __forceinline__ uint64_t barrett128(U128 x, uint64_t q, uint64_t mu_lo, uint64_t mu_hi) {
  uint64_t t = __umul64hi(x.lo, mu_lo);
  U128 a = mul_wide(x.lo, mu_hi);
  add_to(a, mul_wide(x.hi, mu_lo));
  add_to(a, U128{t, 0});
  uint64_t qhat = x.hi * mu_hi + a.hi;
  uint64_t r = x.lo - qhat * q;
  return r >= q ? r - q : r;
}

__device__ __forceinline__ uint64_t mul_mod(uint64_t a, uint64_t b, const ModTab &M) {
  return barrett128(mul_wide(a, b), M.q, M.mu_lo, M.mu_hi);
}

// ---------------------------------------------------------------------------
// CTA-wide negacyclic NTT, 256 threads x 8 coefficients in registers.
//
// Forward: Cooley-Tukey, natural-order input, bit-reversed output:
//   A[k] = a(psi^(2 brv(k) + 1)), psi the smallest primitive 2N-th root
//   (the transform SEAL's ntt_negacyclic_harvey computes).
// Inverse: Gentleman-Sande, the exact inverse, scaled by N^-1.
//
// The 11 radix-2 stages run as: bits 10-8 in registers, exchange through
// shared memory, bits 7-5 in registers, exchange, bits 4-2 in registers,
// then bits 1-0 with warp shuffles (after the second exchange those index
// bits are lane bits).  Two distributions of coefficients over threads:
//   strided:  r[e] <-> index tid + 256 e          (coalesced global access)
//   slot:     r[e] <-> index (tid>>2)<<5 | e<<2 | (tid&3)
// The forward transform maps strided -> slot, the inverse slot -> strided.
// Pointwise work between them stays in the slot distribution, reading
// operands from global memory at slot_idx() (full 32-byte sectors).
// ---------------------------------------------------------------------------

// shared-memory index with 4 pad words per 32: conflict-free for every
// exchange pattern used here
__device__ __forceinline__ int spad(int i) { return i + ((i >> 5) << 2); }
constexpr int kSmemPoly = kN + (kN / 32) * 4;  // padded polynomial footprint (u64 words)

__device__ __forceinline__ int strided_idx(int tid, int e) { return tid + kNttThreads * e; }
__device__ __forceinline__ int slot_idx(int tid, int e) {
  return ((tid >> 2) << 5) | (e << 2) | (tid & 3);
}
// index of element e of thread tid in the register pass whose 3 bits start at lo
__device__ __forceinline__ int pass_index(int tid, int e, int lo) {
  const int low = tid & ((1 << lo) - 1);
  const int high = tid >> lo;
  return (high << (lo + 3)) | (e << lo) | low;
}

__device__ __forceinline__ void ct_bf(uint64_t &x, uint64_t &y, ulonglong2 w, uint64_t q) {
  const uint64_t v = mul_shoup(y, w.x, w.y, q);
  const uint64_t u = x;
  x = add_mod(u, v, q);
  y = sub_mod(u, v, q);
}
__device__ __forceinline__ void gs_bf(uint64_t &x, uint64_t &y, ulonglong2 w, uint64_t q) {
  const uint64_t u = x, v = y;
  x = add_mod(u, v, q);
  y = mul_shoup(sub_mod(u, v, q), w.x, w.y, q);
}

// Three CT stages (bits lo+2, lo+1, lo).  Stage on bit b: twiddle m + (idx >> (b+1)), m = 2^(10-b).
__device__ __forceinline__ void ct_pass3(uint64_t r[8], int tid, int lo, const ulonglong2 *tw, uint64_t q) {
  const int base = pass_index(tid, 0, lo);
#pragma unroll
  for (int s = 2; s >= 0; --s) {
    const int b = lo + s;
    const int m = 1 << (10 - b);
    const int half = 1 << s;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      if (e & half) continue;
      const int idx = base | (e << lo);
      ct_bf(r[e], r[e | half], __ldg(tw + m + (idx >> (b + 1))), q);
    }
  }
}
__device__ __forceinline__ void gs_pass3(uint64_t r[8], int tid, int lo, const ulonglong2 *tw, uint64_t q) {
  const int base = pass_index(tid, 0, lo);
#pragma unroll
  for (int s = 0; s <= 2; ++s) {
    const int b = lo + s;
    const int m = 1 << (10 - b);
    const int half = 1 << s;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      if (e & half) continue;
      const int idx = base | (e << lo);
      gs_bf(r[e], r[e | half], __ldg(tw + m + (idx >> (b + 1))), q);
    }
  }
}

__device__ __forceinline__ uint64_t shfl_xor64(uint64_t v, int mask) {
  return __shfl_xor_sync(0xffffffffu, v, mask);
}

// CT stage on index bit b in {0, 1} (== lane bit b in the slot distribution).
__device__ __forceinline__ void ct_lane_stage(uint64_t r[8], int tid, int b, const ulonglong2 *tw, uint64_t q) {
  const int m = 1 << (10 - b);
  const bool hi = (tid >> b) & 1;
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int idx = slot_idx(tid, e);
    const ulonglong2 w = __ldg(tw + m + (idx >> (b + 1)));
    const uint64_t own = r[e];
    const uint64_t send = hi ? mul_shoup(own, w.x, w.y, q) : own;
    const uint64_t recv = shfl_xor64(send, 1 << b);
    r[e] = hi ? sub_mod(recv, send, q) : add_mod(own, recv, q);
  }
}
__device__ __forceinline__ void gs_lane_stage(uint64_t r[8], int tid, int b, const ulonglong2 *tw, uint64_t q) {
  const int m = 1 << (10 - b);
  const bool hi = (tid >> b) & 1;
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int idx = slot_idx(tid, e);
    const uint64_t own = r[e];
    const uint64_t recv = shfl_xor64(own, 1 << b);
    if (hi) {
      const ulonglong2 w = __ldg(tw + m + (idx >> (b + 1)));
      r[e] = mul_shoup(sub_mod(recv, own, q), w.x, w.y, q);
    } else {
      r[e] = add_mod(own, recv, q);
    }
  }
}

__device__ __forceinline__ void store_pass(uint64_t *s, const uint64_t r[8], int tid, int lo) {
#pragma unroll
  for (int e = 0; e < 8; ++e) s[spad(pass_index(tid, e, lo))] = r[e];
}
__device__ __forceinline__ void load_pass(const uint64_t *s, uint64_t r[8], int tid, int lo) {
#pragma unroll
  for (int e = 0; e < 8; ++e) r[e] = s[spad(pass_index(tid, e, lo))];
}

// Forward NTT: r strided -> r slot.  sa, sb: two shared buffers of
// kSmemPoly words each (double buffering: two barriers per transform).
// All 256 threads of the calling group must participate.
__device__ __forceinline__ void ntt_fwd(uint64_t r[8], uint64_t *sa, uint64_t *sb,
                                        const ulonglong2 *tw, uint64_t q) {
  const int tid = threadIdx.x & (kNttThreads - 1);
  ct_pass3(r, tid, 8, tw, q);
  store_pass(sa, r, tid, 8);
  __syncthreads();
  load_pass(sa, r, tid, 5);
  ct_pass3(r, tid, 5, tw, q);
  store_pass(sb, r, tid, 5);
  __syncthreads();
  load_pass(sb, r, tid, 2);
  ct_pass3(r, tid, 2, tw, q);
  ct_lane_stage(r, tid, 1, tw, q);
  ct_lane_stage(r, tid, 0, tw, q);
}

// Inverse NTT: r slot -> r strided, scaled by N^-1.
__device__ __forceinline__ void ntt_inv(uint64_t r[8], uint64_t *sa, uint64_t *sb,
                                        const ulonglong2 *tw, uint64_t q, uint64_t n_inv,
                                        uint64_t n_inv_s) {
  const int tid = threadIdx.x & (kNttThreads - 1);
  gs_lane_stage(r, tid, 0, tw, q);
  gs_lane_stage(r, tid, 1, tw, q);
  gs_pass3(r, tid, 2, tw, q);
  store_pass(sa, r, tid, 2);
  __syncthreads();
  load_pass(sa, r, tid, 5);
  gs_pass3(r, tid, 5, tw, q);
  store_pass(sb, r, tid, 5);
  __syncthreads();
  load_pass(sb, r, tid, 8);
  gs_pass3(r, tid, 8, tw, q);
#pragma unroll
  for (int e = 0; e < 8; ++e) r[e] = mul_shoup(r[e], n_inv, n_inv_s, q);
}

__device__ __forceinline__ void ntt_fwd(uint64_t r[8], uint64_t *sa, uint64_t *sb, const ModTab &M) {
  ntt_fwd(r, sa, sb, M.fwd, M.q);
}
__device__ __forceinline__ void ntt_inv(uint64_t r[8], uint64_t *sa, uint64_t *sb, const ModTab &M) {
  ntt_inv(r, sa, sb, M.inv, M.q, M.n_inv, M.n_inv_s);
}

}  // namespace opir
