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
// Butterflies are Harvey's lazy ones: forward values live in [0, 4q),
// inverse values in [0, 2q) (q < 2^60, so 4q < 2^62); both transforms end
// with a full reduction, so every output is in [0, q).
//
// The 11 radix-2 stages run as four register passes -- index bits 10-8,
// 7-5, 4-2 and 1-0 -- separated by three shared-memory exchanges.  Two
// distributions of coefficients over threads:
//   strided:  r[e] <-> index tid + 256 e      (coalesced global access)
//   slot:     r[e] <-> index 8 tid + e        (8 consecutive NTT slots)
// The forward transform maps strided -> slot, the inverse slot -> strided.
// Pointwise work between them stays in the slot distribution and reads its
// operands with 16-byte vector loads (ldg_slot8).
// ---------------------------------------------------------------------------

// shared-memory index with 2 pad words per 16: every exchange pattern below
// is bank-conflict free (the slot exchange uses 16-byte accesses)
__device__ __forceinline__ int spad(int i) { return i + ((i >> 4) << 1); }
constexpr int kSmemPoly = kN + (kN / 16) * 2;  // padded polynomial footprint (u64 words)

__device__ __forceinline__ int strided_idx(int tid, int e) { return tid + kNttThreads * e; }
__device__ __forceinline__ int slot_idx(int tid, int e) { return 8 * tid + e; }
// index of element e of thread tid in the register pass whose 3 bits start at lo
__device__ __forceinline__ int pass_index(int tid, int e, int lo) {
  const int low = tid & ((1 << lo) - 1);
  const int high = tid >> lo;
  return (high << (lo + 3)) | (e << lo) | low;
}

// x * w mod q up to one extra q: result in [0, 2q) for any x < 2^64
__device__ __forceinline__ uint64_t mul_shoup_lazy(uint64_t x, uint64_t w, uint64_t ws, uint64_t q) {
  const uint64_t hq = __umul64hi(x, ws);
  return x * w - hq * q;
}

// x * w mod q up to three extra q: result in [0, 4q) for any x < 2^64.  The
// Shoup quotient x * ws / 2^64 is taken from three of the four 32x32 partial
// products (the low one and the carries out of the middle ones are dropped),
// which undercounts it by at most 2.
__device__ __forceinline__ uint64_t mul_shoup_lazy4(uint64_t x, uint64_t w, uint64_t ws, uint64_t q) {
  const uint32_t x0 = (uint32_t)x, x1 = (uint32_t)(x >> 32);
  const uint32_t s0 = (uint32_t)ws, s1 = (uint32_t)(ws >> 32);
  const uint64_t hq = (uint64_t)x1 * s1 + __umulhi(x1, s0) + __umulhi(x0, s1);
  return x * w - hq * q;
}

// lazy CT butterfly: inputs and outputs in [0, 8q) (q4 = 4q; q < 2^60)
__device__ __forceinline__ void ct_bf(uint64_t &x, uint64_t &y, ulonglong2 w, uint64_t q,
                                      uint64_t q4) {
  const uint64_t u = x >= q4 ? x - q4 : x;
  const uint64_t t = mul_shoup_lazy4(y, w.x, w.y, q);
  x = u + t;
  y = u - t + q4;
}
// lazy GS butterfly: inputs and outputs in [0, 4q)
__device__ __forceinline__ void gs_bf(uint64_t &x, uint64_t &y, ulonglong2 w, uint64_t q,
                                      uint64_t q4) {
  const uint64_t u = x, v = y;
  const uint64_t s = u + v;
  x = s >= q4 ? s - q4 : s;
  y = mul_shoup_lazy4(u - v + q4, w.x, w.y, q);
}

// Twiddle reads: from global memory through the read-only path, or from a
// copy staged in shared memory (prefetch_tw), which latency-bound kernels
// with few CTAs per SM use -- an L2 round trip per register pass otherwise
// sits on the critical path of every transform.
template <bool kSmemTw>
__device__ __forceinline__ ulonglong2 tw_ld(const ulonglong2 *p) {
  if constexpr (kSmemTw) return *p;
  else return __ldg(p);
}

// Three CT stages (bits lo+2, lo+1, lo).  Stage on bit b: twiddle m + (idx >> (b+1)), m = 2^(10-b).
template <bool kSmemTw = false>
__device__ __forceinline__ void ct_pass3(uint64_t r[8], int tid, int lo, const ulonglong2 *tw,
                                         uint64_t q, uint64_t q4) {
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
      ct_bf(r[e], r[e | half], tw_ld<kSmemTw>(tw + m + (idx >> (b + 1))), q, q4);
    }
  }
}
template <bool kSmemTw = false>
__device__ __forceinline__ void gs_pass3(uint64_t r[8], int tid, int lo, const ulonglong2 *tw,
                                         uint64_t q, uint64_t q4) {
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
      gs_bf(r[e], r[e | half], tw_ld<kSmemTw>(tw + m + (idx >> (b + 1))), q, q4);
    }
  }
}
// Stages on bits 1 and 0: the thread's slots 8 tid .. 8 tid + 7 form the
// radix-4 groups g = 2 tid and 2 tid + 1.
template <bool kSmemTw = false>
__device__ __forceinline__ void ct_pass2(uint64_t r[8], int tid, const ulonglong2 *tw, uint64_t q,
                                         uint64_t q4) {
#pragma unroll
  for (int gsub = 0; gsub < 2; ++gsub) {
    const int g = 2 * tid + gsub;
    uint64_t *x = r + 4 * gsub;
    const ulonglong2 w1 = tw_ld<kSmemTw>(tw + 512 + g);
    ct_bf(x[0], x[2], w1, q, q4);
    ct_bf(x[1], x[3], w1, q, q4);
    ct_bf(x[0], x[1], tw_ld<kSmemTw>(tw + 1024 + 2 * g), q, q4);
    ct_bf(x[2], x[3], tw_ld<kSmemTw>(tw + 1024 + 2 * g + 1), q, q4);
  }
}
template <bool kSmemTw = false>
__device__ __forceinline__ void gs_pass2(uint64_t r[8], int tid, const ulonglong2 *tw, uint64_t q,
                                         uint64_t q4) {
#pragma unroll
  for (int gsub = 0; gsub < 2; ++gsub) {
    const int g = 2 * tid + gsub;
    uint64_t *x = r + 4 * gsub;
    gs_bf(x[0], x[1], tw_ld<kSmemTw>(tw + 1024 + 2 * g), q, q4);
    gs_bf(x[2], x[3], tw_ld<kSmemTw>(tw + 1024 + 2 * g + 1), q, q4);
    const ulonglong2 w1 = tw_ld<kSmemTw>(tw + 512 + g);
    gs_bf(x[0], x[2], w1, q, q4);
    gs_bf(x[1], x[3], w1, q, q4);
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
__device__ __forceinline__ void store_slots(uint64_t *s, const uint64_t r[8], int tid) {
#pragma unroll
  for (int j = 0; j < 4; ++j)
    *reinterpret_cast<ulonglong2 *>(s + spad(8 * tid + 2 * j)) = make_ulonglong2(r[2 * j], r[2 * j + 1]);
}
__device__ __forceinline__ void load_slots(const uint64_t *s, uint64_t r[8], int tid) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(s + spad(8 * tid + 2 * j));
    r[2 * j] = v.x;
    r[2 * j + 1] = v.y;
  }
}

// 8 consecutive slots of a global array (16-byte aligned) for this thread
__device__ __forceinline__ void ldg_slot8(const uint64_t *base, uint64_t v[8]) {
  const ulonglong2 *p = reinterpret_cast<const ulonglong2 *>(base) + 4 * (threadIdx.x & (kNttThreads - 1));
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const ulonglong2 t = __ldg(p + j);
    v[2 * j] = t.x;
    v[2 * j + 1] = t.y;
  }
}
// the slot layout of ldg_slot8 from shared memory
__device__ __forceinline__ void lds_slot8(const uint64_t *base, uint64_t v[8]) {
  const ulonglong2 *p = reinterpret_cast<const ulonglong2 *>(base) + 4 * (threadIdx.x & (kNttThreads - 1));
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const ulonglong2 t = p[j];
    v[2 * j] = t.x;
    v[2 * j + 1] = t.y;
  }
}
// the slot layout of ldg_slot8 through the coherent path (for data the
// calling kernel itself writes later)
__device__ __forceinline__ void ld_slot8(const uint64_t *base, uint64_t v[8]) {
  const ulonglong2 *p = reinterpret_cast<const ulonglong2 *>(base) + 4 * (threadIdx.x & (kNttThreads - 1));
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const ulonglong2 t = p[j];
    v[2 * j] = t.x;
    v[2 * j + 1] = t.y;
  }
}
__device__ __forceinline__ void stg_slot8(uint64_t *base, const uint64_t v[8]) {
  ulonglong2 *p = reinterpret_cast<ulonglong2 *>(base) + 4 * (threadIdx.x & (kNttThreads - 1));
#pragma unroll
  for (int j = 0; j < 4; ++j) p[j] = make_ulonglong2(v[2 * j], v[2 * j + 1]);
}

// Forward NTT: r strided (values < 8q) -> r slot (fully reduced).  sa, sb:
// two shared buffers of kSmemPoly words; all 256 threads of the group take
// part; ends with a barrier so sa/sb may be reused at once.
template <bool kSmemTw = false>
__device__ __forceinline__ void ntt_fwd(uint64_t r[8], uint64_t *sa, uint64_t *sb,
                                        const ulonglong2 *tw, uint64_t q) {
  const int tid = threadIdx.x & (kNttThreads - 1);
  const uint64_t q2 = 2 * q, q4 = 4 * q;
  ct_pass3<kSmemTw>(r, tid, 8, tw, q, q4);
  store_pass(sa, r, tid, 8);
  __syncthreads();
  load_pass(sa, r, tid, 5);
  ct_pass3<kSmemTw>(r, tid, 5, tw, q, q4);
  store_pass(sb, r, tid, 5);
  __syncthreads();
  load_pass(sb, r, tid, 2);
  ct_pass3<kSmemTw>(r, tid, 2, tw, q, q4);
  store_pass(sa, r, tid, 2);
  __syncthreads();
  load_slots(sa, r, tid);
  ct_pass2<kSmemTw>(r, tid, tw, q, q4);
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    uint64_t v = r[e] >= q4 ? r[e] - q4 : r[e];
    v = v >= q2 ? v - q2 : v;
    r[e] = v >= q ? v - q : v;
  }
  __syncthreads();
}

// Inverse NTT: r slot (values < 4q) -> r strided (fully reduced), scaled by N^-1.
template <bool kSmemTw = false>
__device__ __forceinline__ void ntt_inv(uint64_t r[8], uint64_t *sa, uint64_t *sb,
                                        const ulonglong2 *tw, uint64_t q, uint64_t n_inv,
                                        uint64_t n_inv_s) {
  const int tid = threadIdx.x & (kNttThreads - 1);
  const uint64_t q2 = 2 * q, q4 = 4 * q;
  gs_pass2<kSmemTw>(r, tid, tw, q, q4);
  store_slots(sa, r, tid);
  __syncthreads();
  load_pass(sa, r, tid, 2);
  gs_pass3<kSmemTw>(r, tid, 2, tw, q, q4);
  store_pass(sb, r, tid, 2);
  __syncthreads();
  load_pass(sb, r, tid, 5);
  gs_pass3<kSmemTw>(r, tid, 5, tw, q, q4);
  store_pass(sa, r, tid, 5);
  __syncthreads();
  load_pass(sa, r, tid, 8);
  gs_pass3<kSmemTw>(r, tid, 8, tw, q, q4);
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    uint64_t v = mul_shoup_lazy4(r[e], n_inv, n_inv_s, q);
    v = v >= q2 ? v - q2 : v;
    r[e] = v >= q ? v - q : v;
  }
  __syncthreads();
}

__device__ __forceinline__ void ntt_fwd(uint64_t r[8], uint64_t *sa, uint64_t *sb, const ModTab &M) {
  ntt_fwd(r, sa, sb, M.fwd, M.q);
}
__device__ __forceinline__ void ntt_inv(uint64_t r[8], uint64_t *sa, uint64_t *sb, const ModTab &M) {
  ntt_inv(r, sa, sb, M.inv, M.q, M.n_inv, M.n_inv_s);
}
// forward transform with M's twiddle table staged in shared memory at s_fwd
__device__ __forceinline__ void ntt_fwd_s(uint64_t r[8], uint64_t *sa, uint64_t *sb,
                                          const ulonglong2 *s_fwd, const ModTab &M) {
  ntt_fwd<true>(r, sa, sb, s_fwd, M.q);
}
// Stage a 2048-entry twiddle table in shared memory: one 16-byte cp.async
// per entry, issued now; tw_wait() completes it (every thread of the CTA
// must call tw_wait before the first transform that reads the copy).
__device__ __forceinline__ void prefetch_tw(ulonglong2 *dst, const ulonglong2 *src) {
  for (int i = threadIdx.x; i < kN; i += blockDim.x) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst + i);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src + i) : "memory");
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
// the same for `words` 64-bit words (even, both addresses 16-byte aligned)
__device__ __forceinline__ void prefetch_words(uint64_t *dst, const uint64_t *src, int words) {
  for (int i = 2 * threadIdx.x; i < words; i += 2 * blockDim.x) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst + i);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src + i) : "memory");
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
// inverse transform with M's inverse twiddle table staged at s_inv
__device__ __forceinline__ void ntt_inv_s(uint64_t r[8], uint64_t *sa, uint64_t *sb,
                                          const ulonglong2 *s_inv, const ModTab &M) {
  ntt_inv<true>(r, sa, sb, s_inv, M.q, M.n_inv, M.n_inv_s);
}
__device__ __forceinline__ void tw_wait() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();
}
// wait until at most `Pending` of this thread's most recent staging groups
// are still in flight (groups complete in commit order), then make every
// thread's completed copies visible to the CTA
template <int Pending>
__device__ __forceinline__ void stage_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(Pending) : "memory");
  __syncthreads();
}

// Programmatic dependent launch (PTX griddepcontrol).  A kernel launched with
// programmatic stream serialization may become resident while the previous
// kernel of its stream still runs: what it does before grid_dep_wait() may
// read only data that no launch of the current pipeline writes (twiddle
// tables, client keys).  grid_dep_wait() returns once the previous kernel has
// completed and its writes are visible -- at once for a normal launch.
// grid_dep_launch(), called after the wait, lets the next programmatic launch
// become resident; every kernel that calls it has passed its own wait, so
// when a kernel starts, all launches before the previous one are complete.
__device__ __forceinline__ void grid_dep_wait() {
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
}
__device__ __forceinline__ void grid_dep_launch() {
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}
// both, at the point where a kernel starts reading its predecessor's output
__device__ __forceinline__ void grid_dep_sync() {
  grid_dep_wait();
  grid_dep_launch();
}

}  // namespace opir
