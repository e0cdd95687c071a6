// rns.cu -- the multi-modulus server query path on GB300 (sm_103a): R = 1 or
// 2 ciphertext primes plus the special prime p, any power-of-two N up to
// 4096 (the PolyDegree = 4096, CoeffMods = {60, 60, 60} presets,
// src/includes/database_constants.h:13-172).
//
// Layouts are SEAL's (poly, then prime, then coefficient): a ciphertext is
// [2][R][N], an RGSW ciphertext [rows][2][R][N], the Galois keys of one level
// [R][2][R+1][N] (decomposition prime, key polynomial, modulus q_0 .. q_{R-1}, p).
// The database is stored per NTT slot cc = i N + c of prime i as a plane
// [n1][n_rest], so a CTA of the scan streams one contiguous plane.
//
// The stages run as separate kernels with their intermediates in global
// memory: every polynomial transform is one CTA over a shared-memory copy
// (radix-2, all residues fully reduced), every pointwise stage is one CTA per
// polynomial.  All arithmetic is exact; results equal the CPU restatement
// (oracle/opir_oracle_rns.c) bit for bit.
#include "rns.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "async.cuh"
#include "common.cuh"
#include "entry.cuh"
#include "hostmath.h"

namespace opir {

namespace {

using u128 = unsigned __int128;
constexpr int kRT = 512;  // threads of the transform and ingest CTAs
constexpr int kPT = 256;  // threads of the pointwise CTAs
// The pointwise kernels give every thread one coefficient: blockIdx.x runs
// over (unit, chunk of kPT coefficients) -- narrow tree levels (a node or a
// pair) still spread over N / kPT CTAs per polynomial.
__device__ __forceinline__ int pw_unit(int n) { return (int)blockIdx.x / (n / kPT); }
__device__ __forceinline__ int pw_coeff(int n) {
  return (int)(blockIdx.x % (unsigned)(n / kPT)) * kPT + (int)threadIdx.x;
}

__device__ __forceinline__ uint64_t rmod(U128 x, const RnsMod &M) {
  return barrett128(x, M.q, M.mu_lo, M.mu_hi);
}

// One polynomial in shared memory, all threads of the CTA.  Forward:
// Cooley-Tukey, natural order in, A[k] = a(psi^(2 brv(k) + 1)) out (SEAL's
// ntt_negacyclic_harvey).  Inverse: Gentleman-Sande, scaled by N^-1.
__device__ void smem_ntt_fwd(uint64_t *s, const ulonglong2 *tw, uint64_t q, int n, int logn) {
  for (int m = 1, lt = logn - 1; m < n; m <<= 1, --lt) {
    const int t = 1 << lt;
    for (int bf = threadIdx.x; bf < (n >> 1); bf += blockDim.x) {
      const int i = bf >> lt, j = bf & (t - 1);
      const int x = 2 * i * t + j, y = x + t;
      const ulonglong2 w = tw[m + i];
      const uint64_t u = s[x], v = mul_shoup(s[y], w.x, w.y, q);
      s[x] = add_mod(u, v, q);
      s[y] = sub_mod(u, v, q);
    }
    __syncthreads();
  }
}

__device__ void smem_ntt_inv(uint64_t *s, const ulonglong2 *tw, const RnsMod &M, int n) {
  const uint64_t q = M.q;
  for (int m = n >> 1, lt = 0; m >= 1; m >>= 1, ++lt) {
    const int t = 1 << lt;
    for (int bf = threadIdx.x; bf < (n >> 1); bf += blockDim.x) {
      const int i = bf >> lt, j = bf & (t - 1);
      const int x = 2 * i * t + j, y = x + t;
      const ulonglong2 w = tw[m + i];
      const uint64_t u = s[x], v = s[y];
      s[x] = add_mod(u, v, q);
      s[y] = mul_shoup(sub_mod(u, v, q), w.x, w.y, q);
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) s[i] = mul_shoup(s[i], M.n_inv, M.n_inv_s, q);
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Register-resident transform of N = 4096 (the two-prime presets): 512
// threads x 8 coefficients, four register passes of three radix-2 stages
// (index bits 11-9, 8-6, 5-3, 2-0) separated by shared-memory exchanges --
// the one-prime transform's scheme at twice the size -- with the same lazy
// Harvey butterflies (forward values in [0, 8q), inverse in [0, 4q); every
// prime < 2^60) and the same twiddle tables as smem_ntt_fwd / smem_ntt_inv
// (stage on index bit b: twiddle m + (x >> (b + 1)), m = N / 2^(b+1)).
// Forward: natural order in, SEAL's bit-reversed order out; inverse the
// reverse, scaled by N^-1; both fully reduced.
// ---------------------------------------------------------------------------
constexpr int kLogN4096 = 12;
constexpr int kT4096 = 512;
constexpr int kSmem4096 = 4096 + (4096 / 16) * 2;  // padded exchange buffer (u64 words)

template <int LO>
__device__ __forceinline__ void ct_pass3_4096(uint64_t r[8], int tid, const ulonglong2 *tw,
                                              uint64_t q, uint64_t q4) {
  const int base = pass_index(tid, 0, LO);
#pragma unroll
  for (int st = 2; st >= 0; --st) {
    const int b = LO + st, half = 1 << st;
    const int m = 1 << (kLogN4096 - 1 - b);
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      if (e & half) continue;
      ct_bf(r[e], r[e | half], __ldg(tw + m + ((base | (e << LO)) >> (b + 1))), q, q4);
    }
  }
}
template <int LO>
__device__ __forceinline__ void gs_pass3_4096(uint64_t r[8], int tid, const ulonglong2 *tw,
                                              uint64_t q, uint64_t q4) {
  const int base = pass_index(tid, 0, LO);
#pragma unroll
  for (int st = 0; st <= 2; ++st) {
    const int b = LO + st, half = 1 << st;
    const int m = 1 << (kLogN4096 - 1 - b);
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      if (e & half) continue;
      gs_bf(r[e], r[e | half], __ldg(tw + m + ((base | (e << LO)) >> (b + 1))), q, q4);
    }
  }
}
// exchange between passes through one buffer: every thread's loads of the
// previous exchange are done before anyone stores again
template <int FROM, int TO>
__device__ __forceinline__ void exchange_4096(uint64_t *s, uint64_t r[8], int tid) {
  __syncthreads();
  store_pass(s, r, tid, FROM);
  __syncthreads();
  load_pass(s, r, tid, TO);
}

// forward core: r strided (values < 8q) -> r in SEAL's order, 8 tid + e
// (fully reduced)
__device__ __forceinline__ void ntt4096_fwd(uint64_t r[8], uint64_t *s, int tid,
                                            const ulonglong2 *tw, uint64_t q) {
  const uint64_t q2 = 2 * q, q4 = 4 * q;
  ct_pass3_4096<9>(r, tid, tw, q, q4);
  exchange_4096<9, 6>(s, r, tid);
  ct_pass3_4096<6>(r, tid, tw, q, q4);
  exchange_4096<6, 3>(s, r, tid);
  ct_pass3_4096<3>(r, tid, tw, q, q4);
  exchange_4096<3, 0>(s, r, tid);
  ct_pass3_4096<0>(r, tid, tw, q, q4);
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    uint64_t w = r[e] >= q4 ? r[e] - q4 : r[e];
    w = w >= q2 ? w - q2 : w;
    r[e] = w >= q ? w - q : w;
  }
}
// inverse core: r in SEAL's order, 8 tid + e (values < 4q) -> r strided,
// scaled by N^-1 (fully reduced)
__device__ __forceinline__ void ntt4096_inv(uint64_t r[8], uint64_t *s, int tid,
                                            const ulonglong2 *tw, const RnsMod &M) {
  const uint64_t q = M.q, q2 = 2 * q, q4 = 4 * q;
  gs_pass3_4096<0>(r, tid, tw, q, q4);
  exchange_4096<0, 3>(s, r, tid);
  gs_pass3_4096<3>(r, tid, tw, q, q4);
  exchange_4096<3, 6>(s, r, tid);
  gs_pass3_4096<6>(r, tid, tw, q, q4);
  exchange_4096<6, 9>(s, r, tid);
  gs_pass3_4096<9>(r, tid, tw, q, q4);
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    uint64_t v = mul_shoup_lazy4(r[e], M.n_inv, M.n_inv_s, q);
    v = v >= q2 ? v - q2 : v;
    r[e] = v >= q ? v - q : v;
  }
}
__device__ __forceinline__ void store_slot8(uint64_t *out, const uint64_t r[8], int tid) {
  ulonglong2 *o = reinterpret_cast<ulonglong2 *>(out + 8 * tid);
#pragma unroll
  for (int e = 0; e < 8; e += 2) o[e / 2] = make_ulonglong2(r[e], r[e + 1]);
}

__global__ void __launch_bounds__(kT4096) rns_ntt4096_kernel(const uint64_t *src, size_t src_stride,
                                                             uint64_t *dst, size_t dst_stride,
                                                             int period, int inverse, RnsConsts C) {
  __shared__ uint64_t s[kSmem4096];
  const int tid = threadIdx.x;
  const size_t x = blockIdx.x, y = blockIdx.y;
  const int mi = (int)(x % (size_t)period);
  const uint64_t *in = src + y * src_stride + x * 4096;
  uint64_t *out = dst + y * dst_stride + x * 4096;
  uint64_t r[8];
  if (!inverse) {
#pragma unroll
    for (int e = 0; e < 8; ++e) r[e] = in[tid + kT4096 * e];
    ntt4096_fwd(r, s, tid, C.fwd + (size_t)mi * 4096, C.m[mi].q);
    store_slot8(out, r, tid);
  } else {
    const ulonglong2 *i2 = reinterpret_cast<const ulonglong2 *>(in + 8 * tid);
#pragma unroll
    for (int e = 0; e < 8; e += 2) {
      const ulonglong2 v = i2[e / 2];
      r[e] = v.x;
      r[e + 1] = v.y;
    }
    ntt4096_inv(r, s, tid, C.inv + (size_t)mi * 4096, C.m[mi]);
#pragma unroll
    for (int e = 0; e < 8; ++e) out[tid + kT4096 * e] = r[e];
  }
}

// One expansion level's key switch at N = 4096, fused: CTA x = (node R + j) M
// + m gathers sigma_g(c1 mod q_j) through the inverse automorphism (target d
// takes c1[e] or -c1[e - N], e = d g^-1 mod 2N), lifts it to modulus m and
// transforms it into lift[x] (the m = 0 CTAs also write sigma_g(c0 mod q_j)
// into s0, natural order) -- rns_expand_lift_kernel followed by the forward
// transform.
__global__ void __launch_bounds__(kT4096) rns_expand_lift_ntt4096_kernel(
    const uint64_t *cur, uint64_t *lift, uint64_t *s0, uint64_t ginv, RnsConsts C) {
  __shared__ uint64_t s[kSmem4096];
  const int R = C.R, M = R + 1, tid = threadIdx.x;
  const int x = blockIdx.x, m = x % M, j = (x / M) % R, node = x / (M * R);
  const size_t CT = 2 * (size_t)R * 4096;
  const uint64_t *c0 = cur + node * CT + (size_t)j * 4096;
  const uint64_t *c1 = cur + node * CT + (size_t)(R + j) * 4096;
  const uint64_t qj = C.m[j].q, qm = C.m[m].q;
  uint64_t *S = s0 + ((size_t)node * R + j) * 4096;
  uint64_t r[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int d = tid + kT4096 * e;
    const uint64_t src = ((uint64_t)d * ginv) & (2 * 4096 - 1);
    const bool wrap = src >= 4096;
    const int i = (int)(wrap ? src - 4096 : src);
    const uint64_t v = wrap ? neg_mod(c1[i], qj) : c1[i];
    r[e] = v >= qm ? v - qm : v;
    if (m == 0) S[d] = wrap ? neg_mod(c0[i], qj) : c0[i];
  }
  ntt4096_fwd(r, s, tid, C.fwd + (size_t)m * 4096, qm);
  store_slot8(lift + (size_t)x * 4096, r, tid);
}

// ... and CTA x = (node 2 + k) M + m sums lift[node][j][m] key[j][k][m] over
// the decomposition primes j (NTT form) and transforms the sum back into
// acc[x] (natural order) -- rns_ks_mac_kernel followed by the inverse
// transform.
__global__ void __launch_bounds__(kT4096) rns_ks_intt4096_kernel(const uint64_t *lift,
                                                                 const uint64_t *key, uint64_t *acc,
                                                                 RnsConsts C) {
  __shared__ uint64_t s[kSmem4096];
  const int R = C.R, M = R + 1, tid = threadIdx.x;
  const int x = blockIdx.x, m = x % M, k = (x / M) % 2, node = x / (2 * M);
  uint64_t r[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int c = 8 * tid + e;
    U128 sum{0, 0};
    for (int j = 0; j < R; ++j)
      mac_to(sum, lift[(((size_t)node * R + j) * M + m) * 4096 + c],
             key[(((size_t)j * 2 + k) * M + m) * 4096 + c]);
    r[e] = rmod(sum, C.m[m]);
  }
  ntt4096_inv(r, s, tid, C.inv + (size_t)m * 4096, C.m[m]);
  uint64_t *out = acc + (size_t)x * 4096;
#pragma unroll
  for (int e = 0; e < 8; ++e) out[tid + kT4096 * e] = r[e];
}

// Batched transform: polynomial x of group y is src + y src_stride + x N
// (out: dst, same indexing; in place when src == dst); its modulus is
// x mod `period` (ciphertext arrays: period R; key-switching arrays: R + 1).
__global__ void __launch_bounds__(kRT) rns_ntt_kernel(const uint64_t *src, size_t src_stride,
                                                      uint64_t *dst, size_t dst_stride, int period,
                                                      int inverse, RnsConsts C) {
  extern __shared__ uint64_t sm[];
  const int n = C.n;
  const size_t x = blockIdx.x, y = blockIdx.y;
  const int m = (int)(x % (size_t)period);
  const uint64_t *in = src + y * src_stride + x * n;
  uint64_t *out = dst + y * dst_stride + x * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) sm[i] = in[i];
  __syncthreads();
  if (inverse)
    smem_ntt_inv(sm, C.inv + (size_t)m * n, C.m[m], n);
  else
    smem_ntt_fwd(sm, C.fwd + (size_t)m * n, C.m[m].q, n, C.logn);
  for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = sm[i];
}

// ---------------------------------------------------------------------------
// query expansion (fast_expand_qry, server.cpp:383-428): one level
// ---------------------------------------------------------------------------

// CTA (node, j, m): T = sigma_g(c1 mod q_j) (x -> x^g), lifted to modulus m
// (T < q_j < 2 q_m); the m = 0 CTAs also write sigma_g(c0 mod q_j).
__global__ void __launch_bounds__(kPT) rns_expand_lift_kernel(const uint64_t *cur, uint64_t *lift,
                                                              uint64_t *s0, uint64_t g,
                                                              RnsConsts C) {
  const int n = C.n, R = C.R, M = R + 1;
  const int node = pw_unit(n), j = blockIdx.y, m = blockIdx.z;
  const size_t CT = 2 * (size_t)R * n;
  const uint64_t *c0 = cur + node * CT + (size_t)j * n;
  const uint64_t *c1 = cur + node * CT + (size_t)(R + j) * n;
  const uint64_t qj = C.m[j].q, qm = C.m[m].q;
  uint64_t *L = lift + (((size_t)node * R + j) * M + m) * n;
  uint64_t *S = s0 + ((size_t)node * R + j) * n;
  const uint64_t mask = 2 * (uint64_t)n - 1;
  {
    const int i = pw_coeff(n);
    const uint64_t e = ((uint64_t)i * g) & mask;
    const bool wrap = e >= (uint64_t)n;
    const int d = (int)(wrap ? e - n : e);
    const uint64_t v = wrap ? neg_mod(c1[i], qj) : c1[i];
    L[d] = v >= qm ? v - qm : v;
    if (m == 0) S[d] = wrap ? neg_mod(c0[i], qj) : c0[i];
  }
}

// CTA (node, k, m): X_k mod q_m = sum_j lift[node][j][m] key[j][k][m] (NTT form)
__global__ void __launch_bounds__(kPT) rns_ks_mac_kernel(const uint64_t *lift,
                                                         const uint64_t *key, uint64_t *acc,
                                                         RnsConsts C) {
  const int n = C.n, R = C.R, M = R + 1;
  const int node = pw_unit(n), k = blockIdx.y, m = blockIdx.z;
  uint64_t *A = acc + (((size_t)node * 2 + k) * M + m) * n;
  {
    const int c = pw_coeff(n);
    U128 s{0, 0};
    for (int j = 0; j < R; ++j)
      mac_to(s, lift[(((size_t)node * R + j) * M + m) * n + c], key[(((size_t)j * 2 + k) * M + m) * n + c]);
    A[c] = rmod(s, C.m[m]);
  }
}

// CTA (node, poly, i): the key switch divided by p with rounding,
//   ks = (x_i + p/2 - ((x_p + p/2) mod p)) p^-1 mod q_i,
// galois = (sigma(c0) + ks_0, ks_1), then the two children
//   even = c + galois,  odd = (c - galois) x^-k (negacyclic shift, utils.cpp:6-40).
__global__ void __launch_bounds__(kPT) rns_expand_combine_kernel(const uint64_t *cur,
                                                                 const uint64_t *s0,
                                                                 const uint64_t *acc,
                                                                 uint64_t *nxt, int kshift,
                                                                 RnsConsts C) {
  const int n = C.n, R = C.R, M = R + 1;
  const int node = pw_unit(n), poly = blockIdx.y, i = blockIdx.z;
  const size_t CT = 2 * (size_t)R * n;
  const uint64_t q = C.m[i].q, p = C.m[R].q;
  const uint64_t *xq = acc + (((size_t)node * 2 + poly) * M + i) * n;
  const uint64_t *xp = acc + (((size_t)node * 2 + poly) * M + R) * n;
  const uint64_t *x = cur + node * CT + ((size_t)poly * R + i) * n;
  uint64_t *even = nxt + (2 * (size_t)node) * CT + ((size_t)poly * R + i) * n;
  uint64_t *odd = even + CT;
  {
    const int c = pw_coeff(n);
    const uint64_t r = add_mod(xp[c], C.p_half, p);
    const uint64_t rq = r >= q ? r - q : r;
    uint64_t v = sub_mod(add_mod(xq[c], C.p_half_mod[i], q), rq, q);
    v = mul_shoup(v, C.p_inv[i], C.p_inv_s[i], q);
    const uint64_t gal = poly == 0 ? add_mod(s0[((size_t)node * R + i) * n + c], v, q) : v;
    const uint64_t xc = x[c];
    even[c] = add_mod(xc, gal, q);
    const uint64_t d = sub_mod(xc, gal, q);
    if (c >= kshift)
      odd[c - kshift] = d;
    else
      odd[c - kshift + n] = neg_mod(d, q);
  }
}

// ---------------------------------------------------------------------------
// RGSW external products (gsw_eval.cpp:33-224)
// ---------------------------------------------------------------------------

// decomp_rlwe (gsw_eval.cpp:108-182): CTA (e, poly).  The residues of every
// coefficient of ciphertext e (or of y - x, y at x + sub_off, for folding)
// are composed by CRT into X in [0, Q); the digits (X >> (p b)) & (2^b - 1),
// p = l-1 .. 0, are written to every prime: digits[e][poly l + l-1-p][i][c].
__global__ void __launch_bounds__(kPT) rns_decompose_kernel(const uint64_t *src, size_t ct_stride,
                                                            size_t sub_off, int l, int b,
                                                            uint64_t *digits, RnsConsts C) {
  const int n = C.n, R = C.R;
  const int e = pw_unit(n), poly = blockIdx.y;
  const uint64_t q0 = C.m[0].q, q1 = R > 1 ? C.m[1].q : 0;
  const uint64_t *x = src + (size_t)e * ct_stride + (size_t)poly * R * n;
  const u128 mask = (((u128)1) << b) - 1;
  uint64_t *out = digits + ((size_t)e * 2 * l + (size_t)poly * l) * R * n;
  {
    const int c = pw_coeff(n);
    uint64_t r0 = x[c], r1 = R > 1 ? x[n + c] : 0;
    if (sub_off) {
      r0 = sub_mod(x[sub_off + c], r0, q0);
      if (R > 1) r1 = sub_mod(x[sub_off + n + c], r1, q1);
    }
    u128 X = r0;
    if (R > 1) {
      // X = x_1 + q_1 ((x_0 - x_1) q_1^-1 mod q_0)
      const uint64_t r1q0 = r1 >= q0 ? r1 - q0 : r1;
      const uint64_t d = mul_shoup(sub_mod(r0, r1q0, q0), C.last_inv[0], C.last_inv_s[0], q0);
      X = (u128)q1 * d + r1;
    }
    for (int jj = 0; jj < l; ++jj) {
      const uint64_t v = (uint64_t)((X >> ((l - 1 - jj) * b)) & mask);
      for (int i = 0; i < R; ++i) out[((size_t)jj * R + i) * n + c] = v;
    }
  }
}

// CTA (e, k, i): out_e[k][i] = sum_{j < nd} digits[e][j][i] rows[j][k][i] mod q_i
// (NTT form).  Output ciphertext e sits at out + ((e / grp) grp_stride + off + e % grp) CT.
__global__ void __launch_bounds__(kPT) rns_extprod_mac_kernel(const uint64_t *digits, int nd,
                                                              const uint64_t *rows, uint64_t *out,
                                                              int grp, int grp_stride, int off,
                                                              RnsConsts C) {
  const int n = C.n, R = C.R;
  const int e = pw_unit(n), k = blockIdx.y, i = blockIdx.z;
  const size_t CT = 2 * (size_t)R * n;
  uint64_t *o = out + ((size_t)(e / grp) * grp_stride + off + e % grp) * CT + ((size_t)k * R + i) * n;
  const uint64_t *d = digits + (size_t)e * nd * R * n + (size_t)i * n;
  const uint64_t *g = rows + ((size_t)k * R + i) * n;
  {
    const int c = pw_coeff(n);
    U128 s{0, 0};
    for (int j = 0; j < nd; ++j) mac_to(s, d[(size_t)j * R * n + c], g[(size_t)j * CT + c]);
    o[c] = rmod(s, C.m[i]);
  }
}

// CTA (pair, poly, i): x += e (other_dim_mux's final addition, server.cpp:331)
__global__ void __launch_bounds__(kPT) rns_add_kernel(uint64_t *res, const uint64_t *e,
                                                      RnsConsts C) {
  const int n = C.n, R = C.R;
  const size_t CT = 2 * (size_t)R * n;
  const size_t off = (size_t)pw_unit(n) * CT + ((size_t)blockIdx.y * R + blockIdx.z) * n;
  const uint64_t q = C.m[blockIdx.z].q;
  const int c = pw_coeff(n);
  res[off + c] = add_mod(res[off + c], e[off + c], q);
}

// ---------------------------------------------------------------------------
// first dimension (evaluate_first_dim + mat_mat_128 + delay_modulus,
// server.cpp:124-293, matrix.cpp:220-235)
// ---------------------------------------------------------------------------

__device__ __forceinline__ void add_wide(U128 &a, uint32_t &w, U128 v) {
  asm("add.cc.u64 %0, %0, %3;\n\taddc.cc.u64 %1, %1, %4;\n\taddc.u32 %2, %2, 0;"
      : "+l"(a.lo), "+l"(a.hi), "+r"(w)
      : "l"(v.lo), "l"(v.hi));
}

// x + w 2^128 mod q, exactly (x any 128-bit value)
__device__ __forceinline__ uint64_t reduce_wide(U128 x, uint32_t w, const RnsMod &M,
                                                uint64_t two128) {
  const uint64_t hi = rmod(U128{x.hi, 0}, M);
  uint64_t r = rmod(U128{x.lo, hi}, M);
  if (w) r = add_mod(r, rmod(mul_wide(w, two128), M), M.q);
  return r;
}

// the streaming scan's storage form of a residue < 2^60 (the database
// planes hold it): lo30 | hi30 << 32
__device__ __forceinline__ uint64_t split30(uint64_t v) {
  return (v & 0x3FFFFFFFULL) | ((v >> 30) << 32);
}
__device__ __forceinline__ uint64_t join30(uint64_t w) {
  return (w & 0x3FFFFFFFULL) | ((w >> 32) << 30);
}

// The operand of the streaming scan: qs[(i N + c) n1 + k] = the 30-bit halves
// of qn[k][0][i][c] and qn[k][1][i][c], through a 32 x 32 shared-memory tile
// (reads coalesced along c, writes along k).
__global__ void rns_scan_operand_kernel(const uint64_t *qn, uint4 *qs, int n1, RnsConsts C) {
  __shared__ uint4 tile[32][33];  // [c][k]
  const int n = C.n, R = C.R, i = blockIdx.z;
  const int c0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int kk = threadIdx.y; kk < 32; kk += blockDim.y) {
    const int k = k0 + kk, c = c0 + threadIdx.x;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (k < n1 && c < n) {
      const uint64_t a = qn[((size_t)k * 2 * R + i) * n + c];
      const uint64_t b = qn[((size_t)(k * 2 + 1) * R + i) * n + c];
      v = make_uint4((uint32_t)(a & 0x3FFFFFFFu), (uint32_t)(a >> 30), (uint32_t)(b & 0x3FFFFFFFu),
                     (uint32_t)(b >> 30));
    }
    tile[threadIdx.x][kk] = v;
  }
  __syncthreads();
  for (int cc = threadIdx.y; cc < 32; cc += blockDim.y) {
    const int c = c0 + cc, k = k0 + threadIdx.x;
    if (k < n1 && c < n) qs[((size_t)i * n + c) * n1 + k] = tile[cc][threadIdx.x];
  }
}

// Shapes the streaming scan does not take: CTA (cc = i N + c, row block):
// out[row][poly][i][c] = sum_k db[cc][k][row] qn[k][poly][i][c]
__global__ void rns_scan_kernel(const uint64_t *dbs, const uint64_t *qn, uint64_t *out, int n1,
                                int n_rest, RnsConsts C) {
  extern __shared__ uint64_t sq[];  // [n1][2]
  const int n = C.n, R = C.R;
  const int cc = blockIdx.x, i = cc / n, c = cc % n;
  for (int k = threadIdx.x; k < n1; k += blockDim.x) {
    sq[2 * k] = qn[((size_t)k * 2 + 0) * R * n + cc];
    sq[2 * k + 1] = qn[((size_t)k * 2 + 1) * R * n + cc];
  }
  __syncthreads();
  const int row = blockIdx.y * blockDim.x + threadIdx.x;
  if (row >= n_rest) return;
  const uint64_t *a = dbs + (size_t)cc * n1 * n_rest + row;
  const ulonglong2 *sq2 = reinterpret_cast<const ulonglong2 *>(sq);
  U128 s0{0, 0}, s1{0, 0};
  uint32_t w0 = 0, w1 = 0;
  // eight independent loads ahead of their multiply-adds: the scan is bound
  // by the loads a thread keeps in flight, not by its arithmetic
  int k = 0;
  for (; k + 8 <= n1; k += 8) {
    uint64_t v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = join30(__ldg(a + (size_t)(k + u) * n_rest));
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const ulonglong2 qv = sq2[k + u];
      add_wide(s0, w0, mul_wide(v[u], qv.x));
      add_wide(s1, w1, mul_wide(v[u], qv.y));
    }
  }
  for (; k < n1; ++k) {
    const uint64_t v = join30(__ldg(a + (size_t)k * n_rest));
    const ulonglong2 qv = sq2[k];
    add_wide(s0, w0, mul_wide(v, qv.x));
    add_wide(s1, w1, mul_wide(v, qv.y));
  }
  const size_t CT = 2 * (size_t)R * n;
  out[row * CT + (size_t)i * n + c] = reduce_wide(s0, w0, C.m[i], C.two128[i]);
  out[row * CT + ((size_t)R + i) * n + c] = reduce_wide(s1, w1, C.m[i], C.two128[i]);
}

// ---------------------------------------------------------------------------
// modulus switching (server.cpp:567-570, 779-801) and packing (581-633)
// ---------------------------------------------------------------------------

// one thread per coefficient of the folded ciphertext res [2][R][N]: with two
// primes first SEAL's divide-and-round by q_1, (x_0 + q_1/2 - ((x_1 + q_1/2)
// mod q_1)) q_1^-1 mod q_0; then the x87 switch to small_q.
__global__ void rns_finish_kernel(const uint64_t *res, uint64_t *resp, RnsConsts C) {
  const int n = C.n, R = C.R;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 2 * n) return;
  const int poly = idx / n, c = idx % n;
  const uint64_t *x = res + (size_t)poly * R * n;
  uint64_t v = x[c];
  if (R > 1) {
    const uint64_t q0 = C.m[0].q, q1 = C.m[R - 1].q;
    const uint64_t r = add_mod(x[(size_t)(R - 1) * n + c], C.last_half, q1);
    const uint64_t rq = r >= q0 ? r - q0 : r;
    v = sub_mod(add_mod(v, C.last_half_mod[0], q0), rq, q0);
    v = mul_shoup(v, C.last_inv[0], C.last_inv_s[0], q0);
  }
  resp[idx] = mod_switch_x87(v, C.ms_mant, C.ms_shift);
}

// one thread per output byte: the LSB-first stream of ncoeff coefficients of
// w bits each, every coefficient masked to w bits (server.cpp:603-622);
// status_out: also copy the device status word *status there (every earlier
// kernel of the stream has completed)
__global__ void rns_pack_kernel(const uint64_t *resp, size_t resp_stride, uint8_t *packed,
                                size_t nbytes, int ncoeff, int w, const uint32_t *status,
                                uint32_t *status_out) {
  const size_t byte = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (byte >= nbytes) return;
  if (status_out && byte == 0 && blockIdx.y == 0)
    *status_out = *reinterpret_cast<const volatile uint32_t *>(status);
  const uint64_t *r = resp + blockIdx.y * resp_stride;
  const uint64_t mask = (1ULL << w) - 1;
  uint64_t pos = byte * 8;
  uint32_t out = 0;
  int got = 0;
  while (got < 8) {
    const uint64_t ci = pos / (uint64_t)w;
    if (ci >= (uint64_t)ncoeff) break;
    const int off = (int)(pos % (uint64_t)w);
    const int take = min(8 - got, w - off);
    out |= (uint32_t)(((r[ci] & mask) >> off) & ((1u << take) - 1)) << got;
    got += take;
    pos += take;
  }
  packed[blockIdx.y * nbytes + byte] = (uint8_t)out;
}

// ---------------------------------------------------------------------------
// database ingest (gen_data, push_database_chunk, preprocess_ntt, realign_db:
// server.cpp:47-78, 635-748)
// ---------------------------------------------------------------------------

// coefficient c of plaintext pt0 + blockIdx.x: bits [bpc c, bpc c + bpc) of
// its synthetic entries' bytes (LSB-first, zero past the end)
__global__ void rns_db_gen_kernel(uint64_t seed, size_t pt0, uint64_t *coeffs, int n,
                                  int entry_size, int epp, int bpc) {
  const size_t pt = blockIdx.x;
  const uint64_t total_bytes = (uint64_t)epp * entry_size;
  const u128 mask = (((u128)1) << bpc) - 1;
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    const uint64_t bit0 = (uint64_t)c * bpc, byte0 = bit0 >> 3;
    const int off = (int)(bit0 & 7), nb = (off + bpc + 7) >> 3;
    u128 acc = 0;
    for (int j = 0; j < nb; ++j) {
      const uint64_t by = byte0 + j;
      if (by >= total_bytes) break;
      const uint64_t e = (pt0 + pt) * (uint64_t)epp + by / entry_size;
      acc |= (u128)gen_entry_byte(seed, e, by % entry_size) << (8 * j);
    }
    coeffs[pt * n + c] = (uint64_t)((acc >> off) & mask);
  }
}

// CTA (pt, i): the plaintext lifted centred to q_i (SEAL's
// plain_upper_half_increment: v >= (t+1)/2 -> v + q_i - t), forward NTT,
// scattered into the planes dbs[(i N + c) n1 n_rest + col n_rest + row]
// (pt = row n1 + col, server.cpp:740)
__global__ void __launch_bounds__(kRT) rns_db_ntt_scatter_kernel(const uint64_t *coeffs,
                                                                 size_t pt0, uint64_t *dbs,
                                                                 int n1, int n_rest, RnsConsts C) {
  extern __shared__ uint64_t sm[];
  const int n = C.n, i = blockIdx.y;
  const uint64_t q = C.m[i].q, thr = (C.t + 1) >> 1, inc = q - C.t;
  const uint64_t *src = coeffs + (size_t)blockIdx.x * n;
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    const uint64_t v = src[c];
    sm[c] = v >= thr ? v + inc : v;
  }
  __syncthreads();
  smem_ntt_fwd(sm, C.fwd + (size_t)i * n, q, n, C.logn);
  const size_t pt = pt0 + blockIdx.x, row = pt / n1, col = pt % n1;
  const size_t plane = (size_t)n1 * n_rest;
  for (int c = threadIdx.x; c < n; c += blockDim.x)
    dbs[((size_t)i * n + c) * plane + col * n_rest + row] = split30(sm[c]);
}

// reference layout db_aligned[cc num_pt + row n1 + col] -> planes
__global__ void rns_db_from_aligned_kernel(const uint64_t *aligned, uint64_t *dbs, size_t slots,
                                           int n1, int n_rest) {
  const size_t plane = (size_t)n1 * n_rest, total = plane * slots;
  for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total;
       x += (size_t)gridDim.x * blockDim.x) {
    const size_t cc = x / plane, rem = x % plane, col = rem / n_rest, row = rem % n_rest;
    dbs[x] = split30(aligned[cc * plane + row * n1 + col]);
  }
}

}  // namespace

// ===========================================================================
// host side
// ===========================================================================

int RnsServer::fail(int code, const std::string &msg) {
  err_ = msg;
  return code;
}

int RnsServer::cuda_fail(cudaError_t e, const char *what) {
  cudaGetLastError();
  if (e == cudaErrorMemoryAllocation) return fail(OPIR_ERR_OOM, std::string(what) + ": out of device memory");
  return fail(OPIR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define RCK(call, what)                                      \
  do {                                                       \
    const cudaError_t rce_ = (call);                         \
    if (rce_ != cudaSuccess) return cuda_fail(rce_, what);   \
  } while (0)

RnsServer::~RnsServer() {
  clear_graphs();
  for (auto &e : ev_)
    if (e) cudaEventDestroy(e);
}

RnsServer::Lane::~Lane() {
  if (stream) cudaStreamSynchronize(stream);
  if (h_io_) cudaFreeHost(h_io_);
  if (stream) cudaStreamDestroy(stream);
}

int RnsServer::prepare_lane(Lane &L) {
  if (!L.status_.p) {
    RCK(L.status_.alloc(kStatusWords * sizeof(uint32_t)), "status word");
    RCK(cudaMemset(L.status_.p, 0, kStatusWords * sizeof(uint32_t)), "status word");
  }
  if (!L.h_io_) {
    RCK(cudaMallocHost(&L.h_io_, io_status_off_ + 16), "pinned staging");
    RCK(cudaHostGetDevicePointer(reinterpret_cast<void **>(&L.d_io_), L.h_io_, 0),
        "pinned staging");
    std::memset(L.h_io_, 0, io_status_off_ + 16);
  }
  return OPIR_OK;
}

void RnsServer::clear_graphs() {
  for (auto &g : graphs_cache_)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  graphs_cache_.clear();
}

void RnsServer::set_graphs(bool on) {
  graphs_ = on;
  if (!on) clear_graphs();
}

int RnsServer::create(const opir_rns_params &P, int device, std::unique_ptr<RnsServer> *out,
                      std::string *err) {
  using namespace hostmath;
  auto bad = [&](const char *why) {
    *err = why;
    return OPIR_ERR_ARG;
  };
  const uint32_t n = P.poly_degree, R = P.rns_count;
  if (n < 1024 || n > (uint32_t)kRnsMaxDegree || (n & (n - 1)))
    return bad("poly_degree must be a power of two in [1024, 4096]");
  if (R < 1 || R > (uint32_t)kRnsMaxPrimes) return bad("rns_count must be 1 or 2");
  uint64_t mods[kRnsMaxPrimes + 1];
  unsigned qbits = 0;
  for (uint32_t i = 0; i < R; i++) mods[i] = P.coeff_moduli[i];
  mods[R] = P.special_modulus;
  for (uint32_t m = 0; m <= R; m++) {
    if (!is_prime(mods[m]) || mods[m] >= (1ULL << 60) || mods[m] <= (1ULL << 59) ||
        (mods[m] - 1) % (2 * (uint64_t)n))
      return bad("every modulus must be a prime in (2^59, 2^60) that is 1 mod 2N");
    for (uint32_t j = 0; j < m; j++)
      if (mods[j] == mods[m]) return bad("the moduli must be distinct");
    if (m < R) qbits += bitlen(mods[m]);
  }
  if (!is_prime(P.plain_modulus) || P.plain_modulus < 3 || P.plain_modulus >= mods[R])
    return bad("plain_modulus must be an odd prime below the ciphertext primes");
  if (!is_prime(P.small_modulus) || P.small_modulus >= mods[0] || P.small_modulus < 3)
    return bad("small_modulus must be a prime below q_0");
  if (!P.gsw_l || !P.gsw_l_key || P.gsw_base_log2 == 0 || P.gsw_base_log2_key == 0 ||
      P.gsw_base_log2 > 60 || P.gsw_base_log2_key > 60 ||
      P.gsw_l * P.gsw_base_log2 < qbits || P.gsw_l_key * P.gsw_base_log2_key < qbits ||
      (P.gsw_l - 1) * P.gsw_base_log2 >= 128 || (P.gsw_l_key - 1) * P.gsw_base_log2_key >= 128 ||
      2 * P.gsw_l_key > 20 || P.gsw_l > 15)
    return bad("the gadgets must cover log2 Q (l * base_log2 >= bits of Q) with at most 10 digits");
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    *err = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
    return OPIR_ERR_NO_DEVICE;
  }
  std::unique_ptr<RnsServer> s(new RnsServer());
  s->prm_ = P;
  s->device_ = device;
  RnsConsts &C = s->C_;
  C.n = (int)n;
  C.logn = (int)bitlen(n) - 1;
  C.R = (int)R;
  C.t = P.plain_modulus;
  std::vector<ulonglong2> fwd((size_t)(R + 1) * n), inv((size_t)(R + 1) * n);
  for (uint32_t m = 0; m <= R; m++) {
    const uint64_t q = mods[m];
    const uint64_t psi = minimal_root(q, 2 * (uint64_t)n);
    if (!psi) return bad("no primitive 2N-th root of unity");
    const uint64_t psi_inv = powmod(psi, q - 2, q);
    for (uint32_t i = 0; i < n; i++) {
      const uint64_t ex = brv(i, (unsigned)C.logn);
      const uint64_t w = powmod(psi, ex, q), wi = powmod(psi_inv, ex, q);
      fwd[(size_t)m * n + i] = make_ulonglong2(w, shoup(w, q));
      inv[(size_t)m * n + i] = make_ulonglong2(wi, shoup(wi, q));
    }
    RnsMod &M = C.m[m];
    M.q = q;
    const u128 mu = (~(u128)0) / q;
    M.mu_lo = (uint64_t)mu;
    M.mu_hi = (uint64_t)(mu >> 64);
    M.n_inv = powmod(n, q - 2, q);
    M.n_inv_s = shoup(M.n_inv, q);
  }
  const uint64_t p = mods[R], qL = mods[R - 1];
  C.p_half = p >> 1;
  C.last_half = qL >> 1;
  for (uint32_t i = 0; i < R; i++) {
    const uint64_t q = mods[i];
    C.p_half_mod[i] = C.p_half % q;
    C.p_inv[i] = powmod(p % q, q - 2, q);
    C.p_inv_s[i] = shoup(C.p_inv[i], q);
    C.last_half_mod[i] = C.last_half % q;
    C.last_inv[i] = powmod(qL % q, q - 2, q);
    C.last_inv_s[i] = shoup(C.last_inv[i], q);
    const uint64_t t64 = (uint64_t)((((u128)1) << 64) % q);
    C.two128[i] = mulmod(t64, t64, q);
  }
  {
    // (double)small_q / (double)q_0 == mant 2^-shift (server.cpp:790-795)
    const double scale = (double)P.small_modulus / (double)mods[0];
    int ex;
    const double fr = std::frexp(scale, &ex);
    C.ms_mant = (uint64_t)std::ldexp(fr, 53);
    C.ms_shift = 53 - ex;
    if (C.ms_shift < 1 || C.ms_shift > 126) return bad("small_modulus / q_0 out of range");
  }
  C.small_w = (int)std::ceil(std::log2((double)P.small_modulus));  // server.cpp:587-588
  C.l = (int)P.gsw_l;
  C.b = (int)P.gsw_base_log2;
  C.l_key = (int)P.gsw_l_key;
  C.b_key = (int)P.gsw_base_log2_key;
  s->resp_bytes_ = (2 * (uint64_t)n * C.small_w + 7) / 8;
  const size_t tb = fwd.size() * sizeof(ulonglong2);
  if ((e = s->fwd_.alloc(tb)) != cudaSuccess || (e = s->inv_.alloc(tb)) != cudaSuccess ||
      (e = cudaMemcpy(s->fwd_.p, fwd.data(), tb, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(s->inv_.p, inv.data(), tb, cudaMemcpyHostToDevice)) != cudaSuccess) {
    *err = std::string("NTT tables: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? OPIR_ERR_OOM : OPIR_ERR_CUDA;
  }
  C.fwd = static_cast<const ulonglong2 *>(s->fwd_.p);
  C.inv = static_cast<const ulonglong2 *>(s->inv_.p);
  for (uint32_t i = 0; i < R; i++) {
    const uint64_t q = mods[i];
    Consts &K = s->scan_c_[i];
    K.q = q;
    K.two30 = (1ULL << 30) % q;
    K.two30_s = shoup(K.two30, q);
    K.two60 = (1ULL << 60) % q;
    K.two60_s = shoup(K.two60, q);
    const u128 mu = (~(u128)0) / q;
    s->scan_mu_[i][0] = (uint64_t)mu;
    s->scan_mu_[i][1] = (uint64_t)(mu >> 64);
  }
  {
    // a lane's staging: [query 2 R N words][response 2 N words][packed
    // bytes][status word], each part 16-byte aligned
    auto up16 = [](size_t x) { return (x + 15) / 16 * 16; };
    s->io_resp_off_ = up16(2 * (size_t)R * n * 8);
    s->io_packed_off_ = s->io_resp_off_ + up16(2 * (size_t)n * 8);
    s->io_status_off_ = s->io_packed_off_ + up16(s->resp_bytes_);
    const int lrc = s->prepare_lane(s->lanes_[0]);
    if (lrc) {
      *err = s->err_;
      return lrc;
    }
  }
  for (auto &ev : s->ev_)
    if ((e = cudaEventCreate(&ev)) != cudaSuccess) {
      *err = std::string("events: ") + cudaGetErrorString(e);
      return OPIR_ERR_CUDA;
    }
  if (const char *v = getenv("OPIR_GRAPHS")) s->graphs_ = atoi(v) != 0;
  *out = std::move(s);
  return OPIR_OK;
}

void RnsServer::ntt_launch(const uint64_t *src, size_t src_stride, uint64_t *dst,
                           size_t dst_stride, int polys, int groups, int period, bool inverse,
                           cudaStream_t s) {
  if (polys <= 0 || groups <= 0) return;
  if (C_.n == 4096)
    rns_ntt4096_kernel<<<dim3((unsigned)polys, (unsigned)groups), kT4096, 0, s>>>(
        src, src_stride, dst, dst_stride, period, inverse ? 1 : 0, C_);
  else
    rns_ntt_kernel<<<dim3((unsigned)polys, (unsigned)groups), kRT, (size_t)C_.n * 8, s>>>(
        src, src_stride, dst, dst_stride, period, inverse ? 1 : 0, C_);
  launches_++;
}

int RnsServer::db_create(const opir_db_shape &sh, uint32_t *id) {
  if (!sh.fst_dim_sz || !sh.other_dim_sz || (sh.other_dim_sz & (sh.other_dim_sz - 1)) ||
      !sh.entry_size || !sh.entries_per_pt || !sh.bits_per_coeff || sh.bits_per_coeff > 63 ||
      sh.fst_dim_sz > 4096)
    return fail(OPIR_ERR_ARG, "invalid database shape");
  if ((uint64_t)sh.entries_per_pt * sh.entry_size * 8 > (uint64_t)C_.n * sh.bits_per_coeff)
    return fail(OPIR_ERR_ARG, "entries do not fit a plaintext");
  if ((1ULL << sh.bits_per_coeff) > prm_.plain_modulus)
    return fail(OPIR_ERR_ARG, "bits_per_coeff exceeds the plaintext modulus");
  auto db = std::make_unique<Db>();
  db->shape = sh;
  db->num_pt = (uint64_t)sh.fst_dim_sz * sh.other_dim_sz;
  db->ndim = 1;
  while ((1u << (db->ndim - 1)) < sh.other_dim_sz) db->ndim++;
  db->u = (int)sh.fst_dim_sz + C_.l * (db->ndim - 1);
  db->h = 0;
  while ((1 << db->h) < db->u) db->h++;
  if (db->h > C_.logn) return fail(OPIR_ERR_ARG, "expansion tree deeper than log2 N");
  *id = next_db_++;
  dbs_[*id] = std::move(db);
  return OPIR_OK;
}

int RnsServer::db_destroy(uint32_t id) {
  if (!dbs_.erase(id)) return fail(OPIR_ERR_UNKNOWN_DB, "unknown database");
  return OPIR_OK;
}

int RnsServer::db_fill_synthetic(uint32_t id, uint64_t seed, cudaStream_t s) {
  auto it = dbs_.find(id);
  if (it == dbs_.end()) return fail(OPIR_ERR_UNKNOWN_DB, "unknown database");
  Db &db = *it->second;
  const int n = C_.n, R = C_.R;
  RCK(db.dbs.alloc(db.num_pt * (size_t)R * n * 8), "alloc database");
  const size_t chunk = 4096;
  RCK(coeffs_.alloc(chunk * n * 8), "alloc ingest");
  const opir_db_shape &sh = db.shape;
  for (size_t pt0 = 0; pt0 < db.num_pt; pt0 += chunk) {
    const size_t cnt = db.num_pt - pt0 < chunk ? db.num_pt - pt0 : chunk;
    rns_db_gen_kernel<<<(unsigned)cnt, kPT, 0, s>>>(seed, pt0, coeffs_.u64(), n, (int)sh.entry_size,
                                                   (int)sh.entries_per_pt, (int)sh.bits_per_coeff);
    rns_db_ntt_scatter_kernel<<<dim3((unsigned)cnt, (unsigned)R), kRT, (size_t)n * 8, s>>>(
        coeffs_.u64(), pt0, db.dbs.u64(), (int)sh.fst_dim_sz, (int)sh.other_dim_sz, C_);
    launches_ += 2;
  }
  RCK(cudaGetLastError(), "ingest launch");
  RCK(cudaStreamSynchronize(s), "ingest");
  return OPIR_OK;
}

int RnsServer::db_upload_aligned(uint32_t id, const uint64_t *aligned, cudaStream_t s) {
  auto it = dbs_.find(id);
  if (it == dbs_.end()) return fail(OPIR_ERR_UNKNOWN_DB, "unknown database");
  Db &db = *it->second;
  const size_t words = db.num_pt * (size_t)C_.R * C_.n;
  RCK(db.dbs.alloc(words * 8), "alloc database");
  RnsBuf tmp;
  RCK(tmp.alloc(words * 8), "alloc upload");
  RCK(cudaMemcpyAsync(tmp.p, aligned, words * 8, cudaMemcpyHostToDevice, s), "upload database");
  rns_db_from_aligned_kernel<<<152 * 8, 256, 0, s>>>(tmp.u64(), db.dbs.u64(), (size_t)C_.R * C_.n,
                                                      (int)db.shape.fst_dim_sz,
                                                      (int)db.shape.other_dim_sz);
  launches_++;
  RCK(cudaGetLastError(), "realign launch");
  RCK(cudaStreamSynchronize(s), "upload database");
  return OPIR_OK;
}

int RnsServer::set_galois_key(uint64_t id, const uint64_t *keys, uint32_t levels, cudaStream_t s) {
  if (!levels || levels > (uint32_t)C_.logn) return fail(OPIR_ERR_ARG, "bad Galois key level count");
  auto &cl = clients_[id];
  if (!cl) cl = std::make_unique<Client>();
  const size_t words = (size_t)levels * C_.R * 2 * (C_.R + 1) * C_.n;
  RCK(cl->galois.alloc(words * 8), "alloc Galois keys");
  RCK(cudaMemcpyAsync(cl->galois.p, keys, words * 8, cudaMemcpyHostToDevice, s), "upload Galois keys");
  RCK(cudaStreamSynchronize(s), "upload Galois keys");
  cl->levels = levels;
  cl->has_galois = true;
  return OPIR_OK;
}

int RnsServer::set_gsw_key(uint64_t id, const uint64_t *rows, cudaStream_t s) {
  auto &cl = clients_[id];
  if (!cl) cl = std::make_unique<Client>();
  const int R = C_.R, n = C_.n;
  const size_t words = (size_t)2 * C_.l_key * 2 * R * n;
  RCK(cl->gsw.alloc(words * 8), "alloc RGSW key");
  RCK(cudaMemcpyAsync(cl->gsw.p, rows, words * 8, cudaMemcpyHostToDevice, s), "upload RGSW key");
  // server.cpp:497: the rows to NTT form, every prime
  ntt_launch(cl->gsw.u64(), 0, cl->gsw.u64(), 0, 2 * C_.l_key * 2 * R, 1, R, false, s);
  RCK(cudaGetLastError(), "RGSW key transform");
  RCK(cudaStreamSynchronize(s), "upload RGSW key");
  cl->has_gsw = true;
  return OPIR_OK;
}

int RnsServer::erase_client(uint64_t id) {
  if (!clients_.erase(id)) return fail(OPIR_ERR_UNKNOWN_CLIENT, "unknown client");
  return OPIR_OK;
}

int RnsServer::ensure_workspace(Lane &L, const Db &db) {
  const size_t n = C_.n, R = C_.R, M = R + 1, CT = 2 * R * n;
  const size_t w = (size_t)1 << db.h;
  const size_t n1 = db.shape.fst_dim_sz, nr = db.shape.other_dim_sz;
  const size_t live = (w + 1) / 2;  // nodes of the widest level
  const size_t cts = (size_t)(db.ndim > 1 ? db.ndim - 1 : 1) * C_.l;
  RCK(L.exp0_.alloc(w * CT * 8), "alloc expansion");
  RCK(L.exp1_.alloc(w * CT * 8), "alloc expansion");
  RCK(L.lift_.alloc(live * R * M * n * 8), "alloc key switching");
  RCK(L.acc_.alloc(live * 2 * M * n * 8), "alloc key switching");
  RCK(L.s0_.alloc(live * R * n * 8), "alloc key switching");
  RCK(L.gsw_.alloc(cts * 2 * CT * 8), "alloc RGSW rows");
  const size_t dig = std::max(cts * 2 * C_.l_key, (nr / 2 ? nr / 2 : 1) * 2 * C_.l);
  RCK(L.digits_.alloc(dig * R * n * 8), "alloc digits");
  RCK(L.qn_.alloc(n1 * CT * 8), "alloc query operand");
  RCK(L.scan_qs_.alloc(R * n * n1 * 16), "alloc scan operand");
  RCK(L.res_.alloc(nr * CT * 8), "alloc first-dimension result");
  RCK(L.e_.alloc((nr / 2 ? nr / 2 : 1) * CT * 8), "alloc folding");
  return OPIR_OK;
}

int RnsServer::enqueue_query(Lane &L, Db &db, Client &cl, const RnsTrace *trace,
                             bool timed, cudaStream_t s) {
  const int n = C_.n, R = C_.R, M = R + 1;
  const int nch = n / kPT;  // coefficient chunks of the pointwise kernels
  const size_t CT = 2 * (size_t)R * n;
  const int h = db.h, u = db.u, l = C_.l, lk = C_.l_key;
  const size_t w = (size_t)1 << h;
  const int n1 = (int)db.shape.fst_dim_sz, nr = (int)db.shape.other_dim_sz;
  auto mark = [&](int i) {
    if (timed) cudaEventRecord(ev_[i], s);
  };
  mark(0);
  // ---- expansion (fast_expand_qry): live nodes of level a are those whose
  // subtree holds one of the u useful leaves
  const uint64_t *cur = reinterpret_cast<const uint64_t *>(L.d_io_);
  uint64_t *bufs[2] = {L.exp0_.u64(), L.exp1_.u64()};
  const size_t key_level = (size_t)R * 2 * M * n;
  for (int a = 0; a < h; a++) {
    const int live = (int)((u + ((size_t)1 << (h - a)) - 1) >> (h - a));
    const int k = 1 << a;
    const uint64_t g = (uint64_t)n / k + 1;
    uint64_t *nxt = bufs[a & 1];
    if (n == 4096) {
      // the lift fused into the forward transforms, the key-switch sums into
      // the inverse ones
      const uint64_t ginv = hostmath::powmod(g, (uint64_t)n - 1, 2 * (uint64_t)n);  // g odd
      rns_expand_lift_ntt4096_kernel<<<live * R * M, kT4096, 0, s>>>(cur, L.lift_.u64(), L.s0_.u64(),
                                                                     ginv, C_);
      rns_ks_intt4096_kernel<<<live * 2 * M, kT4096, 0, s>>>(
          L.lift_.u64(), cl.galois.u64() + a * key_level, L.acc_.u64(), C_);
      launches_ += 2;
    } else {
      rns_expand_lift_kernel<<<dim3(live * nch, R, M), kPT, 0, s>>>(cur, L.lift_.u64(), L.s0_.u64(), g,
                                                                   C_);
      ntt_launch(L.lift_.u64(), 0, L.lift_.u64(), 0, live * R * M, 1, M, false, s);
      rns_ks_mac_kernel<<<dim3(live * nch, 2, M), kPT, 0, s>>>(
          L.lift_.u64(), cl.galois.u64() + a * key_level, L.acc_.u64(), C_);
      ntt_launch(L.acc_.u64(), 0, L.acc_.u64(), 0, live * 2 * M, 1, M, true, s);
      launches_ += 2;
    }
    rns_expand_combine_kernel<<<dim3(live * nch, 2, R), kPT, 0, s>>>(cur, L.s0_.u64(), L.acc_.u64(), nxt, k, C_);
    launches_ += 1;
    cur = nxt;
  }
  const uint64_t *leaves = cur;
  mark(1);
  // ---- RGSW reconstruction (query_to_gsw, gsw_eval.cpp:254-286): per
  // further dimension, rows 0..l-1 = NTT of its l leaves, rows l..2l-1 =
  // RGSW(sk) (x) leaf with the key gadget
  if (db.ndim > 1) {
    const int E = (db.ndim - 1) * l;  // ciphertexts
    const uint64_t *first = leaves + (size_t)n1 * CT;
    ntt_launch(first, (size_t)l * CT, L.gsw_.u64(), (size_t)2 * l * CT, l * 2 * R, db.ndim - 1, R,
               false, s);
    rns_decompose_kernel<<<dim3(E * nch, 2), kPT, 0, s>>>(first, CT, 0, lk, C_.b_key, L.digits_.u64(), C_);
    ntt_launch(L.digits_.u64(), 0, L.digits_.u64(), 0, E * 2 * lk * R, 1, R, false, s);
    rns_extprod_mac_kernel<<<dim3(E * nch, 2, R), kPT, 0, s>>>(L.digits_.u64(), 2 * lk, cl.gsw.u64(),
                                                        L.gsw_.u64(), l, 2 * l, l, C_);
    launches_ += 2;
  }
  mark(2);
  // ---- first dimension: NTT of the n1 selection ciphertexts, the scan,
  // the inverse NTT of the n_rest results
  ntt_launch(leaves, 0, L.qn_.u64(), 0, n1 * 2 * R, 1, R, false, s);
  {
    // the one-modulus streaming scan over both primes' planes (bulk copies
    // into a shared-memory ring, 30-bit half products), where the shape fits
    bool streamed = false;
    if (nr >= 2 && n1 % 8 == 0) {
      rns_scan_operand_kernel<<<dim3((n + 31) / 32, (n1 + 31) / 32, R), dim3(32, 8), 0, s>>>(
          L.qn_.u64(), static_cast<uint4 *>(L.scan_qs_.p), n1, C_);
      launches_++;
      mark(6);
      // the R N planes of both primes in one launch (slot i N + c reduces mod q_i)
      streamed = launch_scan_planes(db.dbs.u64(), static_cast<const uint4 *>(L.scan_qs_.p),
                                    (size_t)R * n * n1, L.res_.u64(), (size_t)nr * CT, n1, nr, 1,
                                    R * n, CT, (size_t)R * n, n, scan_c_[0], scan_mu_[0],
                                    scan_c_[R - 1], scan_mu_[R - 1],
                                    static_cast<uint32_t *>(L.status_.p), s) >= 0;
      if (streamed) launches_++;
    }
    if (!streamed) {
      mark(6);
      int bd = ((nr + 31) / 32) * 32;
      if (bd > 256) bd = 256;
      rns_scan_kernel<<<dim3(R * n, (nr + bd - 1) / bd), bd, (size_t)n1 * 16, s>>>(
          db.dbs.u64(), L.qn_.u64(), L.res_.u64(), n1, nr, C_);
      launches_++;
    }
    mark(7);
  }
  ntt_launch(L.res_.u64(), 0, L.res_.u64(), 0, nr * 2 * R, 1, R, true, s);
  mark(3);
  if (trace && trace->first_dim)
    RCK(cudaMemcpyAsync(trace->first_dim, L.res_.p, (size_t)nr * CT * 8, cudaMemcpyDeviceToHost, s),
        "trace");
  // ---- further dimensions (other_dim_mux)
  int cnt = nr;
  for (int d = 1; d < db.ndim; d++) {
    const int half = cnt / 2;
    const uint64_t *sel = L.gsw_.u64() + (size_t)(d - 1) * 2 * l * CT;
    rns_decompose_kernel<<<dim3(half * nch, 2), kPT, 0, s>>>(L.res_.u64(), CT, (size_t)half * CT, l, C_.b,
                                                      L.digits_.u64(), C_);
    ntt_launch(L.digits_.u64(), 0, L.digits_.u64(), 0, half * 2 * l * R, 1, R, false, s);
    rns_extprod_mac_kernel<<<dim3(half * nch, 2, R), kPT, 0, s>>>(L.digits_.u64(), 2 * l, sel, L.e_.u64(), 1,
                                                           1, 0, C_);
    ntt_launch(L.e_.u64(), 0, L.e_.u64(), 0, half * 2 * R, 1, R, true, s);
    rns_add_kernel<<<dim3(half * nch, 2, R), kPT, 0, s>>>(L.res_.u64(), L.e_.u64(), C_);
    launches_ += 3;
    cnt = half;
  }
  mark(4);
  // ---- modulus switches and packing
  uint64_t *d_resp = reinterpret_cast<uint64_t *>(L.d_io_ + io_resp_off_);
  rns_finish_kernel<<<(2 * n + kPT - 1) / kPT, kPT, 0, s>>>(L.res_.u64(), d_resp, C_);
  rns_pack_kernel<<<dim3((unsigned)((resp_bytes_ + kPT - 1) / kPT), 1), kPT, 0, s>>>(
      d_resp, 2 * (size_t)n, L.d_io_ + io_packed_off_, resp_bytes_, 2 * n, C_.small_w,
      static_cast<const uint32_t *>(L.status_.p), reinterpret_cast<uint32_t *>(L.d_io_ + io_status_off_));
  launches_ += 2;
  mark(5);
  if (trace) {
    if (trace->leaves)
      RCK(cudaMemcpyAsync(trace->leaves, leaves, (size_t)u * CT * 8, cudaMemcpyDeviceToHost, s), "trace");
    if (trace->gsw && db.ndim > 1)
      RCK(cudaMemcpyAsync(trace->gsw, L.gsw_.p, (size_t)(db.ndim - 1) * 2 * l * CT * 8,
                          cudaMemcpyDeviceToHost, s),
          "trace");
  }
  (void)w;
  return OPIR_OK;
}

int RnsServer::check_query(Db &db, uint64_t client, Client **out) {
  if (!db.dbs.p) return fail(OPIR_ERR_STATE, "database has no data");
  auto cit = clients_.find(client);
  if (cit == clients_.end() || !cit->second->has_galois)
    return fail(OPIR_ERR_UNKNOWN_CLIENT, "no Galois keys for client " + std::to_string(client));
  Client &cl = *cit->second;
  if (cl.levels < (uint32_t)db.h)
    return fail(OPIR_ERR_ARG, "the client's Galois keys have too few levels for this database");
  if (db.ndim > 1 && !cl.has_gsw)
    return fail(OPIR_ERR_UNKNOWN_CLIENT, "no RGSW key for client " + std::to_string(client));
  *out = &cl;
  return OPIR_OK;
}

int RnsServer::start_query(Lane &L, Db &db, Client &cl, const uint64_t *query,
                           const RnsTrace *trace, bool timed, cudaStream_t s) {
  const size_t CT = 2 * (size_t)C_.R * C_.n;
  std::memcpy(L.h_io_, query, CT * 8);  // nothing of this lane is in flight
  if (graphs_ && !trace && !timed) {
    // every pointer and shape the kernels take: a graph whose key matches
    // launches exactly what enqueue_query would
    const std::vector<uint64_t> key = {
        (uint64_t)db.dbs.p, (uint64_t)cl.galois.p, (uint64_t)cl.gsw.p, (uint64_t)db.h,
        (uint64_t)db.u, (uint64_t)db.ndim, db.shape.fst_dim_sz, db.shape.other_dim_sz,
        (uint64_t)L.exp0_.p, (uint64_t)L.exp1_.p, (uint64_t)L.lift_.p, (uint64_t)L.acc_.p,
        (uint64_t)L.s0_.p, (uint64_t)L.gsw_.p, (uint64_t)L.digits_.p, (uint64_t)L.qn_.p,
        (uint64_t)L.scan_qs_.p, (uint64_t)L.res_.p, (uint64_t)L.e_.p, (uint64_t)L.d_io_,
        (uint64_t)L.status_.p};
    Graph *hit = nullptr;
    for (auto &g : graphs_cache_)
      if (g.key == key) hit = &g;
    if (!hit) {
      cudaGraph_t graph = nullptr;
      const uint64_t before = launches_;
      cudaError_t ce = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
      int erc = ce == cudaSuccess ? enqueue_query(L, db, cl, nullptr, false, s) : OPIR_ERR_CUDA;
      if (ce == cudaSuccess) ce = cudaStreamEndCapture(s, &graph);
      cudaGraphExec_t exec = nullptr;
      if (!erc && ce == cudaSuccess && graph)
        ce = cudaGraphInstantiate(&exec, graph, 0);
      if (graph) cudaGraphDestroy(graph);
      const uint64_t captured = launches_ - before;
      launches_ = before;
      if (!erc && ce == cudaSuccess && exec) {
        if ((int)graphs_cache_.size() < kMaxGraphs) {
          graphs_cache_.emplace_back();
          hit = &graphs_cache_.back();
        } else {
          hit = &graphs_cache_[0];
          for (auto &g : graphs_cache_)
            if (g.used < hit->used) hit = &g;
          cudaGraphExecDestroy(hit->exec);
        }
        hit->key = key;
        hit->exec = exec;
        hit->launches = captured;
      } else {
        // capture failed: launch the kernels directly
        if (exec) cudaGraphExecDestroy(exec);
        cudaGetLastError();
      }
    }
    if (hit) {
      hit->used = ++graph_clock_;
      RCK(cudaGraphLaunch(hit->exec, s), "query graph");
      launches_ += hit->launches;
    } else {
      const int rc2 = enqueue_query(L, db, cl, nullptr, false, s);
      if (rc2) return rc2;
    }
  } else {
    const int rc2 = enqueue_query(L, db, cl, trace, timed, s);
    if (rc2) return rc2;
  }
  RCK(cudaGetLastError(), "query launch");
  return OPIR_OK;
}

int RnsServer::finish_query(Lane &L, uint64_t *resp, uint8_t *packed, cudaStream_t s) {
  RCK(cudaStreamSynchronize(s), "query");
  {
    // a bounded device wait of the scan that gave up (async.cuh): the pack
    // kernel copied the status word next to the response
    const uint32_t st = *reinterpret_cast<const volatile uint32_t *>(
        static_cast<uint8_t *>(L.h_io_) + io_status_off_);
    if (st) {
      RCK(cudaMemset(L.status_.p, 0, sizeof st), "clear status");
      char b[16];
      snprintf(b, sizeof b, "%x", st);
      return fail(OPIR_ERR_TIMEOUT, std::string("device pipeline wait timed out (status 0x") + b + ")");
    }
  }
  const uint8_t *io = static_cast<const uint8_t *>(L.h_io_);
  if (resp) std::memcpy(resp, io + io_resp_off_, 2 * (size_t)C_.n * 8);
  if (packed) std::memcpy(packed, io + io_packed_off_, resp_bytes_);
  return OPIR_OK;
}

int RnsServer::make_query(uint32_t db_id, uint64_t client, const uint64_t *query, uint64_t *resp,
                          uint8_t *packed, const RnsTrace *trace, cudaStream_t s) {
  auto dit = dbs_.find(db_id);
  if (dit == dbs_.end()) return fail(OPIR_ERR_UNKNOWN_DB, "unknown database");
  Db &db = *dit->second;
  Client *cl = nullptr;
  int rc = check_query(db, client, &cl);
  if (rc) return rc;
  Lane &L = lanes_[0];
  rc = ensure_workspace(L, db);
  if (rc) return rc;
  const bool timed = timing_ && !trace;
  rc = start_query(L, db, *cl, query, trace, timed, s);
  if (!rc) rc = finish_query(L, resp, packed, s);
  stage_valid_ = timed && !rc;
  return rc;
}

int RnsServer::make_query_batch(uint32_t db_id, uint32_t batch, const uint64_t *clients,
                                const uint64_t *queries, uint64_t *resps, uint8_t *packed,
                                cudaStream_t s) {
  if (batch == 0) return OPIR_OK;
  auto dit = dbs_.find(db_id);
  if (dit == dbs_.end()) return fail(OPIR_ERR_UNKNOWN_DB, "unknown database");
  Db &db = *dit->second;
  std::vector<Client *> cls(batch);
  for (uint32_t b = 0; b < batch; ++b) {
    const int rc = check_query(db, clients[b], &cls[b]);
    if (rc) return rc;
  }
  const int nl = batch < (uint32_t)kLanes ? (int)batch : kLanes;
  for (int i = 0; i < nl; ++i) {
    Lane &L = lanes_[i];
    int rc = prepare_lane(L);
    if (!rc) rc = ensure_workspace(L, db);
    if (rc) return rc;
    if (i > 0 && !L.stream)
      RCK(cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking), "lane stream");
  }
  RCK(cudaStreamSynchronize(s), "batch");  // keys and database written on s are in place
  const size_t CT = 2 * (size_t)C_.R * C_.n, rw = 2 * (size_t)C_.n;
  auto stream_of = [&](int i) { return i == 0 ? s : lanes_[i].stream; };
  std::vector<long long> pending(nl, -1);
  int first = OPIR_OK;
  auto finish = [&](int i) {
    const long long b = pending[i];
    pending[i] = -1;
    const int rc = finish_query(lanes_[i], resps ? resps + b * rw : nullptr,
                                packed ? packed + b * resp_bytes_ : nullptr, stream_of(i));
    if (rc && !first) first = rc;
  };
  // a lane takes its next query as soon as its previous one is out
  for (uint32_t b = 0; b < batch && !first; ++b) {
    const int i = (int)(b % (uint32_t)nl);
    if (pending[i] >= 0) finish(i);
    if (first) break;
    const int rc = start_query(lanes_[i], db, *cls[b], queries + (size_t)b * CT, nullptr, false,
                               stream_of(i));
    if (rc) {
      first = rc;
      break;
    }
    pending[i] = b;
  }
  for (int i = 0; i < nl; ++i)
    if (pending[i] >= 0) finish(i);
  stage_valid_ = false;
  return first;
}

bool RnsServer::stage_times(float *ms6) const {
  if (!stage_valid_) return false;
  const int pairs[6][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 4}, {4, 5}, {6, 7}};
  for (int i = 0; i < 6; i++)
    if (cudaEventElapsedTime(&ms6[i], ev_[pairs[i][0]], ev_[pairs[i][1]]) != cudaSuccess) return false;
  return true;
}

int RnsServer::ntt(int mod, bool inverse, uint64_t *polys, uint64_t count, cudaStream_t s) {
  if (mod < 0 || mod > C_.R) return fail(OPIR_ERR_ARG, "modulus index out of range");
  if (!count) return OPIR_OK;
  const size_t bytes = count * (size_t)C_.n * 8;
  RnsBuf d;
  RCK(d.alloc(bytes), "alloc");
  RCK(cudaMemcpyAsync(d.p, polys, bytes, cudaMemcpyHostToDevice, s), "upload");
  // a period larger than the count keeps every polynomial on modulus `mod`:
  // shift the table view instead
  RnsConsts C = C_;
  C.m[0] = C_.m[mod];
  C.fwd = C_.fwd + (size_t)mod * C_.n;
  C.inv = C_.inv + (size_t)mod * C_.n;
  rns_ntt_kernel<<<dim3((unsigned)count, 1), kRT, (size_t)C_.n * 8, s>>>(
      d.u64(), 0, d.u64(), 0, 1, inverse ? 1 : 0, C);
  launches_++;
  RCK(cudaGetLastError(), "ntt launch");
  RCK(cudaMemcpyAsync(polys, d.p, bytes, cudaMemcpyDeviceToHost, s), "download");
  RCK(cudaStreamSynchronize(s), "ntt");
  return OPIR_OK;
}

int RnsServer::pack_response(const uint64_t *resps, uint32_t count, uint8_t *packed,
                             cudaStream_t s) {
  const size_t in = (size_t)count * 2 * C_.n * 8, out = (size_t)count * resp_bytes_;
  RnsBuf din, dout;
  RCK(din.alloc(in), "alloc");
  RCK(dout.alloc(out), "alloc");
  RCK(cudaMemcpyAsync(din.p, resps, in, cudaMemcpyHostToDevice, s), "upload");
  rns_pack_kernel<<<dim3((unsigned)((resp_bytes_ + kPT - 1) / kPT), count), kPT, 0, s>>>(
      din.u64(), 2 * (size_t)C_.n, static_cast<uint8_t *>(dout.p), resp_bytes_, 2 * C_.n,
      C_.small_w, (const uint32_t *)nullptr, (uint32_t *)nullptr);
  launches_++;
  RCK(cudaGetLastError(), "pack launch");
  RCK(cudaMemcpyAsync(packed, dout.p, out, cudaMemcpyDeviceToHost, s), "download");
  RCK(cudaStreamSynchronize(s), "pack");
  return OPIR_OK;
}

}  // namespace opir
