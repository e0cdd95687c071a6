// tree.cu -- the tree-shaped stages of PirServer::make_query on sm_103a:
// query expansion (fast_expand_qry, server.cpp:383-428), RGSW
// reconstruction (query_to_gsw, gsw_eval.cpp:254-286) and folding of the
// further dimensions (other_dim_mux, server.cpp:295-334).
//
// Each stage has a one-CTA form, which gives a whole ciphertext to one CTA of
// 256 threads (least total work; used when a launch has many ciphertexts),
// and cluster forms, which split one ciphertext's independent NTTs over a
// thread-block cluster and combine the partial results through distributed
// shared memory: that shortens the dependent chain of NTTs per tree level
// where latency dominates.  Expansion and folding have a wide cluster (4 and
// 5 CTAs, the narrowest levels) and a pair form (2 CTAs, levels in between);
// a cluster launch pays off only while it fits one wave (a cluster's CTAs
// share a GPC), which sets the thresholds below.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>

#include "common.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace opir {

namespace {

constexpr int T = kNttThreads;

// ---------------------------------------------------------------------------
// expansion: one level of fast_expand_qry (server.cpp:383-428)
//   c' = apply_galois(c_i, N/k + 1)   (automorphism + key switch with p)
//   c_2i = c_i + c';  c_2i+1 = (c_i - c') * x^-k
// ---------------------------------------------------------------------------
//
// One CTA per node.  The key switch runs modulus by modulus so that only one
// transform operand is live at a time (two CTAs fit on an SM): the q part
// leaves INTT(NTT_q(sigma(c1)) * K_q[kk]) in shared memory, the p part then
// rounds against it and writes polynomial kk of both children.
__global__ void __launch_bounds__(T, 2) expand_level_kernel(const uint64_t *cur, uint64_t *nxt,
                                                            size_t in_stride, size_t out_stride,
                                                            const __grid_constant__ KeyBatch kb,
                                                            int level, ModTab Mq, ModTab Mp,
                                                            Consts C) {
  extern __shared__ uint64_t smem[];
  uint64_t *sa = smem, *sb = smem + kSmemPoly;
  uint64_t *s_sig0 = smem + 2 * kSmemPoly;  // sigma(c0), natural index
  uint64_t *s_sig1 = s_sig0 + kN;           // sigma(c1)
  uint64_t *s_q = s_sig1 + kN;              // [2][N] q part of the key switch, natural index
  const int tid = threadIdx.x;
  const int node = blockIdx.x, b = blockIdx.y;
  const int k = 1 << level;
  const uint64_t g = (uint64_t)(kN / k + 1);
  const uint64_t q = C.q, p = C.p;
  const uint64_t *ci = cur + b * in_stride + (size_t)node * 2 * kN;
  grid_dep_sync();

  // automorphism x -> x^g on both polynomials (scatter to shared memory)
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int i = strided_idx(tid, e);
    const uint32_t j = (uint32_t)(((uint64_t)i * g) & (2 * kN - 1));
    const uint64_t v0 = ci[i], v1 = ci[kN + i];
    if (j < (uint32_t)kN) {
      s_sig0[j] = v0;
      s_sig1[j] = v1;
    } else {
      s_sig0[j - kN] = neg_mod(v0, q);
      s_sig1[j - kN] = neg_mod(v1, q);
    }
  }
  __syncthreads();

  const uint64_t *key = kb.q[b].galois + (size_t)level * 4 * kN;
  const uint64_t *key_s = kb.q[b].galois_s + (size_t)level * 4 * kN;
  // ---- modulus q: s_q[kk] = INTT_q(NTT_q(sigma(c1)) * K[kk] mod q)
  // (Shoup products with the keys' precomputed companions, in [0, 4q): the
  // inverse transform takes inputs below 4q)
  {
    uint64_t t[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) t[e] = s_sig1[strided_idx(tid, e)];
    ntt_fwd(t, sa, sb, Mq);
#pragma unroll 1
    for (int kk = 0; kk < 2; ++kk) {
      uint64_t a[8], as[8];
      ldg_slot8(key + (2 * kk) * kN, a);
      ldg_slot8(key_s + (2 * kk) * kN, as);
#pragma unroll
      for (int e = 0; e < 8; ++e) a[e] = mul_shoup_lazy4(t[e], a[e], as[e], Mq.q);
      ntt_inv(a, sa, sb, Mq);
#pragma unroll
      for (int e = 0; e < 8; ++e) s_q[kk * kN + strided_idx(tid, e)] = a[e];  // own slots only
    }
  }
  // ---- modulus p, rounding and the children
  uint64_t *ce = nxt + b * out_stride + (size_t)(2 * node) * 2 * kN;
  uint64_t *co = ce + 2 * kN;
  uint64_t t[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const uint64_t v = s_sig1[strided_idx(tid, e)];
    t[e] = v >= p ? v - p : v;  // q < 2p
  }
  ntt_fwd(t, sa, sb, Mp);
#pragma unroll 1
  for (int kk = 0; kk < 2; ++kk) {
    uint64_t a[8], as[8];
    ldg_slot8(key + (2 * kk + 1) * kN, a);
    ldg_slot8(key_s + (2 * kk + 1) * kN, as);
#pragma unroll
    for (int e = 0; e < 8; ++e) a[e] = mul_shoup_lazy4(t[e], a[e], as[e], Mp.q);
    ntt_inv(a, sa, sb, Mp);
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int i = strided_idx(tid, e);
      // round(X / p) mod q = (x_q + p/2 - ((x_p + p/2) mod p)) * p^-1 mod q
      const uint64_t rr = add_mod(a[e], C.p_half, p);
      const uint64_t v = sub_mod(add_mod(s_q[kk * kN + i], C.p_half_mod_q, q), rr, q);
      const uint64_t o = mul_shoup(v, C.p_inv_q, C.p_inv_q_s, q);
      // polynomial kk of c' = apply_galois(c_i); children c_i +- c' (the odd one times x^-k)
      const uint64_t cp = kk == 0 ? add_mod(s_sig0[i], o, q) : o;
      const uint64_t x = ci[kk * kN + i];
      ce[kk * kN + i] = add_mod(x, cp, q);
      const uint64_t d = sub_mod(x, cp, q);
      // multiply by x^-k (utils.cpp:6-26): coefficient i moves to i - k, wrapping
      // ones are negated (zero stays zero)
      if (i >= k)
        co[kk * kN + i - k] = d;
      else
        co[kk * kN + kN - k + i] = neg_mod(d, q);
    }
  }
}

// ---------------------------------------------------------------------------
// RGSW external product core (gsw_eval.cpp:33-106, 184-252):
// decompose both polynomials of ct (coefficient form, in shared memory at
// natural index; each thread reads only its own strided slots) into l digits
// of base_log2 bits each, NTT every digit, and accumulate digit_j * gsw[j][k]
// in 128 bits; reduce mod q.  Output: NTT form, slot distribution.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void ext_product_core(const uint64_t *src, const uint64_t *gsw, int l,
                                                 int base_log2, uint64_t *sa, uint64_t *sb,
                                                 const ulonglong2 *s_fwd, const ModTab &M,
                                                 uint64_t out[2][8]) {
  const int tid = threadIdx.x;
  const uint64_t mask = (1ULL << base_log2) - 1;
  U128 acc0[8], acc1[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) acc0[e] = acc1[e] = U128{0, 0};
#pragma unroll 1
  for (int poly = 0; poly < 2; ++poly) {
#pragma unroll 1
    for (int pp = l - 1; pp >= 0; --pp) {
      const int j = poly * l + (l - 1 - pp);
      const int sh = pp * base_log2;
      uint64_t d[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) d[e] = (src[poly * kN + strided_idx(tid, e)] >> sh) & mask;
      ntt_fwd_s(d, sa, sb, s_fwd, M);
      const uint64_t *g0 = gsw + (size_t)j * 2 * kN, *g1 = g0 + kN;
      uint64_t w0[8], w1[8];
      ldg_slot8(g0, w0);
      ldg_slot8(g1, w1);
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        mac_to(acc0[e], d[e], w0[e]);
        mac_to(acc1[e], d[e], w1[e]);
      }
    }
  }
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    out[0][e] = barrett128(acc0[e], M.q, M.mu_lo, M.mu_hi);
    out[1][e] = barrett128(acc1[e], M.q, M.mu_lo, M.mu_hi);
  }
}

// query_to_gsw (gsw_eval.cpp:254-286) for every leaf n1 + j, j < num_cts:
// row (j % l) of RGSW (j / l) = NTT(ct); row l + (j % l) = RGSW(sk) x ct.
__global__ void __launch_bounds__(T, 2) query_to_gsw_kernel(const uint64_t *leaves,
                                                            size_t leaves_stride,
                                                            uint64_t *gsw_out, size_t gsw_stride,
                                                            const __grid_constant__ KeyBatch kb,
                                                            int n1, ModTab M, Consts C) {
  extern __shared__ uint64_t smem[];
  uint64_t *sa = smem, *sb = smem + kSmemPoly, *sx = smem + 2 * kSmemPoly;  // sx: [2][N]
  ulonglong2 *s_fwd = reinterpret_cast<ulonglong2 *>(sx + 2 * kN);
  prefetch_tw(s_fwd, M.fwd);
  grid_dep_sync();
  const int tid = threadIdx.x;
  const int j = blockIdx.x, b = blockIdx.y;
  const int l = C.l;
  const int dim = j / l, kk = j % l;
  const uint64_t *ct = leaves + b * leaves_stride + (size_t)(n1 + j) * 2 * kN;
  uint64_t *rgsw = gsw_out + b * gsw_stride + (size_t)dim * 2 * l * 2 * kN;
  // first half: the ciphertext itself in NTT form
  uint64_t *row0 = rgsw + (size_t)kk * 2 * kN;
  tw_wait();
#pragma unroll 1
  for (int poly = 0; poly < 2; ++poly) {
    uint64_t r[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int i = poly * kN + strided_idx(tid, e);
      r[e] = ct[i];
      sx[i] = r[e];  // own slots only
    }
    ntt_fwd_s(r, sa, sb, s_fwd, M);
    stg_slot8(row0 + poly * kN, r);
  }
  // second half: external product with RGSW(sk) under the key gadget
  uint64_t out[2][8];
  ext_product_core(sx, kb.q[b].gsw_key, C.l_key, C.base_log2_key, sa, sb, s_fwd, M, out);
  uint64_t *row1 = rgsw + (size_t)(l + kk) * 2 * kN;
#pragma unroll
  for (int poly = 0; poly < 2; ++poly) stg_slot8(row1 + poly * kN, out[poly]);
}

// other_dim_mux (server.cpp:295-334) for pair j: y -= x; y = RGSW x y; y =
// INTT(y); x += y.
__global__ void __launch_bounds__(T, 2) fold_kernel(uint64_t *res, size_t res_stride,
                                                    const uint64_t *gsw, size_t gsw_stride,
                                                    int half, ModTab M, Consts C) {
  extern __shared__ uint64_t smem[];
  uint64_t *sa = smem, *sb = smem + kSmemPoly, *sd = smem + 2 * kSmemPoly;  // sd: [2][N]
  ulonglong2 *s_fwd = reinterpret_cast<ulonglong2 *>(sd + 2 * kN);
  prefetch_tw(s_fwd, M.fwd);
  grid_dep_sync();
  const int tid = threadIdx.x;
  const int j = blockIdx.x, b = blockIdx.y;
  const uint64_t q = C.q;
  uint64_t *xp = res + b * res_stride + (size_t)j * 2 * kN;
  const uint64_t *yp = res + b * res_stride + (size_t)(j + half) * 2 * kN;
  // y - x, held in NTT form, back to coefficient form for its digits
#pragma unroll 1
  for (int poly = 0; poly < 2; ++poly) {
    uint64_t d[8], xv[8];
    ldg_slot8(yp + poly * kN, d);
    ld_slot8(xp + poly * kN, xv);
#pragma unroll
    for (int e = 0; e < 8; ++e) d[e] = sub_mod(d[e], xv[e], q);
    ntt_inv(d, sa, sb, M);
#pragma unroll
    for (int e = 0; e < 8; ++e) sd[poly * kN + strided_idx(tid, e)] = d[e];  // own slots only
  }
  tw_wait();
  uint64_t out[2][8];
  ext_product_core(sd, gsw + b * gsw_stride, C.l, C.base_log2, sa, sb, s_fwd, M, out);
  // x + RGSW (x) (y - x), staying in NTT form
#pragma unroll
  for (int poly = 0; poly < 2; ++poly) {
    uint64_t xv[8];
    ld_slot8(xp + poly * kN, xv);
#pragma unroll
    for (int e = 0; e < 8; ++e) xv[e] = add_mod(xv[e], out[poly][e], q);
    stg_slot8(xp + poly * kN, xv);
  }
}


// ---------------------------------------------------------------------------
// cluster forms
// ---------------------------------------------------------------------------

// Cluster barrier halves: arrive (no memory ordering) and wait.  A CTA may
// touch another CTA's shared memory only once that CTA has started; an
// arrive at kernel entry and a wait just before the first remote access
// guarantee it without stalling the CTAs that have work before it.
__device__ __forceinline__ void cluster_arrive_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
  asm volatile("barrier.cluster.wait.aligned;" ::: "memory");
}


// Expansion, 4 CTAs per tree node; CTA rank = 2 m + kk handles modulus m
// (0 = q, 1 = p) and key polynomial kk: NTT_m(sigma(c1)) * K[kk][m], INTT.
// The q-CTA kk then combines with the p-CTA kk through distributed shared
// memory and writes polynomial kk of both children (polynomial kk of c'
// depends on key polynomial kk only).
// kStage: also stage the inverse twiddles and the key polynomial with its
// companions in shared memory (one CTA per SM; for launches of one wave).
template <bool kStage>
__global__ void __cluster_dims__(4, 1, 1) __launch_bounds__(T)
    expand_cluster_kernel(const uint64_t *cur, uint64_t *nxt, size_t in_stride, size_t out_stride,
                          const __grid_constant__ KeyBatch kb, int level, ModTab Mq, ModTab Mp,
                          Consts C) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int m = rank >> 1, kk = rank & 1;
  extern __shared__ uint64_t smem[];
  uint64_t *sa = smem, *sb = smem + kSmemPoly;
  uint64_t *s_sig = smem + 2 * kSmemPoly;  // sigma(c1), then sigma(c0) (natural index)
  uint64_t *s_out = s_sig + kN;            // p-CTAs: their inverse transform (natural index)
  ulonglong2 *s_fwd = reinterpret_cast<ulonglong2 *>(s_out + kN), *s_inv = s_fwd + kN;
  uint64_t *s_key = reinterpret_cast<uint64_t *>(s_inv + kN);  // key polynomial, companions
  const int node = blockIdx.x >> 2, b = blockIdx.y;
  const size_t key_off = (size_t)level * 4 * kN + (size_t)(2 * kk + m) * kN;
  cluster_arrive_relaxed();
  // staging groups, completed in this order: forward twiddles, key,
  // companions, inverse twiddles
  prefetch_tw(s_fwd, m ? Mp.fwd : Mq.fwd);
  if constexpr (kStage) {
    prefetch_words(s_key, kb.q[b].galois + key_off, kN);
    prefetch_words(s_key + kN, kb.q[b].galois_s + key_off, kN);
    prefetch_tw(s_inv, m ? Mp.inv : Mq.inv);
  }
  grid_dep_sync();  // the staged tables and keys are constant; the parent level is not
  const int tid = threadIdx.x;
  const int k = 1 << level;
  const uint64_t g = (uint64_t)(kN / k + 1);
  const uint64_t q = C.q, p = C.p;
  const uint64_t *ci = cur + b * in_stride + (size_t)node * 2 * kN;
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int i = strided_idx(tid, e);
    const uint32_t j = (uint32_t)(((uint64_t)i * g) & (2 * kN - 1));
    const uint64_t v = ci[kN + i];
    if (j < (uint32_t)kN)
      s_sig[j] = v;
    else
      s_sig[j - kN] = neg_mod(v, q);
  }
  if constexpr (kStage)
    stage_wait<3>();
  else
    tw_wait();
  const ModTab &M = m ? Mp : Mq;
  uint64_t t[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const uint64_t v = s_sig[strided_idx(tid, e)];
    t[e] = (m && v >= p) ? v - p : v;  // q < 2p
  }
  ntt_fwd_s(t, sa, sb, s_fwd, M);
  {
    // Shoup product with the key's companion: [0, 4 mod), which the inverse
    // transform takes
    uint64_t kv[8], ks[8];
    if constexpr (kStage) {
      stage_wait<1>();
      lds_slot8(s_key, kv);
      lds_slot8(s_key + kN, ks);
    } else {
      ldg_slot8(kb.q[b].galois + key_off, kv);
      ldg_slot8(kb.q[b].galois_s + key_off, ks);
    }
#pragma unroll
    for (int e = 0; e < 8; ++e) t[e] = mul_shoup_lazy4(t[e], kv[e], ks[e], M.q);
  }
  if constexpr (kStage) {
    stage_wait<0>();
    ntt_inv_s(t, sa, sb, s_inv, M);
  } else {
    ntt_inv(t, sa, sb, M);
  }
  if (m == 1) {
    // the p result goes straight into the shared memory of the q-CTA of the
    // same key polynomial (rank kk), which combines the two: a remote store
    // costs the consumer no round trip
    cluster_wait();
    uint64_t *dst = cluster.map_shared_rank(s_out, kk);
#pragma unroll
    for (int e = 0; e < 8; ++e) dst[strided_idx(tid, e)] = t[e];
    cluster.sync();
    return;  // nothing reads this CTA's shared memory any more
  }
  if (kk == 0) {
    // sigma(c0) into s_sig (its last reads were before the transforms' barriers)
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int i = strided_idx(tid, e);
      const uint32_t j = (uint32_t)(((uint64_t)i * g) & (2 * kN - 1));
      const uint64_t v = ci[i];
      if (j < (uint32_t)kN)
        s_sig[j] = v;
      else
        s_sig[j - kN] = neg_mod(v, q);
    }
  }
  uint64_t xv[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) xv[e] = ci[(size_t)kk * kN + strided_idx(tid, e)];
  cluster_wait();
  cluster.sync();  // the p result is in s_out
  uint64_t *ce = nxt + b * out_stride + (size_t)(2 * node) * 2 * kN + (size_t)kk * kN;
  uint64_t *co = ce + 2 * kN;
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int i = strided_idx(tid, e);
    const uint64_t rr = add_mod(s_out[i], C.p_half, p);
    const uint64_t v = mul_shoup(sub_mod(add_mod(t[e], C.p_half_mod_q, q), rr, q), C.p_inv_q,
                                 C.p_inv_q_s, q);
    const uint64_t cp = kk == 0 ? add_mod(s_sig[i], v, q) : v;
    const uint64_t x = xv[e];
    ce[i] = add_mod(x, cp, q);
    const uint64_t d = sub_mod(x, cp, q);
    if (i >= k)
      co[i - k] = d;
    else
      co[kN - k + i] = neg_mod(d, q);
  }
}

// Expansion, 2 CTAs per tree node (levels too wide for the 4-CTA cluster to
// fit one wave, too narrow to fill the GPU with one CTA per node): CTA m
// handles modulus m (0 = q, 1 = p) for both key polynomials:
// INTT_m(NTT_m(sigma(c1)) * K[kk][m]), kk = 0, 1 -- three dependent transforms
// instead of the one-CTA form's six.  CTA m then writes polynomial kk = m of
// both children from its own and its peer's results (distributed shared
// memory); sigma(c0) is gathered through the inverse automorphism.
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(T, 2)
    expand_pair_kernel(const uint64_t *cur, uint64_t *nxt, size_t in_stride, size_t out_stride,
                       const __grid_constant__ KeyBatch kb, int level, ModTab Mq, ModTab Mp,
                       Consts C) {
  cg::cluster_group cluster = cg::this_cluster();
  const int m = (int)cluster.block_rank();
  extern __shared__ uint64_t smem[];
  uint64_t *sa = smem, *sb = smem + kSmemPoly;
  uint64_t *s_sig = smem + 2 * kSmemPoly;  // sigma(c1), then the kk = 0 result (natural index)
  ulonglong2 *s_fwd = reinterpret_cast<ulonglong2 *>(s_sig + kN);  // staged by cp.async
  const ModTab &M = m ? Mp : Mq;
  prefetch_tw(s_fwd, M.fwd);
  grid_dep_sync();
  const int tid = threadIdx.x;
  const int node = blockIdx.x >> 1, b = blockIdx.y;
  const int k = 1 << level;
  const uint64_t g = (uint64_t)(kN / k + 1);
  const uint64_t q = C.q, p = C.p;
  const uint64_t *ci = cur + b * in_stride + (size_t)node * 2 * kN;
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int i = strided_idx(tid, e);
    const uint32_t j = (uint32_t)(((uint64_t)i * g) & (2 * kN - 1));
    const uint64_t v = ci[kN + i];
    if (j < (uint32_t)kN)
      s_sig[j] = v;
    else
      s_sig[j - kN] = neg_mod(v, q);
  }
  tw_wait();
  uint64_t t[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const uint64_t v = s_sig[strided_idx(tid, e)];
    t[e] = (m && v >= p) ? v - p : v;  // q < 2p
  }
  ntt_fwd_s(t, sa, sb, s_fwd, M);  // its barriers end every read of sigma(c1)
  const uint64_t *key = kb.q[b].galois + (size_t)level * 4 * kN;
  const uint64_t *key_s = kb.q[b].galois_s + (size_t)level * 4 * kN;
#pragma unroll 1
  for (int kk = 0; kk < 2; ++kk) {
    uint64_t a[8], as[8];
    ldg_slot8(key + (size_t)(2 * kk + m) * kN, a);
    ldg_slot8(key_s + (size_t)(2 * kk + m) * kN, as);
#pragma unroll
    for (int e = 0; e < 8; ++e) a[e] = mul_shoup_lazy4(t[e], a[e], as[e], M.q);
    ntt_inv(a, sa, sb, M);  // ends with a barrier: sa is free afterwards
    uint64_t *dst = kk == 0 ? s_sig : sa;  // result of key polynomial kk
#pragma unroll
    for (int e = 0; e < 8; ++e) dst[strided_idx(tid, e)] = a[e];
  }
  cluster.sync();
  // this CTA writes polynomial kk = m of both children
  const int kk = m;
  const uint64_t *xq = kk == 0 ? cluster.map_shared_rank(s_sig, 0) : cluster.map_shared_rank(sa, 0);
  const uint64_t *xp = kk == 0 ? cluster.map_shared_rank(s_sig, 1) : cluster.map_shared_rank(sa, 1);
  uint64_t ginv = g;  // g^-1 mod 2N (g odd): Newton steps double the correct low bits
#pragma unroll
  for (int it = 0; it < 4; ++it) ginv *= 2 - g * ginv;
  uint64_t *ce = nxt + b * out_stride + (size_t)(2 * node) * 2 * kN + (size_t)kk * kN;
  uint64_t *co = ce + 2 * kN;
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int i = strided_idx(tid, e);
    const uint64_t rr = add_mod(xp[i], C.p_half, p);
    const uint64_t v = mul_shoup(sub_mod(add_mod(xq[i], C.p_half_mod_q, q), rr, q), C.p_inv_q,
                                 C.p_inv_q_s, q);
    uint64_t cp = v;
    if (kk == 0) {
      // sigma(c0)[i]: coefficient s = i g^-1 mod 2N of c0, negated when s >= N
      const uint32_t sidx = (uint32_t)(((uint64_t)i * ginv) & (2 * kN - 1));
      const uint64_t s0 = sidx < (uint32_t)kN ? ci[sidx] : neg_mod(ci[sidx - kN], q);
      cp = add_mod(s0, v, q);
    }
    const uint64_t x = ci[(size_t)kk * kN + i];
    ce[i] = add_mod(x, cp, q);
    const uint64_t d = sub_mod(x, cp, q);
    if (i >= k)
      co[i - k] = d;
    else
      co[kN - k + i] = neg_mod(d, q);
  }
  cluster.sync();
}

// MAC of digit polynomials (coefficient form, strided distribution, NTT'd
// here) with RGSW rows, for both output polynomials; 128-bit sums.
__device__ __forceinline__ void digit_mac(uint64_t d[8], const uint64_t *row, uint64_t *sa,
                                          uint64_t *sb, const ulonglong2 *s_fwd, const ModTab &M,
                                          U128 acc0[8], U128 acc1[8]) {
  ntt_fwd_s(d, sa, sb, s_fwd, M);
  uint64_t w0[8], w1[8];
  ldg_slot8(row, w0);
  ldg_slot8(row + kN, w1);
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    mac_to(acc0[e], d[e], w0[e]);
    mac_to(acc1[e], d[e], w1[e]);
  }
}

// Sum over cluster ranks 0 .. R-1 of the 8 slots 8 tid .. 8 tid + 7 of
// `src` (a shared-memory array at the same offset in every CTA), mod q.  The
// 16-byte remote loads of up to five ranks are in flight before the first
// addition (summing element by element serialised the distributed-shared-
// memory latency; five ranks at a time bound the registers they hold).
template <int R>
__device__ __forceinline__ void cluster_sum8(cg::cluster_group &cluster, uint64_t *src, uint64_t q,
                                             uint64_t sum[8]) {
  constexpr int kChunk = 5;
#pragma unroll
  for (int r0 = 0; r0 < R; r0 += kChunk) {
    constexpr int kMaxIn = R < kChunk ? R : kChunk;
    const int nin = R - r0 < kChunk ? R - r0 : kChunk;
    ulonglong2 v[kMaxIn][4];
#pragma unroll
    for (int rr = 0; rr < kMaxIn; ++rr) {
      if (rr >= nin) break;
      const ulonglong2 *pr = reinterpret_cast<const ulonglong2 *>(
          cluster.map_shared_rank(src, r0 + rr) + slot_idx(threadIdx.x, 0));
#pragma unroll
      for (int h = 0; h < 4; ++h) v[rr][h] = pr[h];
    }
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      uint64_t s0 = r0 == 0 ? v[0][h].x : add_mod(sum[2 * h], v[0][h].x, q);
      uint64_t s1 = r0 == 0 ? v[0][h].y : add_mod(sum[2 * h + 1], v[0][h].y, q);
#pragma unroll
      for (int rr = 1; rr < kMaxIn; ++rr) {
        if (rr >= nin) break;
        s0 = add_mod(s0, v[rr][h].x, q);
        s1 = add_mod(s1, v[rr][h].y, q);
      }
      sum[2 * h] = s0;
      sum[2 * h + 1] = s1;
    }
  }
}

// Folding (other_dim_mux), a cluster of CS CTAs per ciphertext pair (l = 5,
// digits of at most 16 bits).  CTAs 0 and 1 transform polynomial 0 / 1 of
// y - x back to coefficient form, split it into its l digits and store each
// digit plane (2 bytes a coefficient) into the shared memory of the CTA that
// multiplies it: with CS = l, CTA k takes digit k of both polynomials (RGSW
// rows k and l + k); with CS = 2 l, CTA p l + k takes digit k of polynomial
// p alone (one transform per CTA, for the narrowest levels).  Each CTA
// leaves its partial sums (reduced mod q) in shared memory, and the sums
// x + sum of partials are split over the cluster: CTA r adds up its share of
// the 2 N coefficients from every CTA and writes it.  Moving digit planes
// instead of 8-byte coefficients, and spreading the final sums, keeps the
// distributed-shared-memory traffic of any one SM small: it, not the
// transforms, bounded these launches.
constexpr int kFoldCluster = 5;
constexpr int kFoldWide = 2 * kFoldCluster;
template <int CS>
__device__ __forceinline__ void fold_cluster_body(uint64_t *res, size_t res_stride,
                                                  const uint64_t *gsw, size_t gsw_stride, int half,
                                                  const ModTab &M, const Consts &C) {
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  extern __shared__ uint64_t smem[];
  uint64_t *sa = smem, *sb = smem + kSmemPoly;
  uint64_t *part = smem + 2 * kSmemPoly;  // [kk][slot]: this CTA's partial sums
  // [polynomial][coefficient]: the digits this CTA multiplies (shares the
  // space of `part`, which is written only after they have been read)
  uint16_t *dig = reinterpret_cast<uint16_t *>(part);
  ulonglong2 *s_fwd = reinterpret_cast<ulonglong2 *>(part + 2 * kN);  // staged by cp.async
  const int tid = threadIdx.x;
  const int j = blockIdx.x / CS, b = blockIdx.y;
  const uint64_t q = C.q;
  const int l = kFoldCluster;
  const int digit = r % l;
  uint64_t *xp = res + b * res_stride + (size_t)j * 2 * kN;
  const uint64_t *yp = res + b * res_stride + (size_t)(j + half) * 2 * kN;
  const uint64_t *rgsw = gsw + b * gsw_stride;
  cluster_arrive_relaxed();
  prefetch_tw(s_fwd, M.fwd);
  grid_dep_sync();
  if (r < 2) {
    uint64_t d[8], xv[8];
    ldg_slot8(yp + (size_t)r * kN, d);
    ld_slot8(xp + (size_t)r * kN, xv);
#pragma unroll
    for (int e = 0; e < 8; ++e) d[e] = sub_mod(d[e], xv[e], q);
    ntt_inv(d, sa, sb, M);
    cluster_wait();
    const uint64_t mask = (1ULL << C.base_log2) - 1;
#pragma unroll
    for (int k = 0; k < l; ++k) {
      uint16_t *dst = cluster.map_shared_rank(dig, CS == kFoldWide ? r * l + k : k) + r * kN;
      const int sh = (l - 1 - k) * C.base_log2;
#pragma unroll
      for (int e = 0; e < 8; ++e) dst[strided_idx(tid, e)] = (uint16_t)((d[e] >> sh) & mask);
    }
  } else {
    cluster_wait();
  }
  cluster.sync();  // digit planes in place
  U128 acc0[8], acc1[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) acc0[e] = acc1[e] = U128{0, 0};
  constexpr int kPolys = CS == kFoldWide ? 1 : 2;
#pragma unroll
  for (int pi = 0; pi < kPolys; ++pi) {
    const int poly = CS == kFoldWide ? r / l : pi;
    uint64_t d[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) d[e] = dig[poly * kN + strided_idx(tid, e)];
    if (pi == 0) tw_wait();
    // the transform's barriers order every thread's digit reads before the
    // partial sums below overwrite them
    digit_mac(d, rgsw + (size_t)(poly * l + digit) * 2 * kN, sa, sb, s_fwd, M, acc0, acc1);
  }
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int si = slot_idx(tid, e);
    part[si] = barrett128(acc0[e], q, M.mu_lo, M.mu_hi);
    part[kN + si] = barrett128(acc1[e], q, M.mu_lo, M.mu_hi);
  }
  cluster.sync();  // partial sums in place
  // x + RGSW (x) (y - x), staying in NTT form: CTA r's share of the N
  // 16-byte units of the two polynomials
  const ulonglong2 *src[CS];
#pragma unroll
  for (int rr = 0; rr < CS; ++rr)
    src[rr] = reinterpret_cast<const ulonglong2 *>(cluster.map_shared_rank(part, rr));
  ulonglong2 *xu = reinterpret_cast<ulonglong2 *>(xp);
  for (int u = r * kN / CS + tid; u < (r + 1) * kN / CS; u += T) {
    ulonglong2 v[CS];
#pragma unroll
    for (int rr = 0; rr < CS; ++rr) v[rr] = src[rr][u];
    const ulonglong2 xv = xu[u];
    uint64_t s0 = xv.x, s1 = xv.y;
#pragma unroll
    for (int rr = 0; rr < CS; ++rr) {
      s0 = add_mod(s0, v[rr].x, q);
      s1 = add_mod(s1, v[rr].y, q);
    }
    xu[u] = make_ulonglong2(s0, s1);
  }
  cluster.sync();  // no CTA leaves while another reads its partial sums
}

__global__ void __cluster_dims__(kFoldCluster, 1, 1) __launch_bounds__(T)
    fold_cluster_kernel(uint64_t *res, size_t res_stride, const uint64_t *gsw, size_t gsw_stride,
                        int half, ModTab M, Consts C) {
  fold_cluster_body<kFoldCluster>(res, res_stride, gsw, gsw_stride, half, M, C);
}

// ten CTAs per pair: a non-portable cluster size, given at launch
__global__ void __launch_bounds__(T)
    fold_wide_kernel(uint64_t *res, size_t res_stride, const uint64_t *gsw, size_t gsw_stride,
                     int half, ModTab M, Consts C) {
  fold_cluster_body<kFoldWide>(res, res_stride, gsw, gsw_stride, half, M, C);
}

// Folding, 2 CTAs per ciphertext pair (the wide levels of few queries): CTA
// a decomposes polynomial a of y - x into its l digits, transforms them and
// multiplies them with RGSW rows a l .. a l + l - 1, leaving partial sums of
// both output polynomials (reduced mod q) in shared memory; CTA a then adds
// the two partials of output polynomial a, transforms back and adds x.  Half
// the dependent transforms of the one-CTA form per pair.
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(T, 2)
    fold_pair_kernel(uint64_t *res, size_t res_stride, const uint64_t *gsw, size_t gsw_stride,
                     int half, ModTab M, Consts C) {
  cg::cluster_group cluster = cg::this_cluster();
  const int a = (int)cluster.block_rank();
  extern __shared__ uint64_t smem[];
  uint64_t *sa = smem, *sb = smem + kSmemPoly;
  uint64_t *part = smem + 2 * kSmemPoly;  // [output polynomial][slot]
  ulonglong2 *s_fwd = reinterpret_cast<ulonglong2 *>(part + 2 * kN);  // staged by cp.async
  prefetch_tw(s_fwd, M.fwd);
  grid_dep_sync();
  const int tid = threadIdx.x;
  const int j = blockIdx.x >> 1, b = blockIdx.y;
  const uint64_t q = C.q;
  const int l = C.l;
  uint64_t *xp = res + b * res_stride + (size_t)j * 2 * kN;
  const uint64_t *yp = res + b * res_stride + (size_t)(j + half) * 2 * kN;
  const uint64_t *rgsw = gsw + b * gsw_stride;
  const uint64_t mask = (1ULL << C.base_log2) - 1;
  // polynomial a of y - x, held in NTT form, back to coefficient form in
  // `part` (each thread reads back only its own strided slots; the
  // transforms' barriers order the last reads before the partial sums
  // overwrite it)
  {
    uint64_t d[8], xv[8];
    ldg_slot8(yp + (size_t)a * kN, d);
    ld_slot8(xp + (size_t)a * kN, xv);
#pragma unroll
    for (int e = 0; e < 8; ++e) d[e] = sub_mod(d[e], xv[e], q);
    ntt_inv(d, sa, sb, M);
#pragma unroll
    for (int e = 0; e < 8; ++e) part[strided_idx(tid, e)] = d[e];
  }
  U128 acc0[8], acc1[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) acc0[e] = acc1[e] = U128{0, 0};
  tw_wait();
#pragma unroll 1
  for (int pp = l - 1; pp >= 0; --pp) {
    const int sh = pp * C.base_log2;
    uint64_t d[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) d[e] = (part[strided_idx(tid, e)] >> sh) & mask;
    digit_mac(d, rgsw + (size_t)(a * l + (l - 1 - pp)) * 2 * kN, sa, sb, s_fwd, M, acc0, acc1);
  }
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int si = slot_idx(tid, e);
    part[si] = barrett128(acc0[e], q, M.mu_lo, M.mu_hi);
    part[kN + si] = barrett128(acc1[e], q, M.mu_lo, M.mu_hi);
  }
  cluster.sync();
  // x + RGSW (x) (y - x), staying in NTT form
  uint64_t sum[8], xv[8];
  cluster_sum8<2>(cluster, part + (size_t)a * kN, q, sum);
  ld_slot8(xp + (size_t)a * kN, xv);
#pragma unroll
  for (int e = 0; e < 8; ++e) xv[e] = add_mod(xv[e], sum[e], q);
  stg_slot8(xp + (size_t)a * kN, xv);
  cluster.sync();
}

// RGSW reconstruction (query_to_gsw), 6 CTAs per ciphertext (l_key = 10):
// CTA 5 writes the first-half row (the ciphertext in NTT form); CTA r < 5
// handles key digit levels 2r and 2r+1 of both polynomials; CTAs 0 and 1 add
// the partials of output polynomial 0 / 1 into the second-half row.
constexpr int kQtgCluster = 6;
__global__ void __cluster_dims__(kQtgCluster, 1, 1) __launch_bounds__(T, 2)
    query_to_gsw_cluster_kernel(const uint64_t *leaves, size_t leaves_stride, uint64_t *gsw_out,
                                size_t gsw_stride, const __grid_constant__ KeyBatch kb, int n1,
                                ModTab M, Consts C) {
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  extern __shared__ uint64_t smem[];
  uint64_t *sa = smem, *sb = smem + kSmemPoly;
  uint64_t *part = smem + 2 * kSmemPoly;
  ulonglong2 *s_fwd = reinterpret_cast<ulonglong2 *>(part + 2 * kN);
  prefetch_tw(s_fwd, M.fwd);
  grid_dep_sync();
  const int tid = threadIdx.x;
  const int jct = blockIdx.x / kQtgCluster, b = blockIdx.y;
  const int l = C.l, lk = C.l_key;
  const int dim = jct / l, kk = jct % l;
  const uint64_t q = C.q;
  const uint64_t *ct = leaves + b * leaves_stride + (size_t)(n1 + jct) * 2 * kN;
  uint64_t *rgsw = gsw_out + b * gsw_stride + (size_t)dim * 2 * l * 2 * kN;
  tw_wait();
  if (r == kQtgCluster - 1) {
    uint64_t *row0 = rgsw + (size_t)kk * 2 * kN;
#pragma unroll 1
    for (int poly = 0; poly < 2; ++poly) {  // one copy of the transform: 43 rather than 45 us
      uint64_t v[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) v[e] = ct[poly * kN + strided_idx(tid, e)];
      ntt_fwd_s(v, sa, sb, s_fwd, M);
      stg_slot8(row0 + poly * kN, v);
    }
  } else {
    const uint64_t *key = kb.q[b].gsw_key;
    const uint64_t mask = (1ULL << C.base_log2_key) - 1;
    U128 acc0[8], acc1[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) acc0[e] = acc1[e] = U128{0, 0};
#pragma unroll 1
    for (int poly = 0; poly < 2; ++poly) {
#pragma unroll 1
      for (int h = 0; h < 2; ++h) {
        const int level = 2 * r + h;          // row index within the poly's l_key rows
        const int sh = (lk - 1 - level) * C.base_log2_key;
        uint64_t d[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) d[e] = (ct[poly * kN + strided_idx(tid, e)] >> sh) & mask;
        digit_mac(d, key + (size_t)(poly * lk + level) * 2 * kN, sa, sb, s_fwd, M, acc0, acc1);
      }
    }
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int si = slot_idx(tid, e);
      part[si] = barrett128(acc0[e], q, M.mu_lo, M.mu_hi);
      part[kN + si] = barrett128(acc1[e], q, M.mu_lo, M.mu_hi);
    }
  }
  cluster.sync();
  if (r < 2) {
    uint64_t *row1 = rgsw + (size_t)(l + kk) * 2 * kN + (size_t)r * kN;
    uint64_t sum[8];
    cluster_sum8<kQtgCluster - 1>(cluster, part + (size_t)r * kN, q, sum);
    stg_slot8(row1, sum);
  }
  cluster.sync();
}

// Cluster form below these many ciphertexts per launch (batch included);
// one-CTA form at or above.  From per-launch timings on GB300 (the one-CTA
// forms at two CTAs per SM): the cluster expansion wins below ~128 nodes
// (128 and 256 measured alike, 1024 and 64 slower), the cluster fold on the
// narrow levels (< 48 pairs), the cluster RGSW reconstruction for one
// query's 45 or 55 ciphertexts (80 -> 45 us; it needs two CTAs per SM so
// that its 6-CTA clusters fit one wave).
int g_expand_threshold = 128;
int g_fold_threshold = 48;
// pair form (2 CTAs per pair) from g_fold_threshold up to this many pairs:
// one query's 64- and 128-pair levels (folding 0.314 -> 0.298 ms; the
// 256-pair level and 32-query batches measured slower in the pair form)
int g_pair_threshold = 130;
// expansion pair form (2 CTAs per node) from g_expand_threshold up to this
// many nodes per launch: one query's 140-node level (expansion 0.223 ->
// 0.212 ms; its 279-node level and 4- or 32-query batches were slower)
int g_expand_pair_threshold = 150;
int g_qtg_threshold = 64;
// wide fold cluster (10 CTAs per pair) below this many pairs per launch, if
// the GPU can place a 10-CTA cluster (g_wide_ok): one query's 8 .. 1-pair
// levels (folding 0.2935 -> 0.287 ms; with the 16- and 32-pair levels too,
// 0.289 and 0.291)
int g_wide_threshold = 9;
bool g_wide_ok = false;

}  // namespace

constexpr size_t kExpandSmem = (2 * kSmemPoly + 4 * kN) * sizeof(uint64_t);

// plus the staged forward twiddle table (2048 x 16 bytes) at the end
constexpr size_t kClusterSmem = (2 * kSmemPoly + 2 * kN) * sizeof(uint64_t) + kN * sizeof(ulonglong2);
// expansion cluster with kStage: plus the inverse table and a key polynomial
// with its companions
// expansion pair: transform buffers, sigma(c1), the staged forward twiddles
constexpr size_t kExpandPairSmem = (2 * kSmemPoly + kN) * sizeof(uint64_t) + kN * sizeof(ulonglong2);
constexpr size_t kExpandClusterSmem = kClusterSmem + kN * sizeof(ulonglong2) + 2 * kN * sizeof(uint64_t);
static_assert(kExpandClusterSmem <= 227 * 1024, "shared memory per CTA");
int g_sms = 152;
// Measured on one query of the 262,144-plaintext database: in a graph, the
// expansion levels gain (836 -> 841 queries/s, their kernels stage 96 KB of
// twiddles and keys), folding loses (-> 819), the other kinds are neutral;
// direct launches gain with every kind (797 -> 814).
int g_pdl_graph = kPdlExpand;
int g_pdl_direct = kPdlExpand | kPdlQtg | kPdlPrep | kPdlNtt | kPdlFold | kPdlModswitch;
// one-CTA fold and RGSW reconstruction: transform buffers + the source
// ciphertext + the staged forward twiddles
constexpr size_t kExtSmem = (2 * kSmemPoly + 2 * kN) * sizeof(uint64_t) + kN * sizeof(ulonglong2);

cudaError_t init_kernel_attributes() {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(expand_level_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kExpandSmem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(fold_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kExtSmem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(query_to_gsw_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kExtSmem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(expand_cluster_kernel<true>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kExpandClusterSmem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(expand_cluster_kernel<false>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kClusterSmem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(fold_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kClusterSmem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(fold_wide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kClusterSmem)) != cudaSuccess)
    return e;
  {
    // a 10-CTA cluster is beyond the portable 8: allowed per kernel, and
    // usable where the occupancy query places at least one
    g_wide_ok = false;
    if (cudaFuncSetAttribute(fold_wide_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
        cudaSuccess) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(kFoldWide);
      cfg.blockDim = dim3(T);
      cfg.dynamicSmemBytes = kClusterSmem;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = kFoldWide;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int nc = 0;
      if (cudaOccupancyMaxActiveClusters(&nc, fold_wide_kernel, &cfg) == cudaSuccess && nc > 0)
        g_wide_ok = true;
    }
    cudaGetLastError();  // a refused attribute or query leaves the wide form off
  }
  if ((e = cudaFuncSetAttribute(fold_pair_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kClusterSmem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(expand_pair_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kExpandPairSmem)) != cudaSuccess)
    return e;
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  if ((e = cudaFuncSetAttribute(query_to_gsw_cluster_kernel,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kClusterSmem)) != cudaSuccess)
    return e;
  g_expand_threshold = 128;
  g_fold_threshold = 48;
  g_pair_threshold = 130;
  g_expand_pair_threshold = 150;
  g_qtg_threshold = 64;
  if (const char *v = getenv("OPIR_CLUSTER_THRESHOLD"))  // one threshold for all (tests, sweeps)
    g_expand_threshold = g_fold_threshold = g_qtg_threshold = atoi(v);
  if (const char *v = getenv("OPIR_EXPAND_THRESHOLD")) g_expand_threshold = atoi(v);
  if (const char *v = getenv("OPIR_FOLD_THRESHOLD")) g_fold_threshold = atoi(v);
  g_wide_threshold = 9;
  if (const char *v = getenv("OPIR_WIDE_THRESHOLD")) g_wide_threshold = atoi(v);
  if (const char *v = getenv("OPIR_QTG_THRESHOLD")) g_qtg_threshold = atoi(v);
  if (const char *v = getenv("OPIR_PAIR_THRESHOLD")) g_pair_threshold = atoi(v);
  if (const char *v = getenv("OPIR_EXPAND_PAIR_THRESHOLD")) g_expand_pair_threshold = atoi(v);
  g_pdl_graph = kPdlExpand;
  g_pdl_direct = kPdlExpand | kPdlQtg | kPdlPrep | kPdlNtt | kPdlFold | kPdlModswitch;
  if (const char *v = getenv("OPIR_PDL_GRAPH")) g_pdl_graph = atoi(v);
  if (const char *v = getenv("OPIR_PDL")) g_pdl_direct = atoi(v);
  return cudaSuccess;
}

bool tree_form_valid(int stage, int form, const Consts &C) {
  switch (form) {
    case kFormOne:
      return true;
    case kFormPair:
      return stage != kStageQtg;
    case kFormCluster:
      return stage == kStageExpand ||
             (stage == kStageFold && C.l == kFoldCluster && C.base_log2 <= 16) ||
             (stage == kStageQtg && C.l_key == 2 * (kQtgCluster - 1));
    case kFormWide:
      return stage == kStageFold && C.l == kFoldCluster && C.base_log2 <= 16 && g_wide_ok;
    default:
      return false;
  }
}

namespace {
// the tuned form for `count`, else the default thresholds
int form_for(int stage, int count, const Consts &C, const TreeForms *forms) {
  const int f = forms ? forms->pick(stage, count) : kFormDefault;
  if (f != kFormDefault && tree_form_valid(stage, f, C)) return f;
  switch (stage) {
    case kStageExpand:
      return count < g_expand_threshold ? kFormCluster
             : count < g_expand_pair_threshold ? kFormPair : kFormOne;
    case kStageQtg:
      return tree_form_valid(kStageQtg, kFormCluster, C) && count < g_qtg_threshold ? kFormCluster
                                                                                      : kFormOne;
    default:
      if (tree_form_valid(kStageFold, kFormWide, C) && count < g_wide_threshold) return kFormWide;
      return tree_form_valid(kStageFold, kFormCluster, C) && count < g_fold_threshold
                 ? kFormCluster
                 : count < g_pair_threshold ? kFormPair : kFormOne;
  }
}
}  // namespace

int tree_default_form(int stage, int count, const Consts &C) {
  return form_for(stage, count, C, nullptr);
}

void launch_expand_level(const uint64_t *cur, uint64_t *nxt, size_t in_stride, size_t out_stride,
                         const QueryDesc *qd, int level, int live_nodes, int batch,
                         const ModTab &Mq, const ModTab &Mp, const Consts &C, cudaStream_t s,
                         bool pdl, const TreeForms *forms) {
  for (int b0 = 0; b0 < batch; b0 += kMaxKeyBatch) {
    const int nb = batch - b0 < kMaxKeyBatch ? batch - b0 : kMaxKeyBatch;
    KeyBatch kb;
    for (int i = 0; i < nb; ++i) kb.q[i] = qd[b0 + i];
    const uint64_t *in = cur + b0 * in_stride;
    uint64_t *out = nxt + b0 * out_stride;
    const int form = form_for(kStageExpand, live_nodes * nb, C, forms);
    if (form == kFormCluster && 4 * live_nodes * nb <= g_sms)
      launch_kernel(pdl, expand_cluster_kernel<true>, dim3(4 * live_nodes, nb), dim3(T),
                    kExpandClusterSmem, s, in, out, in_stride, out_stride, kb, level, Mq, Mp, C);
    else if (form == kFormCluster)
      launch_kernel(pdl, expand_cluster_kernel<false>, dim3(4 * live_nodes, nb), dim3(T),
                    kClusterSmem, s, in, out, in_stride, out_stride, kb, level, Mq, Mp, C);
    else if (form == kFormPair)
      launch_kernel(pdl, expand_pair_kernel, dim3(2 * live_nodes, nb), dim3(T), kExpandPairSmem,
                    s, in, out, in_stride, out_stride, kb, level, Mq, Mp, C);
    else
      launch_kernel(pdl, expand_level_kernel, dim3(live_nodes, nb), dim3(T), kExpandSmem, s, in,
                    out, in_stride, out_stride, kb, level, Mq, Mp, C);
  }
}

void launch_query_to_gsw(const uint64_t *leaves, size_t leaves_stride, uint64_t *gsw_out,
                         size_t gsw_stride, const QueryDesc *qd, int n1, int num_cts, int batch,
                         const ModTab &Mq, const Consts &C, cudaStream_t s, bool pdl,
                         const TreeForms *forms) {
  if (num_cts <= 0) return;
  for (int b0 = 0; b0 < batch; b0 += kMaxKeyBatch) {
    const int nb = batch - b0 < kMaxKeyBatch ? batch - b0 : kMaxKeyBatch;
    KeyBatch kb;
    for (int i = 0; i < nb; ++i) kb.q[i] = qd[b0 + i];
    const uint64_t *in = leaves + b0 * leaves_stride;
    uint64_t *out = gsw_out + b0 * gsw_stride;
    if (form_for(kStageQtg, num_cts * nb, C, forms) == kFormCluster)
      launch_kernel(pdl, query_to_gsw_cluster_kernel, dim3(kQtgCluster * num_cts, nb), dim3(T),
                    kClusterSmem, s, in, leaves_stride, out, gsw_stride, kb, n1, Mq, C);
    else
      launch_kernel(pdl, query_to_gsw_kernel, dim3(num_cts, nb), dim3(T), kExtSmem, s, in,
                    leaves_stride, out, gsw_stride, kb, n1, Mq, C);
  }
}

void launch_fold(uint64_t *res, size_t res_stride, const uint64_t *gsw, size_t gsw_stride,
                 int half, int batch, const ModTab &Mq, const Consts &C, cudaStream_t s,
                 bool pdl, const TreeForms *forms) {
  const int form = form_for(kStageFold, half * batch, C, forms);
  if (form == kFormWide) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kFoldWide * half, batch);
    cfg.blockDim = dim3(T);
    cfg.dynamicSmemBytes = kClusterSmem;
    cfg.stream = s;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = kFoldWide;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 2 : 1;
    cudaLaunchKernelEx(&cfg, fold_wide_kernel, res, res_stride, gsw, gsw_stride, half, Mq, C);
  } else if (form == kFormCluster)
    launch_kernel(pdl, fold_cluster_kernel, dim3(kFoldCluster * half, batch), dim3(T),
                  kClusterSmem, s, res, res_stride, gsw, gsw_stride, half, Mq, C);
  else if (form == kFormPair)
    launch_kernel(pdl, fold_pair_kernel, dim3(2 * half, batch), dim3(T), kClusterSmem, s, res,
                  res_stride, gsw, gsw_stride, half, Mq, C);
  else
    launch_kernel(pdl, fold_kernel, dim3(half, batch), dim3(T), kExtSmem, s, res, res_stride,
                  gsw, gsw_stride, half, Mq, C);
}

}  // namespace opir
