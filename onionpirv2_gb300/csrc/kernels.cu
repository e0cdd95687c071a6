// kernels.cu -- OnionPIRv2 server query path on GB300 (sm_103a).
//
// Each kernel restates one stage of PirServer::make_query (server.cpp:520-579)
// with exact integer arithmetic.  One CTA of 256 threads owns one
// polynomial pair (a ciphertext) and keeps it in registers, 8 coefficients
// per thread; NTTs exchange through shared memory (common.cuh).
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"
#include "entry.cuh"
#include "kernels.h"

namespace opir {

namespace {

constexpr int T = kNttThreads;

// ---------------------------------------------------------------------------
// generic batched NTT
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(T) ntt_kernel(ModTab M, uint64_t *polys, int inverse,
                                                size_t group_stride) {
  __shared__ uint64_t sa[kSmemPoly], sb[kSmemPoly];
  uint64_t *p = polys + blockIdx.y * group_stride + (size_t)blockIdx.x * kN;
  const int tid = threadIdx.x;
  grid_dep_sync();
  uint64_t r[8];
  if (!inverse) {
#pragma unroll
    for (int e = 0; e < 8; ++e) r[e] = p[strided_idx(tid, e)];
    ntt_fwd(r, sa, sb, M);
    stg_slot8(p, r);
  } else {
    ldg_slot8(p, r);
    ntt_inv(r, sa, sb, M);
#pragma unroll
    for (int e = 0; e < 8; ++e) p[strided_idx(tid, e)] = r[e];
  }
}

// ---------------------------------------------------------------------------
// first dimension
// ---------------------------------------------------------------------------

// evaluate_first_dim's NTT of the selection vector (server.cpp:137-139) and
// prep_query's transpose (server.cpp:80-118), into the scan operand:
// qs[c * n1 + k] = {lo30(Q0), hi30(Q0), lo30(Q1), hi30(Q1)} of leaf k.  One
// CTA per leaf and polynomial (blockIdx.z): each writes its half of the
// 16-byte operand words.
__global__ void __launch_bounds__(T) query_prep_kernel(const uint64_t *leaves,
                                                       size_t leaves_stride, uint4 *qs,
                                                       size_t stride_b, size_t stride_c,
                                                       size_t stride_k, ModTab M) {
  __shared__ uint64_t sa[kSmemPoly], sb[kSmemPoly];
  const int tid = threadIdx.x;
  const int k = blockIdx.x, b = blockIdx.y, poly = blockIdx.z;
  const uint64_t *ct = leaves + b * leaves_stride + (size_t)k * 2 * kN + (size_t)poly * kN;
  grid_dep_sync();
  uint64_t r[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) r[e] = ct[strided_idx(tid, e)];
  ntt_fwd(r, sa, sb, M);
  uint2 *dst = reinterpret_cast<uint2 *>(qs + b * stride_b + k * stride_k) + poly;
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int c = slot_idx(tid, e);
    dst[(size_t)c * stride_c * 2] = make_uint2((uint32_t)(r[e] & 0x3FFFFFFFu), (uint32_t)(r[e] >> 30));
  }
}

// The same transform into a plain plane[b][k][poly][c] (NTT form, fully
// reduced): one coalesced 64-byte run per thread and polynomial.  Input of
// the tensor-core product, which splits it into limbs.
__global__ void __launch_bounds__(T) query_prep_plane_kernel(const uint64_t *leaves,
                                                             size_t leaves_stride,
                                                             uint64_t *plane, int n1, ModTab M) {
  __shared__ uint64_t sa[kSmemPoly], sb[kSmemPoly];
  const int tid = threadIdx.x;
  const int k = blockIdx.x, b = blockIdx.y, poly = blockIdx.z;  // one polynomial per CTA
  const uint64_t *ct = leaves + b * leaves_stride + (size_t)k * 2 * kN + (size_t)poly * kN;
  grid_dep_sync();
  uint64_t r[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) r[e] = ct[strided_idx(tid, e)];
  ntt_fwd(r, sa, sb, M);
  stg_slot8(plane + (((size_t)b * n1 + k) * 2 + poly) * kN, r);
}

// ---------------------------------------------------------------------------
// mod switch (server.cpp:779-801) + response packing (server.cpp:581-633)
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint64_t mod_switch_coeff(uint64_t x, const Consts &C) {
  return mod_switch_x87(x, C.ms_mant, C.ms_shift);
}

// One CTA per slice of kModSlices consecutive coefficient ranges of one
// response: 2N / kModSlices coefficients (a multiple of 32, so every slice
// starts on a 32-bit word of the packed stream), one per thread.  kSwitch:
// mod-switch each coefficient first (the query pipeline); else pack the
// coefficients as given (save_resp_to_stream of any response).
constexpr int kModSlices = 16;
template <bool kSwitch>
__global__ void __launch_bounds__(T) modswitch_pack_kernel(const uint64_t *res, size_t res_stride,
                                                           uint64_t *resp, uint8_t *packed,
                                                           int packed_bytes, Consts C,
                                                           const uint32_t *status,
                                                           uint32_t *status_out) {
  extern __shared__ uint32_t words[];
  const int tid = threadIdx.x, slice = blockIdx.x, b = blockIdx.y;
  const int w = C.small_q_width;
  const int per = 2 * kN / kModSlices;
  const int i0 = slice * per;
  const int nwords = per * w / 32;  // the slice's words of the packed stream
  for (int i = tid; i < nwords; i += T) words[i] = 0;
  __syncthreads();
  grid_dep_sync();
  if (status_out && tid == 0 && slice == 0 && b == 0)
    *status_out = *reinterpret_cast<const volatile uint32_t *>(status);
  const uint64_t *ct = res + b * res_stride;
  const uint64_t mask = (1ULL << w) - 1;
  for (int i = i0 + tid; i < i0 + per; i += T) {
    const uint64_t v = kSwitch ? mod_switch_coeff(ct[i], C) : ct[i];
    if (resp) resp[(size_t)b * 2 * kN + i] = v;
    const uint64_t m = v & mask;
    const uint64_t bit = (uint64_t)(i - i0) * w;
    const int wi = (int)(bit >> 5), sh = (int)(bit & 31);
    atomicOr(&words[wi], (uint32_t)(m << sh));
    if (sh + w > 32) atomicOr(&words[wi + 1], (uint32_t)(m >> (32 - sh)));
    if (sh + w > 64) atomicOr(&words[wi + 2], (uint32_t)(m >> (64 - sh)));
  }
  __syncthreads();
  if (packed) {
    uint8_t *dst = packed + (size_t)b * packed_bytes + (size_t)i0 * w / 8;
    for (int i = tid; i < 4 * nwords; i += T) dst[i] = (uint8_t)(words[i >> 2] >> (8 * (i & 3)));
  }
}

// ---------------------------------------------------------------------------
// database ingest (push_database_chunk, preprocess_ntt, realign_db:
// server.cpp:635-748)
// ---------------------------------------------------------------------------

// Coefficient c of a plaintext = bits [bpc*c, bpc*c + bpc) of the
// concatenated bytes of its entries, LSB-first; bits past the end are 0.
template <bool kSynthetic>
__global__ void __launch_bounds__(T) db_pack_kernel(const uint8_t *entries, uint64_t seed,
                                                    size_t pt0, uint64_t *coeffs, int entry_size,
                                                    int epp, int bpc) {
  const size_t pt = blockIdx.x;
  const uint64_t total_bits = (uint64_t)epp * entry_size * 8;
  const uint8_t *base = entries ? entries + pt * (size_t)epp * entry_size : nullptr;
  for (int c = threadIdx.x; c < kN; c += T) {
    const uint64_t bit0 = (uint64_t)c * bpc;
    uint64_t v = 0;
    if (bit0 < total_bits) {
      const uint64_t byte0 = bit0 >> 3;
      const int off = (int)(bit0 & 7);
      const uint64_t nbytes_total = total_bits >> 3;
      uint64_t acc = 0;
      for (int j = 0; j < 4; ++j) {  // bpc <= 24 bits spans at most 4 bytes
        const uint64_t by = byte0 + j;
        if (by >= nbytes_total) break;
        uint32_t val;
        if (kSynthetic) {
          const uint64_t e = (pt0 + pt) * (uint64_t)epp + by / entry_size;
          val = gen_entry_byte(seed, e, by % entry_size);
        } else {
          val = base[by];
        }
        acc |= (uint64_t)val << (8 * j);
      }
      v = (acc >> off) & ((1ULL << bpc) - 1);
    }
    coeffs[pt * kN + c] = v;
  }
}

// transform_to_ntt_inplace(Plaintext) (server.cpp:709): centred lift of the
// t-residues into Z_q, forward NTT; then realign_db into the scan layout
// dbs[c][col][row] with each value stored as lo30 | hi30 << 32.
__global__ void __launch_bounds__(T) db_ntt_scatter_kernel(const uint64_t *coeffs, size_t pt0,
                                                           uint64_t *dbs, int n1, int n_rest,
                                                           ModTab M, Consts C) {
  __shared__ uint64_t sa[kSmemPoly], sb[kSmemPoly];
  const int tid = threadIdx.x;
  const size_t pt = pt0 + blockIdx.x;
  const uint64_t *src = coeffs + (size_t)blockIdx.x * kN;
  const uint64_t thr = (C.t + 1) >> 1, inc = C.q - C.t;
  uint64_t r[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const uint64_t v = src[strided_idx(tid, e)];
    r[e] = v >= thr ? v + inc : v;
  }
  ntt_fwd(r, sa, sb, M);
  const size_t row = pt / n1, col = pt % n1;
  const size_t plane = (size_t)n1 * n_rest;
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const size_t c = slot_idx(tid, e);
    dbs[c * plane + col * n_rest + row] = (r[e] & 0x3FFFFFFFULL) | ((r[e] >> 30) << 32);
  }
}

// One plaintext back from the device database: its NTT slots gathered from
// dbs, the inverse transform, and the plain lift of ingest undone (stored
// coefficients are v or v + q - t for v >= (t + 1) / 2).  Natural order out.
__global__ void __launch_bounds__(T) db_plaintext_kernel(const uint64_t *dbs, int n1, int n_rest,
                                                         size_t pt, uint64_t *out, ModTab M,
                                                         Consts C) {
  __shared__ uint64_t sa[kSmemPoly], sb[kSmemPoly];
  const int tid = threadIdx.x;
  const size_t row = pt / n1, col = pt % n1;
  const size_t plane = (size_t)n1 * n_rest;
  uint64_t r[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const uint64_t w = dbs[(size_t)slot_idx(tid, e) * plane + col * n_rest + row];
    r[e] = (w & 0x3FFFFFFFULL) | ((w >> 32) << 30);
  }
  ntt_inv(r, sa, sb, M);
  const uint64_t thr = (C.t + 1) >> 1, inc = C.q - C.t;
#pragma unroll
  for (int e = 0; e < 8; ++e) out[strided_idx(tid, e)] = r[e] < thr ? r[e] : r[e] - inc;
}

__global__ void db_from_aligned_kernel(const uint64_t *aligned, uint64_t *dbs, int n1,
                                       int n_rest) {
  const size_t plane = (size_t)n1 * n_rest;
  const size_t total = plane * kN;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t c = i / plane, rem = i % plane;
    const size_t col = rem / n_rest, row = rem % n_rest;
    const uint64_t v = aligned[c * plane + row * n1 + col];
    dbs[i] = (v & 0x3FFFFFFFULL) | ((v >> 30) << 32);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

void launch_ntt(const ModTab &M, uint64_t *polys, size_t count, bool inverse, cudaStream_t s,
                bool pdl) {
  if (!count) return;
  launch_kernel(pdl, ntt_kernel, dim3((unsigned)count), dim3(T), 0, s, M, polys, inverse ? 1 : 0,
                (size_t)0);
}

void launch_ntt_groups(const ModTab &M, uint64_t *polys, int count, int groups,
                       size_t group_stride, bool inverse, cudaStream_t s, bool pdl) {
  if (count <= 0 || groups <= 0) return;
  launch_kernel(pdl, ntt_kernel, dim3((unsigned)count, (unsigned)groups), dim3(T), 0, s, M, polys,
                inverse ? 1 : 0, group_stride);
}

void launch_query_prep(const uint64_t *leaves, size_t leaves_stride, uint4 *qs, size_t qs_stride,
                       int n1, int batch, const ModTab &Mq, cudaStream_t s, bool pdl) {
  launch_kernel(pdl, query_prep_kernel, dim3(n1, batch, 2), dim3(T), 0, s,
                leaves, leaves_stride, qs, qs_stride, (size_t)n1, (size_t)1, Mq);
}

void launch_query_prep_batched(const uint64_t *leaves, size_t leaves_stride, uint4 *qsb, int n1,
                               int batch, const ModTab &Mq, cudaStream_t s, bool pdl) {
  launch_kernel(pdl, query_prep_kernel, dim3(n1, batch, 2), dim3(T), 0, s,
                leaves, leaves_stride, qsb, (size_t)1, (size_t)n1 * batch, (size_t)batch, Mq);
}

void launch_query_prep_plane(const uint64_t *leaves, size_t leaves_stride, uint64_t *plane,
                             int n1, int batch, const ModTab &Mq, cudaStream_t s, bool pdl) {
  launch_kernel(pdl, query_prep_plane_kernel, dim3(n1, batch, 2), dim3(T), 0, s, leaves,
                leaves_stride, plane, n1, Mq);
}

void launch_modswitch_pack(const uint64_t *res, size_t res_stride, uint64_t *resp,
                           uint8_t *packed, size_t packed_bytes, int batch, const Consts &C,
                           cudaStream_t s, bool pdl, const uint32_t *status,
                           uint32_t *status_out) {
  // the packed stream is 2N w bits exactly; each slice fills its own words
  const size_t smem = ((size_t)(2 * kN / kModSlices) * C.small_q_width / 32 + 2) * sizeof(uint32_t);
  launch_kernel(pdl, modswitch_pack_kernel<true>, dim3(kModSlices, batch), dim3(T), smem, s, res,
                res_stride, resp, packed, (int)packed_bytes, C, status, status_out);
}

void launch_pack_response(const uint64_t *resps, size_t stride, uint8_t *packed,
                          size_t packed_bytes, int batch, const Consts &C, cudaStream_t s) {
  const size_t smem = ((size_t)(2 * kN / kModSlices) * C.small_q_width / 32 + 2) * sizeof(uint32_t);
  launch_kernel(false, modswitch_pack_kernel<false>, dim3(kModSlices, batch), dim3(T), smem, s,
                resps, stride, (uint64_t *)nullptr, packed, (int)packed_bytes, C,
                (const uint32_t *)nullptr, (uint32_t *)nullptr);
}

void launch_db_pack(const uint8_t *entries, uint64_t *coeffs, size_t num_pt, int entry_size,
                    int entries_per_pt, int bits_per_coeff, cudaStream_t s) {
  if (!num_pt) return;
  db_pack_kernel<false><<<(unsigned)num_pt, T, 0, s>>>(entries, 0, 0, coeffs, entry_size,
                                                      entries_per_pt, bits_per_coeff);
}

void launch_db_gen_pack(uint64_t seed, size_t pt0, uint64_t *coeffs, size_t num_pt,
                        int entry_size, int entries_per_pt, int bits_per_coeff, cudaStream_t s) {
  if (!num_pt) return;
  db_pack_kernel<true><<<(unsigned)num_pt, T, 0, s>>>(nullptr, seed, pt0, coeffs, entry_size,
                                                     entries_per_pt, bits_per_coeff);
}

void launch_db_ntt_scatter(uint64_t *coeffs, size_t pt0, size_t count, uint64_t *dbs, int n1,
                           int n_rest, const ModTab &Mq, const Consts &C, cudaStream_t s) {
  if (!count) return;
  db_ntt_scatter_kernel<<<(unsigned)count, T, 0, s>>>(coeffs, pt0, dbs, n1, n_rest, Mq, C);
}

void launch_db_plaintext(const uint64_t *dbs, int n1, int n_rest, size_t pt, uint64_t *out,
                         const ModTab &Mq, const Consts &C, cudaStream_t s) {
  db_plaintext_kernel<<<1, T, 0, s>>>(dbs, n1, n_rest, pt, out, Mq, C);
}

void launch_db_from_aligned(const uint64_t *aligned, uint64_t *dbs, int n1, int n_rest,
                            cudaStream_t s) {
  db_from_aligned_kernel<<<152 * 8, 256, 0, s>>>(aligned, dbs, n1, n_rest);
}

}  // namespace opir
