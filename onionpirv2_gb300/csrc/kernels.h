// kernels.h -- launchers for the OnionPIRv2 query-path kernels (sm_103a).
// Host code calls these; every launcher enqueues on the given stream and
// returns without synchronising.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace opir {

// Per-query key pointers.
struct QueryDesc {
  const uint64_t *galois;    // [h][2][2][N]   key k, modulus (q, p), NTT form
  const uint64_t *galois_s;  // the same layout: Shoup companions floor(k 2^64 / modulus)
  const uint64_t *gsw_key;   // [2 l_key][2][N] RGSW(sk), NTT form
};

// Key pointers of up to kMaxKeyBatch queries, passed to kernels by value
// (no per-query host->device copy); launchers split larger batches.
constexpr int kMaxKeyBatch = 64;
struct KeyBatch {
  QueryDesc q[kMaxKeyBatch];
};

// Scalars of the parameter set shared by all kernels.
struct Consts {
  uint64_t q, p, t;
  uint64_t p_half;            // p >> 1
  uint64_t p_half_mod_q;
  uint64_t p_inv_q, p_inv_q_s;  // p^-1 mod q and Shoup companion
  uint64_t two30, two30_s;    // 2^30 mod q
  uint64_t two60, two60_s;    // 2^60 mod q
  uint64_t ms_mant;           // (double)small_q / (double)q == ms_mant * 2^-ms_shift
  int ms_shift;
  int small_q_width;
  int l, base_log2, l_key, base_log2_key;
};

// Per-device kernel attributes (dynamic shared memory opt-in); call once per
// device before the first launch.
cudaError_t init_kernel_attributes();

// Which dependent kernels of the query pipeline are programmatic launches, a
// bit per launch kind: in a captured CUDA graph (g_pdl_graph, OPIR_PDL_GRAPH)
// and in direct launches (g_pdl_direct, OPIR_PDL); set by
// init_kernel_attributes.
enum { kPdlExpand = 1, kPdlQtg = 2, kPdlPrep = 4, kPdlNtt = 8, kPdlFold = 16, kPdlModswitch = 32 };
extern int g_pdl_graph, g_pdl_direct;

// Launch `k` on stream s; with `pdl` the launch may become
// resident while the previous kernel of the stream still runs, so `k` must
// call grid_dep_wait() (common.cuh) before touching what earlier launches
// write.  Errors surface through cudaGetLastError like <<< >>> launches.
template <typename... P, typename... A>
inline void launch_kernel(bool pdl, void (*k)(P...), dim3 grid, dim3 block, size_t smem,
                          cudaStream_t s, A &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, k, static_cast<A &&>(args)...);
}

// ---- batched transforms on polynomials in global memory (natural order in,
// NTT slot order out for forward; slot order in, natural out for inverse)
// (pdl: a programmatic launch after the previous kernel of the pipeline)
void launch_ntt(const ModTab &M, uint64_t *polys, size_t count, bool inverse, cudaStream_t s,
                bool pdl = false);
// `count` consecutive polynomials in each of `groups` groups group_stride
// words apart (one per query of a batch)
void launch_ntt_groups(const ModTab &M, uint64_t *polys, int count, int groups,
                       size_t group_stride, bool inverse, cudaStream_t s, bool pdl = false);

// ---- launch forms of the tree stages
// Every tree stage has a one-CTA form (a whole ciphertext per CTA), a
// two-CTA form (expansion and folding: the two polynomials' transforms on two
// CTAs), a thread-block-cluster form (one ciphertext's independent
// transforms spread over 4-6 CTAs) and, for folding, a wide cluster (ten
// CTAs per pair: one transform each).  Which is fastest depends on the launch's
// work count (nodes, RGSW ciphertexts or fold pairs, times the queries of the
// launch) and on the GPU: TreeForms holds the autotuner's choice per count;
// a count it does not hold takes the measured default thresholds.
enum { kStageExpand = 0, kStageQtg = 1, kStageFold = 2 };
enum { kFormDefault = -1, kFormOne = 0, kFormPair = 1, kFormCluster = 2, kFormWide = 3 };
constexpr int kTreeForms = 4;
struct TreeForms {
  static constexpr int kMax = 96;
  int n[3] = {0, 0, 0};
  int count[3][kMax] = {}, form[3][kMax] = {};
  int pick(int stage, int cnt) const {
    for (int i = 0; i < n[stage]; ++i)
      if (count[stage][i] == cnt) return form[stage][i];
    return kFormDefault;
  }
  bool set(int stage, int cnt, int f) {
    for (int i = 0; i < n[stage]; ++i)
      if (count[stage][i] == cnt) {
        form[stage][i] = f;
        return true;
      }
    if (n[stage] == kMax) return false;
    count[stage][n[stage]] = cnt;
    form[stage][n[stage]++] = f;
    return true;
  }
};
// whether `form` exists for this stage and parameter set (the cluster forms
// are written for l = 5 data digits and l_key = 10 key digits)
bool tree_form_valid(int stage, int form, const Consts &C);
// the form the measured default thresholds give a launch of `count` items
int tree_default_form(int stage, int count, const Consts &C);

// ---- query expansion, one tree level for every query of the batch
// cur: [B][nodes_in][2][N], nxt: [B][2*nodes_in][2][N]
void launch_expand_level(const uint64_t *cur, uint64_t *nxt, size_t in_stride, size_t out_stride,
                         const QueryDesc *qd, int level, int live_nodes, int batch,
                         const ModTab &Mq, const ModTab &Mp, const Consts &C, cudaStream_t s,
                         bool pdl = false, const TreeForms *forms = nullptr);

// ---- RGSW reconstruction (query_to_gsw) for all further dimensions
// leaves: [B][u][2][N] (coefficient form), gsw_out: [B][ndim-1][2l][2][N]
void launch_query_to_gsw(const uint64_t *leaves, size_t leaves_stride, uint64_t *gsw_out,
                         size_t gsw_stride, const QueryDesc *qd, int n1, int num_cts, int batch,
                         const ModTab &Mq, const Consts &C, cudaStream_t s, bool pdl = false,
                         const TreeForms *forms = nullptr);

// ---- first dimension
// NTT the first n1 leaves and transpose to the scan operand Qs[b][c][k]
void launch_query_prep(const uint64_t *leaves, size_t leaves_stride, uint4 *qs, size_t qs_stride,
                       int n1, int batch, const ModTab &Mq, cudaStream_t s, bool pdl = false);
// the same into the batched operand layout qsb[c][k][b]
void launch_query_prep_batched(const uint64_t *leaves, size_t leaves_stride, uint4 *qsb, int n1,
                               int batch, const ModTab &Mq, cudaStream_t s, bool pdl = false);
// out[b][row][poly][c] = sum_k DB[c][k][row] * Q[b][c][k][poly] mod q  (NTT form)
// (bulk-copy pipelined kernel in tile configuration `cfg` -- < 0: the
// default -- when the shape fits it, else a plain kernel; status collects
// bounded-wait timeouts, see async.cuh).  Returns the configuration that
// ran, -1 for the plain kernel.
int launch_scan(const uint64_t *dbs, const uint4 *qs, size_t qs_stride, uint64_t *out,
                size_t out_stride, int n1, int n_rest, int batch, const Consts &C,
                uint64_t mu_lo, uint64_t mu_hi, uint32_t *status, cudaStream_t s, int cfg = -1);
// The bulk-copy kernel over `planes` NTT slots, writing slot c of row `row`
// at out[row o_row + c] and out[row o_row + o_poly + c]; slots below
// mod_planes reduce mod C0 (q, 2^30 and 2^60 mod q with Shoup companions,
// Barrett mu0), the rest mod C1: the multi-modulus path runs both primes in
// one launch.  Returns the configuration that ran, -1 when the shape does
// not fit it (nothing launched).
int launch_scan_planes(const uint64_t *dbs, const uint4 *qs, size_t qs_stride, uint64_t *out,
                       size_t out_stride, int n1, int n_rest, int batch, int planes,
                       size_t o_row, size_t o_poly, int mod_planes, const Consts &C0,
                       const uint64_t mu0[2], const Consts &C1, const uint64_t mu1[2],
                       uint32_t *status, cudaStream_t s);
// compiled tile configurations of the bulk scan: {rows per thread, warps,
// k-steps per stage, stages, CTAs per SM, Karatsuba products}
int scan_config_count();
void scan_config_desc(int i, uint32_t out[6]);
cudaError_t init_scan_attributes();
// Batched product: one pass over the database for up to 32 queries at a time
// (qsb[c][k][b], out as launch_scan).  Returns false if the shape is not
// supported (caller falls back to launch_scan).
bool launch_scan_batched(const uint64_t *dbs, const uint4 *qsb, uint64_t *out, size_t out_stride,
                         int n1, int n_rest, int batch, const Consts &C, uint64_t mu_lo,
                         uint64_t mu_hi, uint32_t *status, cudaStream_t s);

// NTT the first n1 leaves into a plain plane[b][k][poly][c] of residues
// (query operand of the tensor-core path)
void launch_query_prep_plane(const uint64_t *leaves, size_t leaves_stride, uint64_t *plane,
                             int n1, int batch, const ModTab &Mq, cudaStream_t s,
                             bool pdl = false);
// Batched product on the tcgen05 tensor cores (tc_scan.cu): residues split
// into 8-bit (database) and 8- or 9-bit (query) limbs held as bf16, exact
// fp32 accumulation in tensor memory.
// The database needs its limb plane dbl (tc_db_limb_bytes, built by
// launch_db_limbs from dbs).  launch_tc_query_limbs splits the query plane
// of launch_query_prep_plane into ql (tc_query_limb_bytes(n1, batch) bytes);
// launch_tc_scan then writes the output of launch_scan and returns the number
// of kernels it launched.
bool tc_scan_supported(int n1, int n_rest);
size_t tc_db_limb_bytes(int n1, int n_rest);
size_t tc_query_limb_bytes(int n1, int batch);
cudaError_t init_tc_attributes();
void launch_db_limbs(const uint64_t *dbs, uint16_t *dbl, int n1, int n_rest, cudaStream_t s);
// limbs: the width of the query limbs, 8 bits (eight limbs, 64 limb products
// per modular multiply-add) or 9 bits (seven limbs, 56); -1 takes the one
// with fewer MMA columns for each pass.  launch_tc_query_limbs and
// launch_tc_scan must be given the same choice.
enum { kTcLimbs8 = 0, kTcLimbs9 = 1 };
// pair: the kernel form, one CTA per tile (0, and the default -1) or CTA
// pairs sharing M = 256 MMAs (1, tcgen05 cta_group::2: each CTA loads half
// of the query tile; where the rows form pairs of 16-row tiles).  The query
// limb layout depends on it: give both calls the same.
void launch_tc_query_limbs(const uint64_t *plane, uint16_t *ql, int n1, int n_rest, int batch,
                           cudaStream_t s, int limbs = -1, int pair = -1);
// the passes (of up to 64 queries) a batch takes, and the query limb width
// (8 or 9) that a pass of min(batch, 64) queries uses
int tc_pass_count(int batch);
int tc_query_limb_width(int batch, int limbs);
// whether a pass of min(batch, 64) queries runs as CTA pairs
bool tc_pair_form(int n_rest, int batch, int limbs, int pair);
// launch_tc_scan returns -1 when a pass could not be launched (the tensor
// copy maps of a CTA pair could not be made).
// ring: the shared-memory pipeline of the tensor kernel, 64 k x 4 stages
// (n1 a multiple of 64) or 32 k x 8 stages; an invalid choice (or -1) takes
// the first that fits.
enum { kTcRing64x4 = 0, kTcRing32x8 = 1 };
bool tc_ring_valid(int ring, int n1);
int launch_tc_scan(const uint16_t *dbl, const uint16_t *ql, uint64_t *out, size_t out_stride,
                   int n1, int n_rest, int batch, uint64_t q, uint64_t mu_lo, uint64_t mu_hi,
                   uint64_t r64, uint64_t r128, uint32_t *status, cudaStream_t s, int ring = -1,
                   int limbs = -1, int pair = -1);

// ---- one folding level (other_dim_mux) on ciphertexts held in NTT form:
// res[b][j] += RGSW x INTT(res[j+half] - res[j]) for j < half (the
// difference goes back to coefficient form for its gadget digits; the sum
// stays in NTT form)
void launch_fold(uint64_t *res, size_t res_stride, const uint64_t *gsw, size_t gsw_stride,
                 int half, int batch, const ModTab &Mq, const Consts &C, cudaStream_t s,
                 bool pdl = false, const TreeForms *forms = nullptr);

// ---- mod switch to small_q + response bit packing
// (status_out: block 0 also copies the device status word *status there,
// once every earlier kernel of the stream has completed)
void launch_modswitch_pack(const uint64_t *res, size_t res_stride, uint64_t *resp,
                           uint8_t *packed, size_t packed_bytes, int batch, const Consts &C,
                           cudaStream_t s, bool pdl = false, const uint32_t *status = nullptr,
                           uint32_t *status_out = nullptr);

// ---- response bit packing alone (save_resp_to_stream of any response
// mod small_q): resps[b] at stride words -> packed[b][packed_bytes]
void launch_pack_response(const uint64_t *resps, size_t stride, uint8_t *packed,
                          size_t packed_bytes, int batch, const Consts &C, cudaStream_t s);

// ---- database ingest
// entry bytes (device) -> plaintext coefficients (bits_per_coeff LSB-first)
void launch_db_pack(const uint8_t *entries, uint64_t *coeffs, size_t num_pt, int entry_size,
                    int entries_per_pt, int bits_per_coeff, cudaStream_t s);
// seeded synthetic entries straight to plaintext coefficients
void launch_db_gen_pack(uint64_t seed, size_t pt0, uint64_t *coeffs, size_t num_pt,
                        int entry_size, int entries_per_pt, int bits_per_coeff, cudaStream_t s);
// centred lift + NTT + scatter into the scan layout dbs[c][col][row] (30-bit split words)
void launch_db_ntt_scatter(uint64_t *coeffs, size_t pt0, size_t count, uint64_t *dbs, int n1,
                           int n_rest, const ModTab &Mq, const Consts &C, cudaStream_t s);
// reference layout db_aligned[c][row*n1+col] (NTT form) -> scan layout
// plaintext `pt` of the database back in coefficient form (plain lift undone)
void launch_db_plaintext(const uint64_t *dbs, int n1, int n_rest, size_t pt, uint64_t *out,
                         const ModTab &Mq, const Consts &C, cudaStream_t s);
void launch_db_from_aligned(const uint64_t *aligned, uint64_t *dbs, int n1, int n_rest,
                            cudaStream_t s);

// ---- keys: coefficient-form RGSW rows -> NTT form (in place, slot order)
// (same as launch_ntt forward; kept for readability at the call site)

}  // namespace opir
