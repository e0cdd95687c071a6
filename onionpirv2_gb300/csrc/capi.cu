// capi.cu -- host side of the GB300 OnionPIRv2 server: context, device
// memory, key and database ingest, and the query pipeline behind the C ABI
// declared in include/onionpir_gpu.h.
//
// Pipeline per query batch (PirServer::make_query, server.cpp:520-579):
//   expand   h launches      fast_expand_qry          server.cpp:383-428
//   convert  1 launch        query_to_gsw             gsw_eval.cpp:254-286
//   1st dim  3 launches      evaluate_first_dim       server.cpp:124-293
//   fold     ndim-1 launches other_dim_mux            server.cpp:295-334
//   finish   1 launch        mod_switch_inplace + save_resp_to_stream
//                                                      server.cpp:581-633,779-801
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/onionpir_gpu.h"
#include "kernels.h"

using namespace opir;

namespace {

using u128 = unsigned __int128;

uint64_t mulmod(uint64_t a, uint64_t b, uint64_t q) { return (uint64_t)(((u128)a * b) % q); }
uint64_t powmod(uint64_t b, uint64_t e, uint64_t q) {
  uint64_t r = 1 % q;
  b %= q;
  while (e) {
    if (e & 1) r = mulmod(r, b, q);
    b = mulmod(b, b, q);
    e >>= 1;
  }
  return r;
}
bool is_prime(uint64_t n) {
  static const uint64_t bases[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
  if (n < 2) return false;
  for (uint64_t b : bases) {
    if (n == b) return true;
    if (n % b == 0) return false;
  }
  uint64_t d = n - 1;
  int s = 0;
  while (!(d & 1)) d >>= 1, s++;
  for (uint64_t b : bases) {
    uint64_t x = powmod(b, d, n);
    if (x == 1 || x == n - 1) continue;
    bool comp = true;
    for (int r = 1; r < s && comp; r++) {
      x = mulmod(x, x, n);
      if (x == n - 1) comp = false;
    }
    if (comp) return false;
  }
  return true;
}
uint64_t shoup(uint64_t w, uint64_t q) { return (uint64_t)(((u128)w << 64) / q); }
unsigned bitlen(uint64_t x) { return x ? 64 - __builtin_clzll(x) : 0; }
uint64_t brv(uint64_t x, unsigned bits) {
  uint64_t y = 0;
  for (unsigned i = 0; i < bits; i++) y = (y << 1) | ((x >> i) & 1);
  return y;
}
// smallest primitive 2N-th root of unity mod q
uint64_t minimal_root(uint64_t q) {
  const uint64_t two_n = 2 * kN, cof = (q - 1) / two_n;
  uint64_t psi = 0;
  for (uint64_t g = 2; g < q && !psi; g++) {
    uint64_t c = powmod(g, cof, q);
    if (powmod(c, two_n / 2, q) == q - 1) psi = c;
  }
  if (!psi) return 0;
  uint64_t best = psi, sq = mulmod(psi, psi, q), cur = psi;
  for (uint64_t k = 1; k < two_n / 2; k++) {
    cur = mulmod(cur, sq, q);
    if (cur < best) best = cur;
  }
  return best;
}

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t alloc(size_t n) {
    if (n <= bytes && p) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&p, n ? n : 16);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  template <class T>
  T *as() const {
    return static_cast<T *>(p);
  }
};

struct PinnedBuf {
  void *p = nullptr;
  size_t bytes = 0;
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
  cudaError_t alloc(size_t n) {
    if (n <= bytes && p) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMallocHost(&p, n ? n : 16);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
};

struct ModTables {
  DevBuf fwd, inv;
  ModTab tab{};
  uint64_t psi = 0;
};

struct Db {
  opir_db_shape shape{};
  uint64_t num_pt = 0;
  int ndim = 1, u = 1, h = 0;
  DevBuf dbs;
  DevBuf dbl;              // bf16 limb plane of dbs for the tensor-core product (built on demand)
  bool dbl_valid = false;  // cleared whenever dbs changes
};

struct Client {
  DevBuf galois;
  uint32_t levels = 0;
  DevBuf gsw;
  bool has_gsw = false;
};

struct Workspace {
  // sized for (batch, shape); grown on demand
  DevBuf exp0, exp1, gsw, qs, ql, res, resp, packed, queries, ingest, coeffs;
  PinnedBuf h_in, h_out;
};

struct Err {
  int code;
};

}  // namespace

struct opir_ctx {
  std::mutex mu;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  opir_params prm{};
  Consts C{};
  ModTables Mq, Mp;
  uint64_t resp_bytes = 0;
  std::map<uint32_t, std::unique_ptr<Db>> dbs;
  uint32_t next_db = 1;
  std::map<uint64_t, std::unique_ptr<Client>> clients;
  Workspace ws;
  DevBuf status;  // device status word: bounded-wait timeouts (async.cuh)
  bool batch_scan = true;  // batched GEMM for batches >= 2 (OPIR_BATCH_SCAN=0 turns it off)
  // batched GEMM engine: 0 = integer multiply-add kernel, 1 = tensor cores
  // from tc_min_batch queries on (OPIR_TC, OPIR_TC_MIN_BATCH)
  int tc_mode = 1;
  int tc_min_batch = 2;
  uint64_t r64 = 0, r128 = 0;  // 2^64 and 2^128 mod q
  bool timing = false;
  cudaEvent_t ev[8] = {};
  float stage_ms[6] = {};
  bool stage_valid = false;
  uint64_t launches = 0;
  std::string err;

  int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    err = buf;
    return code;
  }
  int cuda_fail(cudaError_t e, const char *what) {
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      return fail(OPIR_ERR_OOM, "%s: out of device memory", what);
    }
    return fail(OPIR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  }
};

#define CK(call, what)                                   \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return ctx->cuda_fail(e_, what); \
  } while (0)

namespace {

int build_modtab(opir_ctx *ctx, ModTables &T, uint64_t q) {
  T.psi = minimal_root(q);
  if (!T.psi) return ctx->fail(OPIR_ERR_ARG, "no primitive 2N-th root mod %llu", (unsigned long long)q);
  std::vector<uint64_t> pw(kN), pwi(kN);
  const uint64_t psi_inv = powmod(T.psi, q - 2, q);
  pw[0] = pwi[0] = 1;
  for (int i = 1; i < kN; i++) {
    pw[i] = mulmod(pw[i - 1], T.psi, q);
    pwi[i] = mulmod(pwi[i - 1], psi_inv, q);
  }
  std::vector<ulonglong2> fwd(kN), inv(kN);
  for (int i = 0; i < kN; i++) {
    const uint64_t e = brv(i, kLogN);
    fwd[i].x = pw[e];
    fwd[i].y = shoup(pw[e], q);
    inv[i].x = pwi[e];
    inv[i].y = shoup(pwi[e], q);
  }
  CK(T.fwd.alloc(kN * sizeof(ulonglong2)), "alloc twiddles");
  CK(T.inv.alloc(kN * sizeof(ulonglong2)), "alloc twiddles");
  CK(cudaMemcpy(T.fwd.p, fwd.data(), kN * sizeof(ulonglong2), cudaMemcpyHostToDevice), "upload twiddles");
  CK(cudaMemcpy(T.inv.p, inv.data(), kN * sizeof(ulonglong2), cudaMemcpyHostToDevice), "upload twiddles");
  T.tab.fwd = T.fwd.as<ulonglong2>();
  T.tab.inv = T.inv.as<ulonglong2>();
  T.tab.q = q;
  T.tab.n_inv = powmod(kN, q - 2, q);
  T.tab.n_inv_s = shoup(T.tab.n_inv, q);
  const u128 mu = (~(u128)0) / q;
  T.tab.mu_lo = (uint64_t)mu;
  T.tab.mu_hi = (uint64_t)(mu >> 64);
  return OPIR_OK;
}

// ---- per-query workspace
int ensure_workspace(opir_ctx *ctx, const Db &db, int batch) {
  Workspace &W = ctx->ws;
  const size_t CT = 2 * (size_t)kN * 8;
  const size_t w = (size_t)1 << db.h;
  const size_t n1 = db.shape.fst_dim_sz, nr = db.shape.other_dim_sz;
  const size_t l = ctx->prm.gsw_l;
  CK(W.exp0.alloc(batch * w * CT), "alloc expansion");
  CK(W.exp1.alloc(batch * w * CT), "alloc expansion");
  CK(W.gsw.alloc(batch * (size_t)(db.ndim > 1 ? db.ndim - 1 : 1) * 2 * l * CT), "alloc gsw");
  CK(W.qs.alloc(batch * (size_t)kN * n1 * sizeof(uint4)), "alloc query operand");
  CK(W.res.alloc(batch * nr * CT), "alloc first-dim result");
  CK(W.resp.alloc(batch * CT), "alloc response");
  CK(W.packed.alloc(batch * ctx->resp_bytes + 16), "alloc packed");
  CK(W.queries.alloc(batch * CT), "alloc queries");
  return OPIR_OK;
}

struct Trace {
  uint64_t *leaves = nullptr, *gsw = nullptr, *first_dim = nullptr;
};

void record(opir_ctx *ctx, int i) {
  if (ctx->timing) cudaEventRecord(ctx->ev[i], ctx->stream);
}

// Enqueue the whole query pipeline for `batch` queries already on the device.
int run_pipeline(opir_ctx *ctx, Db &db, int batch, const uint64_t *client_ids,
                 const uint64_t *d_queries, uint64_t *d_resp, uint8_t *d_packed,
                 const Trace *trace) {
  if (batch <= 0) return ctx->fail(OPIR_ERR_ARG, "batch must be positive");
  if (!db.dbs.p) return ctx->fail(OPIR_ERR_STATE, "database has no data");
  std::vector<QueryDesc> desc(batch);
  for (int b = 0; b < batch; b++) {
    auto it = ctx->clients.find(client_ids[b]);
    if (it == ctx->clients.end() || !it->second->galois.p)
      return ctx->fail(OPIR_ERR_UNKNOWN_CLIENT, "no Galois keys for client %llu",
                       (unsigned long long)client_ids[b]);
    if (it->second->levels < (uint32_t)db.h)
      return ctx->fail(OPIR_ERR_ARG, "client %llu has %u Galois levels, database needs %d",
                       (unsigned long long)client_ids[b], it->second->levels, db.h);
    if (db.ndim > 1 && !it->second->has_gsw)
      return ctx->fail(OPIR_ERR_UNKNOWN_CLIENT, "no RGSW key for client %llu",
                       (unsigned long long)client_ids[b]);
    desc[b].galois = it->second->galois.as<uint64_t>();
    desc[b].gsw_key = it->second->gsw.as<uint64_t>();
  }
  int rc = ensure_workspace(ctx, db, batch);
  if (rc) return rc;
  Workspace &W = ctx->ws;
  cudaStream_t s = ctx->stream;
  const QueryDesc *qd = desc.data();  // host array: launchers pass it by value
  const size_t CTW = 2 * (size_t)kN;  // words per ciphertext
  const int h = db.h, u = db.u;
  const size_t w = (size_t)1 << h;
  const size_t n1 = db.shape.fst_dim_sz, nr = db.shape.other_dim_sz;
  const int l = (int)ctx->prm.gsw_l;

  record(ctx, 0);
  // ---- expansion
  const uint64_t *cur = d_queries;
  size_t cur_stride = CTW;
  uint64_t *bufs[2] = {W.exp0.as<uint64_t>(), W.exp1.as<uint64_t>()};
  for (int a = 0; a < h; a++) {
    const int live = (int)((u + ((size_t)1 << (h - a)) - 1) >> (h - a));
    uint64_t *nxt = bufs[a & 1];
    launch_expand_level(cur, nxt, cur_stride, w * CTW, qd, a, live, batch, ctx->Mq.tab,
                        ctx->Mp.tab, ctx->C, s);
    ctx->launches++;
    cur = nxt;
    cur_stride = w * CTW;
  }
  const uint64_t *leaves = cur;
  const size_t leaves_stride = cur_stride;
  record(ctx, 1);
  // ---- convert
  const size_t gsw_stride = (size_t)(db.ndim > 1 ? db.ndim - 1 : 1) * 2 * l * CTW;
  if (db.ndim > 1) {
    launch_query_to_gsw(leaves, leaves_stride, W.gsw.as<uint64_t>(), gsw_stride, qd, (int)n1,
                        (db.ndim - 1) * l, batch, ctx->Mq.tab, ctx->C, s);
    ctx->launches++;
  }
  record(ctx, 2);
  // ---- first dimension
  const size_t qs_stride = (size_t)kN * n1;
  const size_t res_stride = nr * CTW;
  // a batch of queries shares one pass over the database (batched GEMM);
  // a single query (or an unsupported shape) streams it once per query
  const bool batched = batch >= 2 && ctx->batch_scan && nr % 32 == 0 && n1 % 16 == 0;
  const bool tensor = batch >= 2 && ctx->batch_scan && ctx->tc_mode == 1 &&
                      batch >= ctx->tc_min_batch && tc_scan_supported((int)n1, (int)nr);
  if (tensor) {
    if (!db.dbl_valid) {
      CK(db.dbl.alloc(tc_db_limb_bytes((int)n1, (int)nr)), "alloc database limb plane");
      launch_db_limbs(db.dbs.as<uint64_t>(), db.dbl.as<uint16_t>(), (int)n1, (int)nr, s);
      ctx->launches++;
      db.dbl_valid = true;
    }
    CK(W.ql.alloc(tc_query_limb_bytes((int)n1)), "alloc query limbs");
    launch_query_prep_plane(leaves, leaves_stride, W.qs.as<uint64_t>(), (int)n1, batch,
                            ctx->Mq.tab, s);
    record(ctx, 6);
    ctx->launches += launch_tc_scan_batched(
        db.dbl.as<uint16_t>(), W.qs.as<uint64_t>(), W.ql.as<uint16_t>(), W.res.as<uint64_t>(),
        res_stride, (int)n1, (int)nr, batch, ctx->Mq.tab.q, ctx->Mq.tab.mu_lo, ctx->Mq.tab.mu_hi,
        ctx->r64, ctx->r128, ctx->status.as<uint32_t>(), s) - 1;
  } else if (batched) {
    launch_query_prep_batched(leaves, leaves_stride, W.qs.as<uint4>(), (int)n1, batch,
                              ctx->Mq.tab, s);
    record(ctx, 6);
    launch_scan_batched(db.dbs.as<uint64_t>(), W.qs.as<uint4>(), W.res.as<uint64_t>(), res_stride,
                        (int)n1, (int)nr, batch, ctx->C, ctx->Mq.tab.mu_lo, ctx->Mq.tab.mu_hi,
                        ctx->status.as<uint32_t>(), s);
  } else {
    launch_query_prep(leaves, leaves_stride, W.qs.as<uint4>(), qs_stride, (int)n1, batch,
                      ctx->Mq.tab, s);
    record(ctx, 6);
    launch_scan(db.dbs.as<uint64_t>(), W.qs.as<uint4>(), qs_stride, W.res.as<uint64_t>(),
                res_stride, (int)n1, (int)nr, batch, ctx->C, ctx->Mq.tab.mu_lo,
                ctx->Mq.tab.mu_hi, ctx->status.as<uint32_t>(), s);
  }
  record(ctx, 7);
  launch_ntt(ctx->Mq.tab, W.res.as<uint64_t>(), (size_t)batch * nr * 2, true, s);
  ctx->launches += 3;
  record(ctx, 3);
  if (trace && trace->first_dim)
    CK(cudaMemcpyAsync(trace->first_dim, W.res.p, nr * CTW * 8, cudaMemcpyDeviceToHost, s),
       "trace first dim");
  // ---- other dimensions
  size_t cnt = nr;
  for (int i = 1; i < db.ndim; i++) {
    const int half = (int)(cnt / 2);
    launch_fold(W.res.as<uint64_t>(), res_stride, W.gsw.as<uint64_t>() + (size_t)(i - 1) * 2 * l * CTW,
                gsw_stride, half, batch, ctx->Mq.tab, ctx->C, s);
    ctx->launches++;
    cnt = half;
  }
  record(ctx, 4);
  // ---- mod switch + pack
  launch_modswitch_pack(W.res.as<uint64_t>(), res_stride, d_resp, d_packed, ctx->resp_bytes, batch,
                        ctx->C, s);
  ctx->launches++;
  record(ctx, 5);
  CK(cudaGetLastError(), "kernel launch");
  if (trace) {
    if (trace->leaves)
      CK(cudaMemcpyAsync(trace->leaves, leaves, (size_t)u * CTW * 8, cudaMemcpyDeviceToHost, s),
         "trace leaves");
    if (trace->gsw && db.ndim > 1)
      CK(cudaMemcpyAsync(trace->gsw, W.gsw.p, (size_t)(db.ndim - 1) * 2 * l * CTW * 8,
                         cudaMemcpyDeviceToHost, s),
         "trace gsw");
  }
  ctx->stage_valid = ctx->timing;
  return OPIR_OK;
}

// Read and clear the device status word (call with the stream idle).
int check_status(opir_ctx *ctx) {
  uint32_t st = 0;
  CK(cudaMemcpy(&st, ctx->status.p, sizeof st, cudaMemcpyDeviceToHost), "read status");
  if (st) {
    CK(cudaMemset(ctx->status.p, 0, sizeof st), "clear status");
    return ctx->fail(OPIR_ERR_TIMEOUT, "device pipeline wait timed out (status 0x%x)", st);
  }
  return OPIR_OK;
}

int collect_times(opir_ctx *ctx) {
  if (!ctx->timing || !ctx->stage_valid) return OPIR_OK;
  CK(cudaEventSynchronize(ctx->ev[5]), "timing");
  float ms;
  const int pairs[6][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 4}, {4, 5}, {6, 7}};
  for (int i = 0; i < 6; i++) {
    CK(cudaEventElapsedTime(&ms, ctx->ev[pairs[i][0]], ctx->ev[pairs[i][1]]), "timing");
    ctx->stage_ms[i] = ms;
  }
  return OPIR_OK;
}

Db *find_db(opir_ctx *ctx, uint32_t id) {
  auto it = ctx->dbs.find(id);
  return it == ctx->dbs.end() ? nullptr : it->second.get();
}

int ensure_db_storage(opir_ctx *ctx, Db &db) {
  CK(db.dbs.alloc(db.num_pt * (size_t)kN * 8), "alloc database");
  return OPIR_OK;
}

int ingest_chunk_coeffs(opir_ctx *ctx, Db &db, size_t pt0, size_t count) {
  db.dbl_valid = false;
  launch_db_ntt_scatter(ctx->ws.coeffs.as<uint64_t>(), pt0, count, db.dbs.as<uint64_t>(),
                        (int)db.shape.fst_dim_sz, (int)db.shape.other_dim_sz, ctx->Mq.tab, ctx->C,
                        ctx->stream);
  ctx->launches++;
  CK(cudaGetLastError(), "ingest launch");
  return OPIR_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

int opir_ctx_create(const opir_params *P, int device, opir_ctx **out) {
  if (!P || !out) return OPIR_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return OPIR_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return OPIR_ERR_ARG;
  std::unique_ptr<opir_ctx> ctx(new opir_ctx());
  ctx->device = device;
  ctx->prm = *P;
  const uint64_t q = P->coeff_modulus, p = P->special_modulus;
  if (P->poly_degree != (uint32_t)kN) return OPIR_ERR_ARG;
  if (!is_prime(q) || !is_prime(p) || q % (2 * kN) != 1 || p % (2 * kN) != 1) return OPIR_ERR_ARG;
  // the 30-bit split of the scan needs q < 2^60; expansion reduces mod p
  // with one subtraction (q < 2p)
  if (q >= (1ULL << 60) || p >= q || q >= 2 * p) return OPIR_ERR_ARG;
  if (!P->gsw_l || !P->gsw_l_key || P->gsw_l > 60 || P->gsw_l_key > 60) return OPIR_ERR_ARG;
  if ((uint64_t)P->gsw_l * P->gsw_base_log2 < bitlen(q) ||
      (uint64_t)P->gsw_l_key * P->gsw_base_log2_key < bitlen(q) || P->gsw_base_log2 > 32 ||
      P->gsw_base_log2_key > 32)
    return OPIR_ERR_ARG;
  if (!is_prime(P->small_modulus) || P->small_modulus >= q || P->plain_modulus < 2)
    return OPIR_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return OPIR_ERR_CUDA;
  opir_ctx *c = ctx.get();
  int rc = build_modtab(c, c->Mq, q);
  if (rc) return rc;
  rc = build_modtab(c, c->Mp, p);
  if (rc) return rc;
  if (init_kernel_attributes() != cudaSuccess || init_scan_attributes() != cudaSuccess ||
      init_tc_attributes() != cudaSuccess)
    return OPIR_ERR_CUDA;
  if (c->status.alloc(sizeof(uint32_t)) != cudaSuccess ||
      cudaMemset(c->status.p, 0, sizeof(uint32_t)) != cudaSuccess)
    return OPIR_ERR_CUDA;
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return OPIR_ERR_CUDA;
  c->stream = c->own_stream;
  if (const char *v = getenv("OPIR_BATCH_SCAN")) c->batch_scan = atoi(v) != 0;
  if (const char *v = getenv("OPIR_TC")) c->tc_mode = atoi(v) != 0;
  if (const char *v = getenv("OPIR_TC_MIN_BATCH")) c->tc_min_batch = atoi(v);
  c->r64 = (uint64_t)(((u128)1 << 64) % q);
  c->r128 = mulmod(c->r64, c->r64, q);
  for (auto &e : c->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return OPIR_ERR_CUDA;
  Consts &C = c->C;
  C.q = q;
  C.p = p;
  C.t = P->plain_modulus;
  C.p_half = p >> 1;
  C.p_half_mod_q = C.p_half % q;
  C.p_inv_q = powmod(p % q, q - 2, q);
  C.p_inv_q_s = shoup(C.p_inv_q, q);
  C.two30 = (uint64_t)(((u128)1 << 30) % q);
  C.two30_s = shoup(C.two30, q);
  C.two60 = (uint64_t)(((u128)1 << 60) % q);
  C.two60_s = shoup(C.two60, q);
  {
    // server.cpp:795: scale = (double)small_q / (double)q, as mantissa * 2^exp
    const double scale = (double)P->small_modulus / (double)q;
    int e;
    const double m = std::frexp(scale, &e);
    C.ms_mant = (uint64_t)std::ldexp(m, 53);
    C.ms_shift = 53 - e;
    if (C.ms_shift <= 0 || C.ms_shift >= 127) return OPIR_ERR_ARG;
  }
  C.small_q_width = (int)std::ceil(std::log2((double)P->small_modulus));  // server.cpp:587-588
  C.l = (int)P->gsw_l;
  C.base_log2 = (int)P->gsw_base_log2;
  C.l_key = (int)P->gsw_l_key;
  C.base_log2_key = (int)P->gsw_base_log2_key;
  c->resp_bytes = (2 * (uint64_t)kN * C.small_q_width + 7) / 8;
  *out = ctx.release();
  return OPIR_OK;
}

void opir_ctx_destroy(opir_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto &e : ctx->ev)
    if (e) cudaEventDestroy(e);
  ctx->dbs.clear();
  ctx->clients.clear();
  cudaStream_t own = ctx->own_stream;
  delete ctx;
  if (own) cudaStreamDestroy(own);
}

int opir_ctx_set_stream(opir_ctx *ctx, void *stream) {
  if (!ctx) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return OPIR_OK;
}

const char *opir_last_error(const opir_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

uint64_t opir_response_bytes(const opir_ctx *ctx) { return ctx ? ctx->resp_bytes : 0; }

int opir_db_create(opir_ctx *ctx, const opir_db_shape *shape, uint32_t *db_id) {
  if (!ctx || !shape || !db_id) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  const opir_db_shape &S = *shape;
  if (!S.fst_dim_sz || !S.other_dim_sz || (S.other_dim_sz & (S.other_dim_sz - 1)))
    return ctx->fail(OPIR_ERR_ARG, "dimensions must be positive, other_dim_sz a power of two");
  if (!S.entry_size || !S.entries_per_pt || !S.bits_per_coeff || S.bits_per_coeff > 24 ||
      (uint64_t)S.entries_per_pt * S.entry_size * 8 > (uint64_t)S.bits_per_coeff * kN)
    return ctx->fail(OPIR_ERR_ARG, "entries do not fit a plaintext");
  if ((1ULL << S.bits_per_coeff) > ctx->prm.plain_modulus)
    return ctx->fail(OPIR_ERR_ARG, "bits_per_coeff exceeds the plaintext modulus");
  auto db = std::make_unique<Db>();
  db->shape = S;
  db->num_pt = (uint64_t)S.fst_dim_sz * S.other_dim_sz;
  int nd = 1;
  while ((1u << (nd - 1)) < S.other_dim_sz) nd++;
  db->ndim = nd;
  db->u = (int)(S.fst_dim_sz + ctx->prm.gsw_l * (nd - 1));
  int h = 0;
  while ((1 << h) < db->u) h++;
  db->h = h;  // pir.h:66-68
  if (h > kLogN) return ctx->fail(OPIR_ERR_ARG, "expansion height %d exceeds log2(N)", h);
  if (cudaSetDevice(ctx->device) != cudaSuccess) return OPIR_ERR_CUDA;
  int rc = ensure_db_storage(ctx, *db);
  if (rc) return rc;
  *db_id = ctx->next_db++;
  ctx->dbs[*db_id] = std::move(db);
  return OPIR_OK;
}

int opir_db_destroy(opir_ctx *ctx, uint32_t db_id) {
  if (!ctx) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (!ctx->dbs.erase(db_id)) return ctx->fail(OPIR_ERR_UNKNOWN_DB, "unknown database %u", db_id);
  return OPIR_OK;
}

int opir_db_push_chunk(opir_ctx *ctx, uint32_t db_id, const uint8_t *entries, uint64_t num_entries,
                       uint64_t chunk_idx) {
  if (!ctx || !entries) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  Db *db = find_db(ctx, db_id);
  if (!db) return ctx->fail(OPIR_ERR_UNKNOWN_DB, "unknown database %u", db_id);
  const opir_db_shape &S = db->shape;
  if (chunk_idx >= S.other_dim_sz) return ctx->fail(OPIR_ERR_ARG, "chunk index out of range");
  if (num_entries != (uint64_t)S.fst_dim_sz * S.entries_per_pt)
    return ctx->fail(OPIR_ERR_ARG, "a chunk holds fst_dim_sz * entries_per_pt entries");
  cudaSetDevice(ctx->device);
  const size_t bytes = num_entries * S.entry_size;
  Workspace &W = ctx->ws;
  CK(W.ingest.alloc(bytes), "alloc ingest");
  CK(W.coeffs.alloc((size_t)S.fst_dim_sz * kN * 8), "alloc ingest");
  CK(W.h_in.alloc(bytes), "alloc pinned");
  // the previous chunk's copy out of h_in must be finished before reuse
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  std::memcpy(W.h_in.p, entries, bytes);
  CK(cudaMemcpyAsync(W.ingest.p, W.h_in.p, bytes, cudaMemcpyHostToDevice, ctx->stream), "upload chunk");
  launch_db_pack(W.ingest.as<uint8_t>(), W.coeffs.as<uint64_t>(), S.fst_dim_sz, (int)S.entry_size,
                 (int)S.entries_per_pt, (int)S.bits_per_coeff, ctx->stream);
  ctx->launches++;
  int rc = ingest_chunk_coeffs(ctx, *db, (size_t)chunk_idx * S.fst_dim_sz, S.fst_dim_sz);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream), "ingest");
  return OPIR_OK;
}

int opir_db_fill_synthetic(opir_ctx *ctx, uint32_t db_id, uint64_t seed) {
  if (!ctx) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  Db *db = find_db(ctx, db_id);
  if (!db) return ctx->fail(OPIR_ERR_UNKNOWN_DB, "unknown database %u", db_id);
  cudaSetDevice(ctx->device);
  const opir_db_shape &S = db->shape;
  const size_t chunk = 16384;
  CK(ctx->ws.coeffs.alloc(chunk * kN * 8), "alloc ingest");
  for (size_t pt0 = 0; pt0 < db->num_pt; pt0 += chunk) {
    const size_t cnt = db->num_pt - pt0 < chunk ? db->num_pt - pt0 : chunk;
    launch_db_gen_pack(seed, pt0, ctx->ws.coeffs.as<uint64_t>(), cnt, (int)S.entry_size,
                       (int)S.entries_per_pt, (int)S.bits_per_coeff, ctx->stream);
    ctx->launches++;
    int rc = ingest_chunk_coeffs(ctx, *db, pt0, cnt);
    if (rc) return rc;
  }
  CK(cudaStreamSynchronize(ctx->stream), "ingest");
  return OPIR_OK;
}

int opir_db_upload_aligned(opir_ctx *ctx, uint32_t db_id, const uint64_t *aligned) {
  if (!ctx || !aligned) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  Db *db = find_db(ctx, db_id);
  if (!db) return ctx->fail(OPIR_ERR_UNKNOWN_DB, "unknown database %u", db_id);
  cudaSetDevice(ctx->device);
  DevBuf tmp;
  const size_t bytes = db->num_pt * (size_t)kN * 8;
  CK(tmp.alloc(bytes), "alloc upload");
  CK(cudaMemcpyAsync(tmp.p, aligned, bytes, cudaMemcpyHostToDevice, ctx->stream), "upload database");
  db->dbl_valid = false;
  launch_db_from_aligned(tmp.as<uint64_t>(), db->dbs.as<uint64_t>(), (int)db->shape.fst_dim_sz,
                         (int)db->shape.other_dim_sz, ctx->stream);
  ctx->launches++;
  CK(cudaGetLastError(), "upload launch");
  CK(cudaStreamSynchronize(ctx->stream), "upload database");
  return OPIR_OK;
}

int opir_set_galois_key(opir_ctx *ctx, uint64_t client_id, const uint64_t *keys, uint32_t levels) {
  if (!ctx || !keys || !levels || levels > (uint32_t)kLogN) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  auto &cl = ctx->clients[client_id];
  if (!cl) cl = std::make_unique<Client>();
  const size_t bytes = (size_t)levels * 4 * kN * 8;
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  CK(cl->galois.alloc(bytes), "alloc Galois keys");
  CK(cudaMemcpy(cl->galois.p, keys, bytes, cudaMemcpyHostToDevice), "upload Galois keys");
  cl->levels = levels;
  return OPIR_OK;
}

int opir_set_gsw_key(opir_ctx *ctx, uint64_t client_id, const uint64_t *rows) {
  if (!ctx || !rows) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  auto &cl = ctx->clients[client_id];
  if (!cl) cl = std::make_unique<Client>();
  const size_t polys = 2 * (size_t)ctx->prm.gsw_l_key * 2;
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  CK(cl->gsw.alloc(polys * kN * 8), "alloc RGSW key");
  CK(cudaMemcpy(cl->gsw.p, rows, polys * kN * 8, cudaMemcpyHostToDevice), "upload RGSW key");
  launch_ntt(ctx->Mq.tab, cl->gsw.as<uint64_t>(), polys, false, ctx->stream);  // server.cpp:497
  ctx->launches++;
  CK(cudaGetLastError(), "key NTT");
  CK(cudaStreamSynchronize(ctx->stream), "key NTT");
  cl->has_gsw = true;
  return OPIR_OK;
}

int opir_erase_client(opir_ctx *ctx, uint64_t client_id) {
  if (!ctx) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (!ctx->clients.erase(client_id))
    return ctx->fail(OPIR_ERR_UNKNOWN_CLIENT, "unknown client %llu", (unsigned long long)client_id);
  return OPIR_OK;
}

static int query_host(opir_ctx *ctx, uint32_t db_id, uint32_t batch, const uint64_t *client_ids,
                      const uint64_t *queries, uint64_t *resps, uint8_t *packed,
                      const Trace *trace) {
  Db *db = find_db(ctx, db_id);
  if (!db) return ctx->fail(OPIR_ERR_UNKNOWN_DB, "unknown database %u", db_id);
  cudaSetDevice(ctx->device);
  const size_t CTB = 2 * (size_t)kN * 8;
  Workspace &W = ctx->ws;
  CK(W.queries.alloc(batch * CTB), "alloc queries");
  CK(W.resp.alloc(batch * CTB), "alloc response");
  CK(W.packed.alloc(batch * ctx->resp_bytes + 16), "alloc packed");
  CK(W.h_in.alloc(batch * CTB), "alloc pinned");
  CK(W.h_out.alloc(batch * (CTB + ctx->resp_bytes)), "alloc pinned");
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  std::memcpy(W.h_in.p, queries, batch * CTB);
  CK(cudaMemcpyAsync(W.queries.p, W.h_in.p, batch * CTB, cudaMemcpyHostToDevice, ctx->stream),
     "upload queries");
  int rc = run_pipeline(ctx, *db, (int)batch, client_ids, W.queries.as<uint64_t>(),
                        W.resp.as<uint64_t>(), W.packed.as<uint8_t>(), trace);
  if (rc) return rc;
  uint8_t *h_resp = static_cast<uint8_t *>(W.h_out.p);
  uint8_t *h_packed = h_resp + batch * CTB;
  if (resps)
    CK(cudaMemcpyAsync(h_resp, W.resp.p, batch * CTB, cudaMemcpyDeviceToHost, ctx->stream),
       "download responses");
  if (packed)
    CK(cudaMemcpyAsync(h_packed, W.packed.p, batch * ctx->resp_bytes, cudaMemcpyDeviceToHost,
                       ctx->stream),
       "download responses");
  CK(cudaStreamSynchronize(ctx->stream), "query");
  {
    int rc2 = check_status(ctx);
    if (rc2) return rc2;
  }
  if (resps) std::memcpy(resps, h_resp, batch * CTB);
  if (packed) std::memcpy(packed, h_packed, batch * ctx->resp_bytes);
  return collect_times(ctx);
}

int opir_make_query(opir_ctx *ctx, uint32_t db_id, uint64_t client_id, const uint64_t *query,
                    uint64_t *resp, uint8_t *packed) {
  if (!ctx || !query) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  return query_host(ctx, db_id, 1, &client_id, query, resp, packed, nullptr);
}

int opir_make_query_batch(opir_ctx *ctx, uint32_t db_id, uint32_t batch, const uint64_t *client_ids,
                          const uint64_t *queries, uint64_t *resps, uint8_t *packed) {
  if (!ctx || !queries || !client_ids || !batch) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  return query_host(ctx, db_id, batch, client_ids, queries, resps, packed, nullptr);
}

int opir_make_query_device(opir_ctx *ctx, uint32_t db_id, uint32_t batch, const uint64_t *client_ids,
                           const uint64_t *d_queries, uint64_t *d_resps, uint8_t *d_packed) {
  if (!ctx || !d_queries || !client_ids || !batch) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  Db *db = find_db(ctx, db_id);
  if (!db) return ctx->fail(OPIR_ERR_UNKNOWN_DB, "unknown database %u", db_id);
  cudaSetDevice(ctx->device);
  return run_pipeline(ctx, *db, (int)batch, client_ids, d_queries, d_resps, d_packed, nullptr);
}

int opir_make_query_trace(opir_ctx *ctx, uint32_t db_id, uint64_t client_id, const uint64_t *query,
                          uint64_t *leaves, uint64_t *gsw, uint64_t *first_dim, uint64_t *resp,
                          uint8_t *packed) {
  if (!ctx || !query) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  Trace t;
  t.leaves = leaves;
  t.gsw = gsw;
  t.first_dim = first_dim;
  return query_host(ctx, db_id, 1, &client_id, query, resp, packed, &t);
}

int opir_set_timing(opir_ctx *ctx, int enable) {
  if (!ctx) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  ctx->timing = enable != 0;
  ctx->stage_valid = false;
  return OPIR_OK;
}

int opir_stage_times(opir_ctx *ctx, float *ms6) {
  if (!ctx || !ms6) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (!ctx->timing || !ctx->stage_valid) return ctx->fail(OPIR_ERR_STATE, "no timed query");
  int rc = collect_times(ctx);
  if (rc) return rc;
  std::memcpy(ms6, ctx->stage_ms, sizeof ctx->stage_ms);
  return OPIR_OK;
}

uint64_t opir_launch_count(const opir_ctx *ctx) { return ctx ? ctx->launches : 0; }

int opir_sync(opir_ctx *ctx) {
  if (!ctx) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  return check_status(ctx);
}

int opir_ntt(opir_ctx *ctx, int mod, int inverse, uint64_t *polys, uint64_t count) {
  if (!ctx || !polys || (mod != 0 && mod != 1)) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  DevBuf d;
  const size_t bytes = count * (size_t)kN * 8;
  CK(d.alloc(bytes), "alloc");
  CK(cudaMemcpyAsync(d.p, polys, bytes, cudaMemcpyHostToDevice, ctx->stream), "upload");
  launch_ntt(mod ? ctx->Mp.tab : ctx->Mq.tab, d.as<uint64_t>(), count, inverse != 0, ctx->stream);
  ctx->launches++;
  CK(cudaGetLastError(), "ntt launch");
  CK(cudaMemcpyAsync(polys, d.p, bytes, cudaMemcpyDeviceToHost, ctx->stream), "download");
  CK(cudaStreamSynchronize(ctx->stream), "ntt");
  return OPIR_OK;
}

int opir_ntt_device(opir_ctx *ctx, int mod, int inverse, uint64_t *d_polys, uint64_t count) {
  if (!ctx || !d_polys || (mod != 0 && mod != 1)) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  launch_ntt(mod ? ctx->Mp.tab : ctx->Mq.tab, d_polys, count, inverse != 0, ctx->stream);
  ctx->launches++;
  CK(cudaGetLastError(), "ntt launch");
  return OPIR_OK;
}

}  // extern "C"

// ===========================================================================
// First dimension without allocation
//
// For callers that must not allocate device memory during a call: a request
// thread with a latency budget (cudaMalloc/cudaFree synchronise the device),
// a host process whose device memory is pre-reserved by another allocator,
// or code that later records the work into a CUDA graph.  The query operand
// of the scan lives in the file-scope array below instead of context
// workspace.  Every GPU that loads this library holds the array until the
// process exits.
// ===========================================================================

// Room for the transposed query operand: n1 * N * 16 bytes, so n1 <= 512.
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;  // 16 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
std::mutex g_noalloc_mu;
constexpr int kMaxDevices = 64;
void *g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once
// per device; the host-side symbol is not a device address).
cudaError_t noalloc_scratch(int device, void **out) {
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  if (!g_noalloc_ptr[device]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[device] = p;
  }
  *out = g_noalloc_ptr[device];
  return cudaSuccess;
}
}  // namespace

extern "C" int opir_first_dim_noalloc(opir_ctx *ctx, uint32_t db_id, const uint64_t *d_fst_cts,
                                      uint64_t *d_out) {
  if (!ctx || !d_fst_cts || !d_out) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  Db *db = find_db(ctx, db_id);
  if (!db) return ctx->fail(OPIR_ERR_UNKNOWN_DB, "unknown database %u", db_id);
  const size_t n1 = db->shape.fst_dim_sz, nr = db->shape.other_dim_sz;
  const size_t need = n1 * (size_t)kN * sizeof(uint4);
  if (need > kNoAllocScratchBytes)
    return ctx->fail(OPIR_ERR_ARG,
                     "first dimension %zu needs %zu bytes of scratch; the static scratch holds "
                     "%zu (first dimension <= %zu)",
                     n1, need, kNoAllocScratchBytes, kNoAllocScratchBytes / (kN * sizeof(uint4)));
  CK(cudaSetDevice(ctx->device), "set device");
  void *scratch = nullptr;
  CK(noalloc_scratch(ctx->device, &scratch), "cudaGetSymbolAddress(static scratch)");
  uint4 *qs = static_cast<uint4 *>(scratch);
  cudaStream_t s = ctx->stream;
  const size_t CTW = 2 * (size_t)kN;
  // the operand is fully rewritten before the scan reads it: nothing to clear
  launch_query_prep(d_fst_cts, n1 * CTW, qs, (size_t)kN * n1, (int)n1, 1, ctx->Mq.tab, s);
  launch_scan(db->dbs.as<uint64_t>(), qs, (size_t)kN * n1, d_out, nr * CTW, (int)n1, (int)nr, 1,
              ctx->C, ctx->Mq.tab.mu_lo, ctx->Mq.tab.mu_hi, ctx->status.as<uint32_t>(), s);
  launch_ntt(ctx->Mq.tab, d_out, nr * 2, true, s);
  ctx->launches += 3;
  CK(cudaGetLastError(), "first dimension launch");
  return OPIR_OK;
}
