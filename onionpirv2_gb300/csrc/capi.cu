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

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/onionpir_gpu.h"
#include "async.cuh"
#include "hostmath.h"
#include "kernels.h"
#include "rns.h"
#include "serve_core.h"
#include "tune_core.h"

using namespace opir;

namespace {

using u128 = unsigned __int128;
using hostmath::bitlen;
using hostmath::brv;
using hostmath::is_prime;
using hostmath::mulmod;
using hostmath::powmod;
using hostmath::shoup;

// smallest primitive 2N-th root of unity mod q
uint64_t minimal_root(uint64_t q) { return hostmath::minimal_root(q, 2 * kN); }

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
  void *d = nullptr;  // its device address (mapped), looked up once per allocation
  size_t bytes = 0;
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
  cudaError_t alloc(size_t n) {
    if (n <= bytes && p) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = d = nullptr;
    bytes = 0;
    cudaError_t e = cudaMallocHost(&p, n ? n : 16);
    if (e == cudaSuccess) {
      bytes = n;
      if (cudaHostGetDevicePointer(&d, p, 0) != cudaSuccess) {
        d = nullptr;
        cudaGetLastError();
      }
    }
    return e;
  }
};

struct ModTables {
  DevBuf fwd, inv;
  ModTab tab{};
  uint64_t psi = 0;
};

constexpr int kGraphKey = 15;  // words identifying a captured single-query graph

struct Db {
  opir_db_shape shape{};
  uint64_t num_pt = 0;
  int ndim = 1, u = 1, h = 0;
  DevBuf dbs;
  DevBuf dbl;              // bf16 limb plane of dbs for the tensor-core product (built on demand)
  bool dbl_valid = false;  // cleared whenever dbs changes
  // opir_autotune's choices: scan tile configuration (-1: the default) and
  // the engine per batch size (empty: the fixed crossovers)
  int scan_cfg = -1;
  tune::EngineTable engines;
  int tc_ring = -1;   // tensor kernel ring shape (kTcRing*), -1: the default
  int tc_limbs = -1;  // query limb width (kTcLimbs*), -1: the default per pass
  int tc_pair = -1;   // tensor kernel form: 0 one CTA per tile, 1 CTA pairs, -1: the default
  TreeForms forms;   // tuned launch form per tree-stage work count
  // the synchronous single-query pipeline as CUDA graphs: executables keyed
  // by everything their kernel parameters hold (client keys, buffers, tile
  // configuration); the least recently used one is updated in place on a miss
  struct Graph {
    uint64_t key[kGraphKey];
    cudaGraphExec_t exec = nullptr;
    uint64_t used = 0;
    uint64_t launches = 0;  // kernels in the graph
  };
  std::vector<Graph> graphs;
  uint64_t graph_clock = 0;
  Db() = default;
  Db(const Db &) = delete;
  Db &operator=(const Db &) = delete;
  ~Db() {
    for (auto &g : graphs)
      if (g.exec) cudaGraphExecDestroy(g.exec);
  }
};

struct Client {
  DevBuf galois;  // device copies (no key budget): keys, then their Shoup companions
  uint32_t levels = 0;
  DevBuf gsw;
  bool has_galois = false, has_gsw = false;
  // key budget: host copies; the device copy lives in a key-pool slot while
  // resident (serve::KeyLru decides which clients are)
  std::vector<uint64_t> h_galois, h_gsw;  // keys + companions; gsw rows in coefficient form
  int inflight = 0;                       // serving batches reading these keys
};

struct Workspace {
  // sized for (batch, shape); grown on demand
  DevBuf exp0, exp1, gsw, qs, ql, res, resp, packed, queries, ingest, coeffs;
  PinnedBuf h_in, h_out;
};

struct Err {
  int code;
};

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// Where one pipeline run enqueues its work.
struct PipeEnv {
  Workspace *W;
  cudaStream_t s;
  uint32_t *status;  // device status word (bounded-wait timeouts)
  bool timed;        // record the stage events
  bool keep_pins;    // leave the batch's clients pinned (serving: until the batch completes)
  bool graph = false;  // launches recorded into a CUDA graph
  bool fork = false;   // one query: RGSW reconstruction on the context's side stream
  // where the last kernel copies the status word (the host-mapped staging
  // buffer of a host-buffer call), else nullptr
  uint32_t *status_out = nullptr;
};

// ---- serving (continuous batching)
struct Ticket {
  uint32_t db = 0;
  uint64_t client = 0;
  std::vector<uint64_t> query, resp;
  std::vector<uint8_t> packed;
  int state = 0;  // 0 queued, 1 on the device, 2 done
  int rc = 0;
  double t_submit = 0, t_done = 0;
};
struct Serving;
struct Lane {
  Serving *owner = nullptr;
  cudaStream_t stream = nullptr;
  Workspace ws;
  DevBuf status;
  PinnedBuf h_status;
  cudaEvent_t done = nullptr;
  bool busy = false;
  std::atomic<bool> finished{false};  // set by the stream callback
  uint32_t db = 0;
  std::vector<serve::Pending> reqs;
  std::vector<uint64_t> clients;
};
struct Serving {
  bool active = false, stop = false;
  opir_serve_config cfg{};
  std::thread worker;
  // Wake-ups of the worker (submission, finished batch, stop): a counter
  // under its own mutex, which nobody holds across a CUDA call -- the stream
  // callback takes it, and a callback that blocked would stall its stream and
  // any device-wide synchronisation behind it.
  std::mutex wake_mu;
  std::condition_variable wake_cv;
  uint64_t wake_seq = 0;
  void wake() {
    {
      std::lock_guard<std::mutex> g(wake_mu);
      wake_seq++;
    }
    wake_cv.notify_all();
  }
  std::mutex mu;  // everything below; taken after opir_ctx::mu when both are held
  std::condition_variable done_cv;
  serve::BatchQueue queue;
  std::unordered_map<uint64_t, Ticket> tickets;
  uint64_t next_ticket = 1;
  std::vector<std::unique_ptr<Lane>> lanes;
  std::vector<double> lat_ms;
  uint64_t submitted = 0, completed = 0, failed = 0, batches = 0, batched_queries = 0;
  double t_first = 0, t_last = 0;
  ~Serving() {
    for (auto &L : lanes) {
      if (L->done) cudaEventDestroy(L->done);
      if (L->stream) cudaStreamDestroy(L->stream);
    }
  }
};

}  // namespace

struct opir_ctx {
  std::mutex mu;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  // a single query's RGSW reconstruction runs on `side`, beside its first
  // dimension, inside the captured graph (fork and join events)
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  bool fork_convert = true;  // OPIR_FORK=0: keep it on the query's stream
  opir_params prm{};
  Consts C{};
  ModTables Mq, Mp;
  uint64_t resp_bytes = 0;
  std::map<uint32_t, std::unique_ptr<Db>> dbs;
  uint32_t next_db = 1;
  std::map<uint64_t, std::unique_ptr<Client>> clients;
  Workspace ws;
  DevBuf status;  // device status word: bounded-wait timeouts (async.cuh)
  // first-dimension engine of batches (opir_set_batch_engine): AUTO takes the
  // tensor cores from tc_min_batch queries on, else the integer GEMM from
  // imad_min_batch (shapes the tensor engine does not take), else one scan
  // per query -- the crossovers measured on GB300 (bench.py --batch-sweep)
  int engine = OPIR_ENGINE_AUTO;
  int tc_min_batch = 4;
  int imad_min_batch = 32;
  uint64_t r64 = 0, r128 = 0;  // 2^64 and 2^128 mod q
  // key budget: client keys in a pool of fixed slots, least recently used out
  uint64_t key_budget = 0;
  size_t slot_words = 0;  // galois [kLogN][2][2][N] x 2 (keys, companions) + RGSW(sk) [2 l_key][2][N]
  DevBuf key_pool;
  serve::KeyLru lru;
  std::unique_ptr<Serving> serving;
  bool timing = false;
  bool graphs = true;  // single queries on the synchronous path replay a CUDA graph
  bool host_copies = false;  // host calls stage through device buffers (else mapped pinned memory)
  cudaEvent_t ev[8] = {};
  float stage_ms[6] = {};
  bool stage_valid = false;
  uint64_t launches = 0;
  void *noalloc_scratch = nullptr;  // device address of the static scratch (opir_first_dim_noalloc)
  // multi-modulus parameter sets (opir_ctx_create_rns): the entry points that
  // support them dispatch here, the others return OPIR_ERR_STATE
  std::unique_ptr<RnsServer> rns;
  uint32_t rns_count = 1;
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

// Entry points of a multi-modulus context (opir_ctx_create_rns) run on its
// RnsServer, under the context's lock and with its error message copied.
#define RNS_DISPATCH(call)                          \
  if (ctx && ctx->rns) {                            \
    std::lock_guard<std::mutex> g_(ctx->mu);        \
    cudaSetDevice(ctx->device);                     \
    const int rc_ = (call);                         \
    if (rc_ != OPIR_OK) ctx->err = ctx->rns->error(); \
    return rc_;                                     \
  }
#define RNS_UNSUPPORTED(what)                                                         \
  if (ctx && ctx->rns)                                                                \
    return ctx->fail(OPIR_ERR_STATE, "%s is not available for multi-modulus parameter sets", what);

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
int ensure_workspace(opir_ctx *ctx, const Db &db, int batch, Workspace &W) {
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

void record(opir_ctx *ctx, const PipeEnv &E, int i) {
  if (E.timed) cudaEventRecord(ctx->ev[i], E.s);
}

bool serving_active(const opir_ctx *ctx) { return ctx->serving && ctx->serving->active; }

bool imad_supported(int n1, int nr) { return nr % 32 == 0 && n1 % 16 == 0; }

// The first-dimension engine of a batch (OPIR_ENGINE_SCAN/IMAD/TENSOR): the
// explicit choice of opir_set_batch_engine, else the database's tuned table,
// else the fixed crossovers.
int engine_for(const opir_ctx *ctx, const Db &db, int batch) {
  const int n1 = (int)db.shape.fst_dim_sz, nr = (int)db.shape.other_dim_sz;
  const bool tc_ok = tc_scan_supported(n1, nr), imad_ok = imad_supported(n1, nr);
  if (batch < 2) return OPIR_ENGINE_SCAN;
  if (ctx->engine == OPIR_ENGINE_AUTO && db.engines.points) {
    const int e = tune::engine_at(db.engines, batch);
    if (e == OPIR_ENGINE_TENSOR && tc_ok) return e;
    if (e == OPIR_ENGINE_IMAD && imad_ok) return e;
    return OPIR_ENGINE_SCAN;
  }
  switch (ctx->engine) {
    case OPIR_ENGINE_TENSOR:
      return tc_ok ? OPIR_ENGINE_TENSOR : imad_ok ? OPIR_ENGINE_IMAD : OPIR_ENGINE_SCAN;
    case OPIR_ENGINE_IMAD:
      return imad_ok ? OPIR_ENGINE_IMAD : OPIR_ENGINE_SCAN;
    case OPIR_ENGINE_SCAN:
      return OPIR_ENGINE_SCAN;
    default:
      if (tc_ok && batch >= ctx->tc_min_batch) return OPIR_ENGINE_TENSOR;
      if (imad_ok && batch >= ctx->imad_min_batch) return OPIR_ENGINE_IMAD;
      return OPIR_ENGINE_SCAN;
  }
}

// Device key pointers of a client for a query on stream s.  With a key
// budget the client is made resident first (its keys copied into a pool
// slot on stream s, evicting the least recently used unpinned client) and
// pinned; the caller unpins.
int resolve_keys(opir_ctx *ctx, uint64_t id, const Db &db, cudaStream_t s, QueryDesc *d) {
  auto it = ctx->clients.find(id);
  if (it == ctx->clients.end() || !it->second->has_galois)
    return ctx->fail(OPIR_ERR_UNKNOWN_CLIENT, "no Galois keys for client %llu",
                     (unsigned long long)id);
  Client &cl = *it->second;
  if (cl.levels < (uint32_t)db.h)
    return ctx->fail(OPIR_ERR_ARG, "client %llu has %u Galois levels, database needs %d",
                     (unsigned long long)id, cl.levels, db.h);
  if (db.ndim > 1 && !cl.has_gsw)
    return ctx->fail(OPIR_ERR_UNKNOWN_CLIENT, "no RGSW key for client %llu", (unsigned long long)id);
  const size_t gwords = (size_t)cl.levels * 4 * kN;
  if (!ctx->key_budget) {
    d->galois = cl.galois.as<uint64_t>();
    d->galois_s = d->galois + gwords;
    d->gsw_key = cl.gsw.as<uint64_t>();
    return OPIR_OK;
  }
  uint64_t evicted;
  bool fresh;
  const int slot = ctx->lru.admit(id, &evicted, &fresh);
  if (slot < 0)
    return ctx->fail(OPIR_ERR_OOM, "key budget: all %d key slots are held by queries in flight",
                     ctx->lru.slots());
  uint64_t *base = ctx->key_pool.as<uint64_t>() + (size_t)slot * ctx->slot_words;
  uint64_t *gal = base, *gsw = base + (size_t)kLogN * 8 * kN;
  if (fresh) {
    // a slot is only reused once no queued work reads it: same-stream order
    // on the synchronous path, pins on the serving lanes
    CK(cudaMemcpyAsync(gal, cl.h_galois.data(), cl.h_galois.size() * 8, cudaMemcpyHostToDevice, s),
       "upload Galois keys");
    if (cl.has_gsw) {
      CK(cudaMemcpyAsync(gsw, cl.h_gsw.data(), cl.h_gsw.size() * 8, cudaMemcpyHostToDevice, s),
         "upload RGSW key");
      launch_ntt(ctx->Mq.tab, gsw, cl.h_gsw.size() / kN, false, s);  // server.cpp:497
      ctx->launches++;
    }
  }
  ctx->lru.pin(id);
  d->galois = gal;
  d->galois_s = gal + gwords;
  d->gsw_key = gsw;
  return OPIR_OK;
}

// First dimension (evaluate_first_dim, server.cpp:124-175) of `batch`
// queries' n1 leaves (coefficient form) into W.res[b][n_rest][2][N], in NTT
// form: one pass over the database per batch (batched GEMM on the tensor or
// integer engine) or per query (the streaming scan), as engine_for decides.
int enqueue_first_dim(opir_ctx *ctx, Db &db, Workspace &W, const uint64_t *leaves,
                      size_t leaves_stride, int batch, bool pdl_prep, const PipeEnv &E) {
  cudaStream_t s = E.s;
  const size_t CTW = 2 * (size_t)kN;
  const size_t n1 = db.shape.fst_dim_sz, nr = db.shape.other_dim_sz;
  const size_t qs_stride = (size_t)kN * n1;
  const size_t res_stride = nr * CTW;
  const int use = engine_for(ctx, db, batch);
  const bool tensor = use == OPIR_ENGINE_TENSOR, batched = use == OPIR_ENGINE_IMAD;
  if (tensor) {
    if (!db.dbl_valid) {
      CK(db.dbl.alloc(tc_db_limb_bytes((int)n1, (int)nr)), "alloc database limb plane");
      launch_db_limbs(db.dbs.as<uint64_t>(), db.dbl.as<uint16_t>(), (int)n1, (int)nr, s);
      ctx->launches++;
      // built once; batches on other streams read it afterwards
      CK(cudaStreamSynchronize(s), "database limb plane");
      db.dbl_valid = true;
    }
    CK(W.ql.alloc(tc_query_limb_bytes((int)n1, batch)), "alloc query limbs");
    launch_query_prep_plane(leaves, leaves_stride, W.qs.as<uint64_t>(), (int)n1, batch,
                            ctx->Mq.tab, s, pdl_prep);
    launch_tc_query_limbs(W.qs.as<uint64_t>(), W.ql.as<uint16_t>(), (int)n1, (int)nr, batch, s,
                          db.tc_limbs, db.tc_pair);
    ctx->launches += tc_pass_count(batch);
    record(ctx, E, 6);
    const int tl = launch_tc_scan(db.dbl.as<uint16_t>(), W.ql.as<uint16_t>(), W.res.as<uint64_t>(),
                                  res_stride, (int)n1, (int)nr, batch, ctx->Mq.tab.q,
                                  ctx->Mq.tab.mu_lo, ctx->Mq.tab.mu_hi, ctx->r64, ctx->r128,
                                  E.status, s, db.tc_ring, db.tc_limbs, db.tc_pair);
    if (tl < 0) return ctx->fail(OPIR_ERR_CUDA, "tensor kernel: tensor copy maps");
    ctx->launches += tl - 1;
  } else if (batched) {
    launch_query_prep_batched(leaves, leaves_stride, W.qs.as<uint4>(), (int)n1, batch,
                              ctx->Mq.tab, s, pdl_prep);
    record(ctx, E, 6);
    launch_scan_batched(db.dbs.as<uint64_t>(), W.qs.as<uint4>(), W.res.as<uint64_t>(), res_stride,
                        (int)n1, (int)nr, batch, ctx->C, ctx->Mq.tab.mu_lo, ctx->Mq.tab.mu_hi,
                        E.status, s);
  } else {
    launch_query_prep(leaves, leaves_stride, W.qs.as<uint4>(), qs_stride, (int)n1, batch,
                      ctx->Mq.tab, s, pdl_prep);
    record(ctx, E, 6);
    launch_scan(db.dbs.as<uint64_t>(), W.qs.as<uint4>(), qs_stride, W.res.as<uint64_t>(),
                res_stride, (int)n1, (int)nr, batch, ctx->C, ctx->Mq.tab.mu_lo,
                ctx->Mq.tab.mu_hi, E.status, s, db.scan_cfg);
  }
  return OPIR_OK;
}

// Enqueue the whole query pipeline for `batch` queries already on the device.
int run_pipeline(opir_ctx *ctx, Db &db, int batch, const uint64_t *client_ids,
                 const uint64_t *d_queries, uint64_t *d_resp, uint8_t *d_packed,
                 const Trace *trace, const PipeEnv &E) {
  if (batch <= 0) return ctx->fail(OPIR_ERR_ARG, "batch must be positive");
  if (!db.dbs.p) return ctx->fail(OPIR_ERR_STATE, "database has no data");
  std::vector<QueryDesc> desc(batch);
  for (int b = 0; b < batch; b++) {
    const int rc = resolve_keys(ctx, client_ids[b], db, E.s, &desc[b]);
    if (rc) {
      if (ctx->key_budget)
        for (int j = 0; j < b; j++) ctx->lru.unpin(client_ids[j]);
      return rc;
    }
  }
  // pins only guard a batch's own clients from each other while it is set
  // up, unless the caller keeps them until the batch completes
  struct Unpin {
    opir_ctx *ctx;
    const uint64_t *ids;
    int n;
    bool keep;
    ~Unpin() {
      if (ctx->key_budget && !keep)
        for (int j = 0; j < n; j++) ctx->lru.unpin(ids[j]);
    }
  } unpin{ctx, client_ids, batch, false};
  int rc = ensure_workspace(ctx, db, batch, *E.W);
  if (rc) return rc;
  Workspace &W = *E.W;
  cudaStream_t s = E.s;
  const QueryDesc *qd = desc.data();  // host array: launchers pass it by value
  const size_t CTW = 2 * (size_t)kN;  // words per ciphertext
  const int h = db.h, u = db.u;
  const size_t w = (size_t)1 << h;
  const size_t n1 = db.shape.fst_dim_sz, nr = db.shape.other_dim_sz;
  const int l = (int)ctx->prm.gsw_l;
  // Programmatic launches (a kernel stages its constant tables while its
  // predecessor runs) of the kinds g_pdl_* select, never across stage events
  // or trace copies; the first kernel follows host copies and launches
  // normally.
  const int pdl = E.timed || trace ? 0 : E.graph ? g_pdl_graph : g_pdl_direct;

  record(ctx, E, 0);
  // ---- expansion
  const uint64_t *cur = d_queries;
  size_t cur_stride = CTW;
  uint64_t *bufs[2] = {W.exp0.as<uint64_t>(), W.exp1.as<uint64_t>()};
  for (int a = 0; a < h; a++) {
    const int live = (int)((u + ((size_t)1 << (h - a)) - 1) >> (h - a));
    uint64_t *nxt = bufs[a & 1];
    launch_expand_level(cur, nxt, cur_stride, w * CTW, qd, a, live, batch, ctx->Mq.tab,
                        ctx->Mp.tab, ctx->C, s, (pdl & kPdlExpand) && a > 0, &db.forms);
    ctx->launches++;
    cur = nxt;
    cur_stride = w * CTW;
  }
  const uint64_t *leaves = cur;
  const size_t leaves_stride = cur_stride;
  record(ctx, E, 1);
  // ---- convert: for one query on its own stream, so that it runs beside
  // the first dimension's query transform; the folds wait for it
  const size_t gsw_stride = (size_t)(db.ndim > 1 ? db.ndim - 1 : 1) * 2 * l * CTW;
  const bool fork = E.fork && ctx->side && db.ndim > 1 && batch == 1 && !trace && !E.timed;
  if (fork) {
    CK(cudaEventRecord(ctx->fork_ev, s), "fork");
    CK(cudaStreamWaitEvent(ctx->side, ctx->fork_ev, 0), "fork");
  }
  if (db.ndim > 1) {
    launch_query_to_gsw(leaves, leaves_stride, W.gsw.as<uint64_t>(), gsw_stride, qd, (int)n1,
                        (db.ndim - 1) * l, batch, ctx->Mq.tab, ctx->C, fork ? ctx->side : s,
                        (pdl & kPdlQtg) && h > 0 && !fork, &db.forms);
    ctx->launches++;
  }
  if (fork) CK(cudaEventRecord(ctx->join_ev, ctx->side), "join");
  record(ctx, E, 2);
  // ---- first dimension
  const size_t res_stride = nr * CTW;
  const bool pdl_prep =
      (pdl & kPdlPrep) && (h > 0 || (db.ndim > 1 && !fork));  // a kernel precedes on s
  rc = enqueue_first_dim(ctx, db, W, leaves, leaves_stride, batch, pdl_prep, E);
  if (rc) return rc;
  record(ctx, E, 7);
  // the n_rest results stay in NTT form: the folds transform only their
  // differences back (evaluate_first_dim's inverse transforms, server.cpp:
  // 239, 290, move into other_dim_mux)
  ctx->launches += 2;
  record(ctx, E, 3);
  if (trace && trace->first_dim) {
    DevBuf fd;
    CK(fd.alloc(nr * CTW * 8), "trace first dim");
    CK(cudaMemcpyAsync(fd.p, W.res.p, nr * CTW * 8, cudaMemcpyDeviceToDevice, s), "trace first dim");
    launch_ntt(ctx->Mq.tab, fd.as<uint64_t>(), nr * 2, true, s);
    CK(cudaMemcpyAsync(trace->first_dim, fd.p, nr * CTW * 8, cudaMemcpyDeviceToHost, s),
       "trace first dim");
    CK(cudaStreamSynchronize(s), "trace first dim");
  }
  // ---- other dimensions
  if (fork) CK(cudaStreamWaitEvent(s, ctx->join_ev, 0), "join");
  size_t cnt = nr;
  for (int i = 1; i < db.ndim; i++) {
    const int half = (int)(cnt / 2);
    launch_fold(W.res.as<uint64_t>(), res_stride, W.gsw.as<uint64_t>() + (size_t)(i - 1) * 2 * l * CTW,
                gsw_stride, half, batch, ctx->Mq.tab, ctx->C, s,
                (pdl & kPdlFold) != 0 && !(fork && i == 1), &db.forms);
    ctx->launches++;
    cnt = half;
  }
  // the folded ciphertext of every query back to coefficient form
  launch_ntt_groups(ctx->Mq.tab, W.res.as<uint64_t>(), 2, batch, res_stride, true, s,
                    (pdl & kPdlNtt) != 0);
  ctx->launches++;
  record(ctx, E, 4);
  // ---- mod switch + pack
  launch_modswitch_pack(W.res.as<uint64_t>(), res_stride, d_resp, d_packed, ctx->resp_bytes, batch,
                        ctx->C, s, (pdl & kPdlModswitch) != 0, E.status, E.status_out);
  ctx->launches++;
  record(ctx, E, 5);
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
  if (E.W == &ctx->ws) ctx->stage_valid = E.timed;  // synchronous path
  unpin.keep = E.keep_pins;
  return OPIR_OK;
}

PipeEnv sync_env(opir_ctx *ctx) {
  return PipeEnv{&ctx->ws, ctx->stream, ctx->status.as<uint32_t>(), ctx->timing, false};
}

// The synchronous path.  One query (no trace, no stage timing, no key
// budget -- whose key upload copies from pageable host memory) runs its 24
// launches as a CUDA graph, which removes the gaps between the dependent
// launches (1.27 -> 1.21 ms per query on the 262,144-plaintext database).
// The database keeps up to kGraphs executables keyed by the values baked
// into their kernel parameters; a hit relaunches one as it is, a miss
// captures the pipeline and updates the least recently used executable in
// place (cudaGraphExecUpdate: the launch topology depends only on the
// database shape).  A capture that fails falls back to direct launches.
constexpr size_t kGraphs = 16;

int run_sync(opir_ctx *ctx, Db &db, int batch, const uint64_t *client_ids,
             const uint64_t *d_queries, uint64_t *d_resp, uint8_t *d_packed, const Trace *trace,
             uint32_t *d_status_out = nullptr) {
  PipeEnv E = sync_env(ctx);
  E.status_out = d_status_out;
  cudaStream_t s = E.s;
  bool capturable = s != nullptr && s != cudaStreamLegacy && s != cudaStreamPerThread;
  if (capturable) {
    // a caller capturing the stream into a graph of its own records the
    // launches themselves
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    capturable = cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone;
  }
  if (batch != 1 || trace || E.timed || !ctx->graphs || ctx->key_budget || !capturable)
    return run_pipeline(ctx, db, batch, client_ids, d_queries, d_resp, d_packed, trace, E);
  int rc = ensure_workspace(ctx, db, batch, *E.W);  // no allocation inside the capture
  if (rc) return rc;
  QueryDesc qd;
  rc = resolve_keys(ctx, client_ids[0], db, s, &qd);  // no budget: pointers only
  if (rc) return rc;
  const Workspace &W = *E.W;
  // every value a kernel parameter of the captured pipeline holds (the
  // context's tables and the database shape are fixed for its lifetime)
  const uint64_t key[kGraphKey] = {
      client_ids[0],      (uint64_t)qd.galois, (uint64_t)qd.galois_s, (uint64_t)qd.gsw_key,
      (uint64_t)d_queries, (uint64_t)d_resp,   (uint64_t)d_packed,    (uint64_t)W.exp0.p,
      (uint64_t)W.exp1.p,  (uint64_t)W.gsw.p,  (uint64_t)W.qs.p,      (uint64_t)W.res.p,
      (uint64_t)db.dbs.p,  (uint64_t)(int64_t)db.scan_cfg, (uint64_t)d_status_out};
  Db::Graph *hit = nullptr, *lru = nullptr;
  for (auto &g : db.graphs) {
    if (std::memcmp(g.key, key, sizeof key) == 0) hit = &g;
    if (!lru || g.used < lru->used) lru = &g;
  }
  if (hit) {
    hit->used = ++db.graph_clock;
    ctx->launches += hit->launches;
    CK(cudaGraphLaunch(hit->exec, s), "graph launch");
    return OPIR_OK;
  }
  const uint64_t launches0 = ctx->launches;
  CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin graph capture");
  PipeEnv Eg = E;
  Eg.graph = true;
  Eg.fork = ctx->side != nullptr && ctx->fork_convert;
  rc = run_pipeline(ctx, db, 1, client_ids, d_queries, d_resp, d_packed, nullptr, Eg);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(s, &g);
  // a launch the capture did not take also ends here: direct launches below
  // then report the error of the launch itself, if it persists
  bool ok = rc == OPIR_OK && ce == cudaSuccess && g != nullptr;
  Db::Graph *slot = nullptr;
  if (ok && db.graphs.size() < kGraphs) {
    db.graphs.push_back(Db::Graph{});
    slot = &db.graphs.back();
    ok = cudaGraphInstantiate(&slot->exec, g, 0) == cudaSuccess;
  } else if (ok) {
    slot = lru;
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(slot->exec, g, &info) != cudaSuccess) {
      cudaGetLastError();
      cudaGraphExecDestroy(slot->exec);
      slot->exec = nullptr;
      ok = cudaGraphInstantiate(&slot->exec, g, 0) == cudaSuccess;
    }
  }
  if (g) cudaGraphDestroy(g);
  if (!ok) {
    cudaGetLastError();
    for (auto &e : db.graphs)
      if (e.exec) cudaGraphExecDestroy(e.exec);
    db.graphs.clear();
    ctx->graphs = false;  // this stream or driver does not take captures: launch directly
    ctx->launches = launches0;
    return run_pipeline(ctx, db, batch, client_ids, d_queries, d_resp, d_packed, nullptr, E);
  }
  std::memcpy(slot->key, key, sizeof key);
  slot->used = ++db.graph_clock;
  slot->launches = ctx->launches - launches0;
  CK(cudaGraphLaunch(slot->exec, s), "graph launch");
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

// The tree-stage part of opir_autotune: for one query and for every batch
// size of the report up to one key chunk (64 queries), every expansion level,
// the RGSW reconstruction and every folding level of database db, each form
// the parameter set allows, on operands of valid residues (the database's)
// and synthetic keys reduced mod their modulus with correct companions.  The
// fastest form per (stage, work count) goes into `out`; the report lists
// every measurement.
template <class TimeIt>
int tune_tree_forms(opir_ctx *ctx, const Db &db, opir_tune_report &R, TreeForms &out,
                    TimeIt &time_it, const DevBuf &leaves_src, const DevBuf &res) {
  std::vector<int> batches{1};
  for (uint32_t i = 0; i < R.batch_points; i++)
    if (R.batch[i] <= (uint32_t)kMaxKeyBatch) batches.push_back((int)R.batch[i]);
  const int bmax = batches.back();
  const size_t CTW = 2 * (size_t)kN, w = (size_t)1 << db.h;
  const int n1 = (int)db.shape.fst_dim_sz, nr = (int)db.shape.other_dim_sz, l = ctx->C.l;
  const int num_cts = (db.ndim - 1) * l;
  const size_t gsw_stride = (size_t)(db.ndim > 1 ? db.ndim - 1 : 1) * 2 * l * CTW;
  cudaStream_t s = ctx->stream;
  // keys: one set for every query, [kLogN][k][q, p][N] then the companions
  const size_t gwords = (size_t)kLogN * 4 * kN;
  std::vector<uint64_t> hk(2 * gwords);
  uint64_t x = 0x9E3779B97F4A7C15ULL;
  for (size_t i = 0; i < gwords; i++) {
    x ^= x << 13, x ^= x >> 7, x ^= x << 17;
    const uint64_t mod = ((i / kN) & 1) ? ctx->Mp.tab.q : ctx->Mq.tab.q;
    hk[i] = x % mod;
    hk[gwords + i] = shoup(hk[i], mod);
  }
  DevBuf keys, gswk, exp0, exp1, gsw;
  CK(keys.alloc(hk.size() * 8), "autotune keys");
  CK(cudaMemcpyAsync(keys.p, hk.data(), hk.size() * 8, cudaMemcpyHostToDevice, s), "autotune keys");
  const size_t kwords = 2 * (size_t)ctx->prm.gsw_l_key * CTW;
  CK(gswk.alloc(kwords * 8), "autotune keys");
  CK(exp0.alloc((size_t)bmax * w * CTW * 8), "autotune expansion");
  CK(exp1.alloc((size_t)bmax * w * CTW * 8), "autotune expansion");
  CK(gsw.alloc((size_t)bmax * gsw_stride * 8), "autotune RGSW rows");
  // fill `words` words of dst with copies of the operand residues
  const size_t src_words = leaves_src.bytes / 8;
  auto fill = [&](uint64_t *dst, size_t words) -> cudaError_t {
    for (size_t off = 0; off < words; off += src_words) {
      const size_t n = std::min(src_words, words - off);
      const cudaError_t e =
          cudaMemcpyAsync(dst + off, leaves_src.p, n * 8, cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  };
  CK(fill(gswk.as<uint64_t>(), kwords), "autotune keys");
  CK(fill(exp0.as<uint64_t>(), (size_t)bmax * w * CTW), "autotune operands");
  CK(fill(gsw.as<uint64_t>(), (size_t)bmax * gsw_stride), "autotune operands");
  std::vector<QueryDesc> qd(bmax);
  for (auto &d : qd) {
    d.galois = keys.as<uint64_t>();
    d.galois_s = keys.as<uint64_t>() + gwords;
    d.gsw_key = gswk.as<uint64_t>();
  }
  CK(fill(exp1.as<uint64_t>(), (size_t)bmax * w * CTW), "autotune operands");
  // A level's form is timed where it runs: inside its stage's whole sequence
  // of launches (each level reading its predecessor's output, programmatic
  // launches as the pipeline makes them), replayed from a CUDA graph for one
  // query as the synchronous path does; timed alone and back to back, a form
  // can look faster than it is in the pipeline.  The other levels keep the
  // choices made so far.
  auto time_graph = [&](auto &&seq) -> float {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      return -1.0f;
    }
    seq();
    if (cudaStreamEndCapture(s, &g) != cudaSuccess || g == nullptr) {
      cudaGetLastError();
      return -1.0f;
    }
    float ms = -1.0f;
    if (cudaGraphInstantiate(&ge, g, 0) == cudaSuccess) {
      ms = time_it([&] { return cudaGraphLaunch(ge, s) == cudaSuccess; });
      cudaGraphExecDestroy(ge);
    }
    cudaGraphDestroy(g);
    cudaGetLastError();
    return ms;
  };
  R.form_points = 0;
  auto measure = [&](int stage, int count, int B, auto &&seq) {
    if (out.pick(stage, count) != kFormDefault) return;  // measured already
    if (R.form_points >= 128) return;
    float ms[kTreeForms];
    for (int f = 0; f < kTreeForms; f++) {
      if (!tree_form_valid(stage, f, ctx->C)) {
        ms[f] = -1.0f;
        continue;
      }
      TreeForms trial = out;
      trial.set(stage, count, f);
      ms[f] = B == 1 ? time_graph([&] { seq(trial); }) : time_it([&] {
        seq(trial);
        return true;
      });
    }
    // the stage's time moves by a level's difference only: a form replaces
    // the default when it saves more than the sequence's timing noise
    const int dflt = tree_default_form(stage, count, ctx->C);
    const int best = tune::pick_over(ms, kTreeForms, dflt, tune::kSeqMargin);
    out.set(stage, count, best);
    const uint32_t i = R.form_points++;
    R.form_stage[i] = (uint32_t)stage;
    R.form_count[i] = (uint32_t)count;
    for (int f = 0; f < kTreeForms; f++) R.form_ms[i][f] = ms[f];
    R.form_choice[i] = best;
  };
  uint64_t *ebuf[2] = {exp0.as<uint64_t>(), exp1.as<uint64_t>()};
  for (int B : batches) {
    const int pdl = B == 1 ? g_pdl_graph : g_pdl_direct;
    auto expand_seq = [&](const TreeForms &f) {
      for (int a = 0; a < db.h; a++) {
        const int live = (int)((db.u + ((size_t)1 << (db.h - a)) - 1) >> (db.h - a));
        launch_expand_level(ebuf[(a + 1) & 1], ebuf[a & 1], w * CTW, w * CTW, qd.data(), a, live, B,
                            ctx->Mq.tab, ctx->Mp.tab, ctx->C, s, (pdl & kPdlExpand) && a > 0, &f);
      }
    };
    for (int a = 0; a < db.h; a++) {
      const int live = (int)((db.u + ((size_t)1 << (db.h - a)) - 1) >> (db.h - a));
      measure(kStageExpand, live * B, B, expand_seq);
    }
    if (db.ndim > 1)
      measure(kStageQtg, num_cts * B, B, [&](const TreeForms &f) {
        launch_query_to_gsw(exp0.as<uint64_t>(), w * CTW, gsw.as<uint64_t>(), gsw_stride, qd.data(),
                            n1, num_cts, B, ctx->Mq.tab, ctx->C, s, false, &f);
      });
    auto fold_seq = [&](const TreeForms &f) {
      int i = 1;
      for (int half = nr / 2; half >= 1; half /= 2, i++)
        launch_fold(res.as<uint64_t>(), (size_t)nr * CTW, gsw.as<uint64_t>() + (size_t)(i - 1) * 2 * l * CTW,
                    gsw_stride, half, B, ctx->Mq.tab, ctx->C, s, (pdl & kPdlFold) != 0 && i > 1, &f);
    };
    for (int half = nr / 2; half >= 1; half /= 2) measure(kStageFold, half * B, B, fold_seq);
  }
  CK(cudaStreamSynchronize(s), "autotune tree stages");
  return OPIR_OK;
}

// make_query_batch on a multi-modulus context (queries [batch][2][R][N],
// resps [batch][2][N], packed [batch][bytes]): the queries spread over the
// path's concurrent lanes, each the single-query pipeline.
int rns_batch(opir_ctx *ctx, uint32_t db_id, uint32_t batch, const uint64_t *ids,
              const uint64_t *queries, uint64_t *resps, uint8_t *packed) {
  return ctx->rns->make_query_batch(db_id, batch, ids, queries, resps, packed, ctx->stream);
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

int opir_ctx_create_rns(const opir_rns_params *P, int device, opir_ctx **out) {
  if (!P || !out) return OPIR_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return OPIR_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return OPIR_ERR_ARG;
  std::unique_ptr<opir_ctx> ctx(new opir_ctx());
  ctx->device = device;
  // the first dimension runs on the one-modulus streaming scan, once per prime
  if (cudaSetDevice(device) != cudaSuccess || init_scan_attributes() != cudaSuccess)
    return OPIR_ERR_CUDA;
  std::string err;
  const int rc = RnsServer::create(*P, device, &ctx->rns, &err);
  if (rc) return rc;
  opir_params &prm = ctx->prm;  // the fields the shared entry points read
  prm.poly_degree = P->poly_degree;
  prm.coeff_modulus = P->coeff_moduli[0];
  prm.special_modulus = P->special_modulus;
  prm.plain_modulus = P->plain_modulus;
  prm.small_modulus = P->small_modulus;
  prm.gsw_l = P->gsw_l;
  prm.gsw_base_log2 = P->gsw_base_log2;
  prm.gsw_l_key = P->gsw_l_key;
  prm.gsw_base_log2_key = P->gsw_base_log2_key;
  ctx->rns_count = P->rns_count;
  ctx->resp_bytes = ctx->rns->response_bytes();
  ctx->graphs = false;
  if (ctx->status.alloc(kStatusWords * sizeof(uint32_t)) != cudaSuccess ||
      cudaMemset(ctx->status.p, 0, kStatusWords * sizeof(uint32_t)) != cudaSuccess)
    return OPIR_ERR_CUDA;
  if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return OPIR_ERR_CUDA;
  ctx->stream = ctx->own_stream;
  *out = ctx.release();
  return OPIR_OK;
}

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
  if (c->status.alloc(kStatusWords * sizeof(uint32_t)) != cudaSuccess ||
      cudaMemset(c->status.p, 0, kStatusWords * sizeof(uint32_t)) != cudaSuccess)
    return OPIR_ERR_CUDA;
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming) != cudaSuccess)
    return OPIR_ERR_CUDA;
  c->stream = c->own_stream;
  // test and sweep overrides of the engine choice
  if (const char *v = getenv("OPIR_TC")) c->engine = atoi(v) ? OPIR_ENGINE_TENSOR : OPIR_ENGINE_IMAD;
  if (const char *v = getenv("OPIR_GRAPHS")) c->graphs = atoi(v) != 0;
  if (const char *v = getenv("OPIR_FORK")) c->fork_convert = atoi(v) != 0;
  if (const char *v = getenv("OPIR_HOST_COPIES")) c->host_copies = atoi(v) != 0;
  if (const char *v = getenv("OPIR_BATCH_SCAN"))
    if (!atoi(v)) c->engine = OPIR_ENGINE_SCAN;
  if (const char *v = getenv("OPIR_TC_MIN_BATCH")) c->tc_min_batch = atoi(v);
  c->slot_words = (size_t)kLogN * 8 * kN + 2 * (size_t)P->gsw_l_key * 2 * kN;
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
  opir_serve_stop(ctx);
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto &e : ctx->ev)
    if (e) cudaEventDestroy(e);
  if (ctx->side) cudaStreamSynchronize(ctx->side);
  if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
  if (ctx->join_ev) cudaEventDestroy(ctx->join_ev);
  ctx->dbs.clear();
  ctx->clients.clear();
  cudaStream_t own = ctx->own_stream, side = ctx->side;
  delete ctx;
  if (own) cudaStreamDestroy(own);
  if (side) cudaStreamDestroy(side);
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
  RNS_DISPATCH(shape && db_id ? ctx->rns->db_create(*shape, db_id) : OPIR_ERR_ARG)
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
  RNS_DISPATCH(ctx->rns->db_destroy(db_id))
  if (!ctx) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (serving_active(ctx)) return ctx->fail(OPIR_ERR_STATE, "serving is active");
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (!ctx->dbs.erase(db_id)) return ctx->fail(OPIR_ERR_UNKNOWN_DB, "unknown database %u", db_id);
  return OPIR_OK;
}

int opir_db_push_chunk(opir_ctx *ctx, uint32_t db_id, const uint8_t *entries, uint64_t num_entries,
                       uint64_t chunk_idx) {
  RNS_UNSUPPORTED("push_database_chunk")
  if (!ctx || !entries) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (serving_active(ctx)) return ctx->fail(OPIR_ERR_STATE, "serving is active");
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
  RNS_DISPATCH(ctx->rns->db_fill_synthetic(db_id, seed, ctx->stream))
  if (!ctx) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (serving_active(ctx)) return ctx->fail(OPIR_ERR_STATE, "serving is active");
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
  RNS_DISPATCH(aligned ? ctx->rns->db_upload_aligned(db_id, aligned, ctx->stream) : OPIR_ERR_ARG)
  if (!ctx || !aligned) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (serving_active(ctx)) return ctx->fail(OPIR_ERR_STATE, "serving is active");
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

int opir_db_get_entry(opir_ctx *ctx, uint32_t db_id, uint64_t entry_index, uint8_t *entry) {
  RNS_UNSUPPORTED("direct_get_entry")
  if (!ctx || !entry) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  Db *db = find_db(ctx, db_id);
  if (!db) return ctx->fail(OPIR_ERR_UNKNOWN_DB, "unknown database %u", db_id);
  if (!db->dbs.p) return ctx->fail(OPIR_ERR_STATE, "database %u holds no data", db_id);
  const opir_db_shape &S = db->shape;
  if (entry_index >= db->num_pt * S.entries_per_pt)
    return ctx->fail(OPIR_ERR_ARG, "entry %llu out of range", (unsigned long long)entry_index);
  cudaSetDevice(ctx->device);
  DevBuf d_plain;
  CK(d_plain.alloc(kN * sizeof(uint64_t)), "alloc plaintext");
  launch_db_plaintext(db->dbs.as<uint64_t>(), (int)S.fst_dim_sz, (int)S.other_dim_sz,
                      (size_t)(entry_index / S.entries_per_pt), d_plain.as<uint64_t>(), ctx->Mq.tab,
                      ctx->C, ctx->stream);
  ctx->launches++;
  std::vector<uint64_t> plain(kN);
  CK(cudaMemcpyAsync(plain.data(), d_plain.p, kN * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                     ctx->stream),
     "read plaintext");
  CK(cudaStreamSynchronize(ctx->stream), "read plaintext");
  // the entry's bytes, LSB first from bits_per_coeff-bit coefficients
  // (push_database_chunk's packing, server.cpp:649-700, read back)
  const uint64_t bpc = S.bits_per_coeff;
  const uint64_t start = (entry_index % S.entries_per_pt) * (uint64_t)S.entry_size * 8;
  uint64_t ci = start / bpc, have = bpc - start % bpc;
  u128 buf = plain[ci] >> (start % bpc);
  for (uint32_t n = 0; n < S.entry_size;) {
    if (have >= 8) {
      entry[n++] = (uint8_t)(buf & 0xFF);
      buf >>= 8;
      have -= 8;
    } else {
      ci++;
      buf |= (u128)(ci < (uint64_t)kN ? plain[ci] : 0) << have;
      have += bpc;
    }
  }
  return OPIR_OK;
}

int opir_set_galois_key(opir_ctx *ctx, uint64_t client_id, const uint64_t *keys, uint32_t levels) {
  RNS_DISPATCH(keys ? ctx->rns->set_galois_key(client_id, keys, levels, ctx->stream) : OPIR_ERR_ARG)
  if (!ctx || !keys || !levels || levels > (uint32_t)kLogN) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  auto &cl = ctx->clients[client_id];
  if (!cl) cl = std::make_unique<Client>();
  if (cl->inflight)
    return ctx->fail(OPIR_ERR_STATE, "client %llu has queries in flight",
                     (unsigned long long)client_id);
  const size_t words = (size_t)levels * 4 * kN;
  // keys (reduced mod their modulus) followed by their Shoup companions
  // floor(k 2^64 / modulus): the expansion multiplies by them with two
  // multiplications instead of a 128-bit product and a Barrett reduction
  std::vector<uint64_t> kc(2 * words);
  for (size_t w = 0; w < words; w++) {
    const uint64_t mod = ((w / kN) & 1) ? ctx->Mp.tab.q : ctx->Mq.tab.q;  // [level][kk][q, p][N]
    kc[w] = keys[w] % mod;
    kc[words + w] = shoup(kc[w], mod);
  }
  if (ctx->key_budget) {
    // host copy; copied to a key slot when a query needs it
    cl->h_galois.swap(kc);
    ctx->lru.erase(client_id);
  } else {
    CK(cudaStreamSynchronize(ctx->stream), "sync");
    CK(cl->galois.alloc(2 * words * 8), "alloc Galois keys");
    CK(cudaMemcpy(cl->galois.p, kc.data(), 2 * words * 8, cudaMemcpyHostToDevice),
       "upload Galois keys");
  }
  cl->levels = levels;
  cl->has_galois = true;
  return OPIR_OK;
}

int opir_set_gsw_key(opir_ctx *ctx, uint64_t client_id, const uint64_t *rows) {
  RNS_DISPATCH(rows ? ctx->rns->set_gsw_key(client_id, rows, ctx->stream) : OPIR_ERR_ARG)
  if (!ctx || !rows) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  auto &cl = ctx->clients[client_id];
  if (!cl) cl = std::make_unique<Client>();
  if (cl->inflight)
    return ctx->fail(OPIR_ERR_STATE, "client %llu has queries in flight",
                     (unsigned long long)client_id);
  const size_t polys = 2 * (size_t)ctx->prm.gsw_l_key * 2;
  if (ctx->key_budget) {
    cl->h_gsw.assign(rows, rows + polys * kN);
    ctx->lru.erase(client_id);
  } else {
    CK(cudaStreamSynchronize(ctx->stream), "sync");
    CK(cl->gsw.alloc(polys * kN * 8), "alloc RGSW key");
    CK(cudaMemcpy(cl->gsw.p, rows, polys * kN * 8, cudaMemcpyHostToDevice), "upload RGSW key");
    launch_ntt(ctx->Mq.tab, cl->gsw.as<uint64_t>(), polys, false, ctx->stream);  // server.cpp:497
    ctx->launches++;
    CK(cudaGetLastError(), "key NTT");
    CK(cudaStreamSynchronize(ctx->stream), "key NTT");
  }
  cl->has_gsw = true;
  return OPIR_OK;
}

int opir_erase_client(opir_ctx *ctx, uint64_t client_id) {
  RNS_DISPATCH(ctx->rns->erase_client(client_id))
  if (!ctx) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  auto it = ctx->clients.find(client_id);
  if (it == ctx->clients.end())
    return ctx->fail(OPIR_ERR_UNKNOWN_CLIENT, "unknown client %llu", (unsigned long long)client_id);
  if (it->second->inflight)
    return ctx->fail(OPIR_ERR_STATE, "client %llu has queries in flight",
                     (unsigned long long)client_id);
  cudaStreamSynchronize(ctx->stream);
  ctx->lru.erase(client_id);
  ctx->clients.erase(it);
  return OPIR_OK;
}

int opir_set_key_budget(opir_ctx *ctx, uint64_t bytes) {
  RNS_UNSUPPORTED("a key budget")
  if (!ctx) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (!ctx->clients.empty() || serving_active(ctx))
    return ctx->fail(OPIR_ERR_STATE, "set the key budget before registering clients");
  cudaSetDevice(ctx->device);
  const size_t slot_bytes = ctx->slot_words * 8;
  const uint64_t slots = bytes / slot_bytes;
  if (bytes && !slots)
    return ctx->fail(OPIR_ERR_ARG, "key budget below one client's keys (%zu bytes)", slot_bytes);
  if (slots > (1u << 20)) return ctx->fail(OPIR_ERR_ARG, "key budget too large");
  ctx->key_pool.release();
  if (slots) CK(ctx->key_pool.alloc(slots * slot_bytes), "alloc key pool");
  ctx->key_budget = bytes;
  ctx->lru.reset((int)slots);
  return OPIR_OK;
}

uint64_t opir_key_bytes_per_client(const opir_ctx *ctx) { return ctx ? ctx->slot_words * 8 : 0; }

int opir_resident_clients(opir_ctx *ctx, uint32_t *resident, uint32_t *slots) {
  RNS_UNSUPPORTED("a key budget")
  if (!ctx || !resident || !slots) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  *resident = ctx->key_budget ? (uint32_t)ctx->lru.used() : (uint32_t)ctx->clients.size();
  *slots = ctx->key_budget ? (uint32_t)ctx->lru.slots() : 0;
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
  // responses, packed bytes, then (16-byte aligned) the device status word
  const size_t status_off = (batch * (CTB + ctx->resp_bytes) + 15) / 16 * 16;
  CK(W.h_out.alloc(status_off + 16), "alloc pinned");
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  std::memcpy(W.h_in.p, queries, batch * CTB);
  uint8_t *h_resp = static_cast<uint8_t *>(W.h_out.p);
  uint8_t *h_packed = h_resp + batch * CTB;
  // The staging buffers are mapped pinned memory: the first expansion level
  // reads the queries and the mod-switch kernel writes the responses across
  // the host link themselves, which saves the copy engine's three round trips
  // (set OPIR_HOST_COPIES=1 for copies through device buffers).
  uint64_t *d_in = static_cast<uint64_t *>(W.h_in.d);
  uint8_t *d_out = static_cast<uint8_t *>(W.h_out.d);
  const bool mapped = !ctx->host_copies && d_in && d_out;
  int rc;
  // the status word travels with the responses: one synchronisation per
  // call; the last kernel copies it into the mapped buffer itself
  uint32_t *h_status = reinterpret_cast<uint32_t *>(h_resp + status_off);
  if (mapped) {
    rc = run_sync(ctx, *db, (int)batch, client_ids, d_in, reinterpret_cast<uint64_t *>(d_out),
                  d_out + batch * CTB, trace, reinterpret_cast<uint32_t *>(d_out + status_off));
  } else {
    CK(cudaMemcpyAsync(W.queries.p, W.h_in.p, batch * CTB, cudaMemcpyHostToDevice, ctx->stream),
       "upload queries");
    rc = run_sync(ctx, *db, (int)batch, client_ids, W.queries.as<uint64_t>(),
                  W.resp.as<uint64_t>(), W.packed.as<uint8_t>(), trace);
  }
  if (rc) return rc;
  if (resps && !mapped)
    CK(cudaMemcpyAsync(h_resp, W.resp.p, batch * CTB, cudaMemcpyDeviceToHost, ctx->stream),
       "download responses");
  if (packed && !mapped)
    CK(cudaMemcpyAsync(h_packed, W.packed.p, batch * ctx->resp_bytes, cudaMemcpyDeviceToHost,
                       ctx->stream),
       "download responses");
  if (!mapped)
    CK(cudaMemcpyAsync(h_status, ctx->status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                       ctx->stream),
       "read status");
  CK(cudaStreamSynchronize(ctx->stream), "query");
  if (*h_status) {
    const uint32_t st = *h_status;
    CK(cudaMemset(ctx->status.p, 0, sizeof(uint32_t)), "clear status");
    return ctx->fail(OPIR_ERR_TIMEOUT, "device pipeline wait timed out (status 0x%x)", st);
  }
  if (resps) std::memcpy(resps, h_resp, batch * CTB);
  if (packed) std::memcpy(packed, h_packed, batch * ctx->resp_bytes);
  return collect_times(ctx);
}

// While serving runs, the synchronous query calls become tickets of the
// serving lanes (continuous batching) that the call waits for: the same
// responses, and the caller need not know whether serving is on.  Returns
// OPIR_ERR_STATE when serving stopped before every query was submitted (the
// tickets already out are waited for and dropped), so that the caller can
// answer the whole call synchronously instead.
static constexpr uint32_t kSyncServeWaitMs = 600000;
static int query_via_serving(opir_ctx *ctx, uint32_t db_id, uint32_t batch, const uint64_t *client_ids,
                      const uint64_t *queries, uint64_t *resps, uint8_t *packed) {
  std::vector<uint64_t> tickets(batch);
  for (uint32_t i = 0; i < batch; i++) {
    const int rc = opir_submit(ctx, db_id, client_ids[i], queries + (size_t)i * 2 * kN, &tickets[i]);
    if (rc) {
      // leave no ticket of this call behind
      for (uint32_t j = 0; j < i; j++) opir_wait(ctx, tickets[j], kSyncServeWaitMs, nullptr, nullptr);
      return rc;
    }
  }
  int first = OPIR_OK;
  for (uint32_t i = 0; i < batch; i++) {
    const int rc = opir_wait(ctx, tickets[i], kSyncServeWaitMs,
                             resps ? resps + (size_t)i * 2 * kN : nullptr,
                             packed ? packed + (size_t)i * ctx->resp_bytes : nullptr);
    if (rc && !first) first = rc;
  }
  return first;
}

static int query_sync_or_served(opir_ctx *ctx, uint32_t db_id, uint32_t batch,
                         const uint64_t *client_ids, const uint64_t *queries, uint64_t *resps,
                         uint8_t *packed) {
  {
    std::lock_guard<std::mutex> g(ctx->mu);
    if (!serving_active(ctx))
      return query_host(ctx, db_id, batch, client_ids, queries, resps, packed, nullptr);
  }
  const int rc = query_via_serving(ctx, db_id, batch, client_ids, queries, resps, packed);
  if (rc != OPIR_ERR_STATE) return rc;
  std::lock_guard<std::mutex> g(ctx->mu);  // serving stopped meanwhile
  if (serving_active(ctx)) return rc;
  return query_host(ctx, db_id, batch, client_ids, queries, resps, packed, nullptr);
}

int opir_make_query(opir_ctx *ctx, uint32_t db_id, uint64_t client_id, const uint64_t *query,
                    uint64_t *resp, uint8_t *packed) {
  RNS_DISPATCH(query ? ctx->rns->make_query(db_id, client_id, query, resp, packed, nullptr, ctx->stream) : OPIR_ERR_ARG)
  if (!ctx || !query) return OPIR_ERR_ARG;
  return query_sync_or_served(ctx, db_id, 1, &client_id, query, resp, packed);
}

int opir_make_query_batch(opir_ctx *ctx, uint32_t db_id, uint32_t batch, const uint64_t *client_ids,
                          const uint64_t *queries, uint64_t *resps, uint8_t *packed) {
  RNS_DISPATCH(queries && client_ids && batch ? rns_batch(ctx, db_id, batch, client_ids, queries, resps, packed) : OPIR_ERR_ARG)
  if (!ctx || !queries || !client_ids || !batch) return OPIR_ERR_ARG;
  return query_sync_or_served(ctx, db_id, batch, client_ids, queries, resps, packed);
}

int opir_make_query_device(opir_ctx *ctx, uint32_t db_id, uint32_t batch, const uint64_t *client_ids,
                           const uint64_t *d_queries, uint64_t *d_resps, uint8_t *d_packed) {
  RNS_UNSUPPORTED("make_query on device buffers")
  if (!ctx || !d_queries || !client_ids || !batch) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (serving_active(ctx))
    return ctx->fail(OPIR_ERR_STATE, "serving is active: submit queries with opir_submit");
  Db *db = find_db(ctx, db_id);
  if (!db) return ctx->fail(OPIR_ERR_UNKNOWN_DB, "unknown database %u", db_id);
  cudaSetDevice(ctx->device);
  return run_sync(ctx, *db, (int)batch, client_ids, d_queries, d_resps, d_packed, nullptr);
}

int opir_make_query_trace(opir_ctx *ctx, uint32_t db_id, uint64_t client_id, const uint64_t *query,
                          uint64_t *leaves, uint64_t *gsw, uint64_t *first_dim, uint64_t *resp,
                          uint8_t *packed) {
  if (ctx && ctx->rns) {
    RnsTrace t;
    t.leaves = leaves;
    t.gsw = gsw;
    t.first_dim = first_dim;
    RNS_DISPATCH(query ? ctx->rns->make_query(db_id, client_id, query, resp, packed, &t, ctx->stream) : OPIR_ERR_ARG)
  }
  if (!ctx || !query) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (serving_active(ctx))
    return ctx->fail(OPIR_ERR_STATE, "serving is active: submit queries with opir_submit");
  Trace t;
  t.leaves = leaves;
  t.gsw = gsw;
  t.first_dim = first_dim;
  return query_host(ctx, db_id, 1, &client_id, query, resp, packed, &t);
}

int opir_set_batch_engine(opir_ctx *ctx, int engine, uint32_t tensor_min_batch) {
  RNS_UNSUPPORTED("the batch engines")
  if (!ctx || engine < OPIR_ENGINE_AUTO || engine > OPIR_ENGINE_TENSOR) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (serving_active(ctx)) return ctx->fail(OPIR_ERR_STATE, "serving is active");
  ctx->engine = engine;
  if (tensor_min_batch) ctx->tc_min_batch = (int)tensor_min_batch;
  return OPIR_OK;
}

int opir_autotune(opir_ctx *ctx, uint32_t db_id, uint32_t max_batch, uint32_t reps,
                  opir_tune_report *report) {
  RNS_UNSUPPORTED("the autotuner")
  if (!ctx) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (serving_active(ctx)) return ctx->fail(OPIR_ERR_STATE, "serving is active");
  Db *db = find_db(ctx, db_id);
  if (!db) return ctx->fail(OPIR_ERR_UNKNOWN_DB, "unknown database %u", db_id);
  if (!db->dbs.p) return ctx->fail(OPIR_ERR_STATE, "database %u holds no data", db_id);
  CK(cudaSetDevice(ctx->device), "set device");
  if (reps == 0) reps = 3;
  if (max_batch > 256) max_batch = 256;
  opir_tune_report R{};
  const int n1 = (int)db->shape.fst_dim_sz, nr = (int)db->shape.other_dim_sz;
  const size_t CTW = 2 * (size_t)kN, res_stride = (size_t)nr * CTW, qs_stride = (size_t)kN * n1;
  const int np = tune::batch_points(max_batch, R.batch);
  const int bmax = np ? (int)R.batch[np - 1] : 1;
  cudaStream_t s = ctx->stream;
  uint32_t *status = ctx->status.as<uint32_t>();
  // operands: bmax queries' n1 first-dimension leaves, copied from the
  // database itself (valid residues mod q whatever q is) -- the work and the
  // memory traffic of every kernel are independent of the values
  DevBuf leaves, qs, ql, res;
  const size_t leaf_words = (size_t)bmax * n1 * CTW, db_words = db->num_pt * (size_t)kN;
  CK(leaves.alloc(leaf_words * 8), "autotune operands");
  for (size_t off = 0; off < leaf_words; off += db_words) {
    const size_t n = std::min(db_words, leaf_words - off);
    CK(cudaMemcpyAsync(leaves.as<uint64_t>() + off, db->dbs.p, n * 8, cudaMemcpyDeviceToDevice, s),
       "autotune operands");
  }
  CK(qs.alloc((size_t)bmax * kN * n1 * sizeof(uint4)), "autotune operands");
  CK(res.alloc((size_t)bmax * res_stride * 8), "autotune output");
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0), "autotune events");
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return ctx->fail(OPIR_ERR_CUDA, "autotune events");
  }
  // ms of one call of fn after one warm-up call; -1 if fn cannot run the shape
  auto time_it = [&](auto &&fn) -> float {
    if (!fn()) return -1.0f;
    cudaEventRecord(e0, s);
    for (uint32_t r = 0; r < reps; r++) fn();
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) != cudaSuccess) return -1.0f;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    return ms / (float)reps;
  };
  // ---- single-query scan: every compiled tile configuration
  R.scan_configs = (uint32_t)std::min(scan_config_count(), 16);
  for (uint32_t c = 0; c < R.scan_configs; c++) {
    scan_config_desc((int)c, R.scan_desc[c]);
    R.scan_ms[c] = time_it([&] {
      launch_query_prep(leaves.as<uint64_t>(), n1 * CTW, qs.as<uint4>(), qs_stride, n1, 1,
                        ctx->Mq.tab, s);
      return launch_scan(db->dbs.as<uint64_t>(), qs.as<uint4>(), qs_stride, res.as<uint64_t>(),
                         res_stride, n1, nr, 1, ctx->C, ctx->Mq.tab.mu_lo, ctx->Mq.tab.mu_hi,
                         status, s, (int)c) == (int)c;
    });
  }
  R.scan_choice = tune::pick(R.scan_ms, (int)R.scan_configs);
  // ---- batches: one scan per query, integer GEMM, tensor-core limb GEMM
  const bool tc_ok = tc_scan_supported(n1, nr), imad_ok = imad_supported(n1, nr);
  bool limbs = db->dbl_valid;
  if (tc_ok && np && !limbs) {
    // an allocation failure (the plane takes 16 bytes per residue) leaves
    // the tensor engine out of the table
    if (db->dbl.alloc(tc_db_limb_bytes(n1, nr)) == cudaSuccess) {
      launch_db_limbs(db->dbs.as<uint64_t>(), db->dbl.as<uint16_t>(), n1, nr, s);
      ctx->launches++;
      limbs = db->dbl_valid = cudaStreamSynchronize(s) == cudaSuccess;
    } else {
      cudaGetLastError();
    }
  }
  if (tc_ok && limbs && np && ql.alloc(tc_query_limb_bytes(n1, bmax)) != cudaSuccess) {
    cudaGetLastError();
    limbs = false;
  }
  R.batch_points = (uint32_t)np;
  for (int i = 0; i < np; i++) {
    const int B = (int)R.batch[i];
    R.engine_ms[i][OPIR_ENGINE_SCAN - 1] = time_it([&] {
      launch_query_prep(leaves.as<uint64_t>(), n1 * CTW, qs.as<uint4>(), qs_stride, n1, B,
                        ctx->Mq.tab, s);
      launch_scan(db->dbs.as<uint64_t>(), qs.as<uint4>(), qs_stride, res.as<uint64_t>(),
                  res_stride, n1, nr, B, ctx->C, ctx->Mq.tab.mu_lo, ctx->Mq.tab.mu_hi, status, s,
                  R.scan_choice);
      return true;
    });
    R.engine_ms[i][OPIR_ENGINE_IMAD - 1] = !imad_ok ? -1.0f : time_it([&] {
      launch_query_prep_batched(leaves.as<uint64_t>(), n1 * CTW, qs.as<uint4>(), n1, B,
                                ctx->Mq.tab, s);
      return launch_scan_batched(db->dbs.as<uint64_t>(), qs.as<uint4>(), res.as<uint64_t>(),
                                 res_stride, n1, nr, B, ctx->C, ctx->Mq.tab.mu_lo,
                                 ctx->Mq.tab.mu_hi, status, s);
    });
    R.engine_ms[i][OPIR_ENGINE_TENSOR - 1] = !(tc_ok && limbs) ? -1.0f : time_it([&] {
      launch_query_prep_plane(leaves.as<uint64_t>(), n1 * CTW, qs.as<uint64_t>(), n1, B,
                              ctx->Mq.tab, s);
      launch_tc_query_limbs(qs.as<uint64_t>(), ql.as<uint16_t>(), n1, nr, B, s);
      return launch_tc_scan(db->dbl.as<uint16_t>(), ql.as<uint16_t>(), res.as<uint64_t>(), res_stride, n1,
                     nr, B, ctx->Mq.tab.q, ctx->Mq.tab.mu_lo, ctx->Mq.tab.mu_hi, ctx->r64,
                     ctx->r128, status, s) >= 0;
    });
  }
  // ---- tensor kernel: both shared-memory rings at the largest batch
  R.tc_ring_choice = -1;
  const uint32_t ring_desc[2][2] = {{64, 4}, {32, 8}};
  std::memcpy(R.tc_ring_desc, ring_desc, sizeof ring_desc);
  for (int ring = 0; ring < 2; ring++) {
    R.tc_ring_ms[ring] = !(tc_ok && limbs && np && tc_ring_valid(ring, n1)) ? -1.0f : time_it([&] {
      return launch_tc_scan(db->dbl.as<uint16_t>(), ql.as<uint16_t>(), res.as<uint64_t>(), res_stride, n1,
                     nr, bmax, ctx->Mq.tab.q, ctx->Mq.tab.mu_lo, ctx->Mq.tab.mu_hi, ctx->r64,
                     ctx->r128, status, s, ring) >= 0;
    });
  }
  if (R.tc_ring_ms[0] >= 0 || R.tc_ring_ms[1] >= 0)
    R.tc_ring_choice = tune::pick_over(R.tc_ring_ms, 2, n1 % 64 == 0 ? kTcRing64x4 : kTcRing32x8,
                                       tune::kTuneMargin);
  // ---- tensor kernel: both query limb widths (limb split and product) at the
  // largest batch size, on the chosen ring
  R.tc_limbs_choice = -1;
  for (int lw = 0; lw < 2; lw++) {
    R.tc_limbs_ms[lw] = !(tc_ok && limbs && np) ? -1.0f : time_it([&] {
      launch_tc_query_limbs(qs.as<uint64_t>(), ql.as<uint16_t>(), n1, nr, bmax, s, lw);
      return launch_tc_scan(db->dbl.as<uint16_t>(), ql.as<uint16_t>(), res.as<uint64_t>(), res_stride, n1,
                     nr, bmax, ctx->Mq.tab.q, ctx->Mq.tab.mu_lo, ctx->Mq.tab.mu_hi, ctx->r64,
                     ctx->r128, status, s, R.tc_ring_choice, lw) >= 0;
    });
  }
  if (R.tc_limbs_ms[0] >= 0 && R.tc_limbs_ms[1] >= 0)
    R.tc_limbs_choice = tune::pick_over(
        R.tc_limbs_ms, 2, tc_query_limb_width(bmax, -1) == 9 ? kTcLimbs9 : kTcLimbs8,
        tune::kTuneMargin);
  // ---- tensor kernel: one CTA per tile or CTA pairs (cta_group::2), with
  // the chosen ring and limbs
  R.tc_pair_choice = -1;
  for (int pr = 0; pr < 2; pr++) {
    const bool applies = tc_ok && limbs && np &&
                         (pr == 0 || tc_pair_form(nr, bmax, R.tc_limbs_choice, 1));
    R.tc_pair_ms[pr] = !applies ? -1.0f : time_it([&] {
      launch_tc_query_limbs(qs.as<uint64_t>(), ql.as<uint16_t>(), n1, nr, bmax, s,
                            R.tc_limbs_choice, pr);
      return launch_tc_scan(db->dbl.as<uint16_t>(), ql.as<uint16_t>(), res.as<uint64_t>(), res_stride, n1,
                     nr, bmax, ctx->Mq.tab.q, ctx->Mq.tab.mu_lo, ctx->Mq.tab.mu_hi, ctx->r64,
                     ctx->r128, status, s, R.tc_ring_choice, R.tc_limbs_choice, pr) >= 0;
    });
  }
  if (R.tc_pair_ms[0] >= 0 && R.tc_pair_ms[1] >= 0)
    R.tc_pair_choice = tune::pick_over(R.tc_pair_ms, 2, 0, tune::kTuneMargin);
  else if (R.tc_pair_ms[0] >= 0)
    R.tc_pair_choice = 0;
  // ---- tree stages: every form of every distinct launch of this database's
  // pipeline, at one query and at the batch sizes up to one key chunk
  TreeForms tuned;
  {
    const int trc = tune_tree_forms(ctx, *db, R, tuned, time_it, leaves, res);
    if (trc) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return trc;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CK(cudaGetLastError(), "autotune launches");
  CK(cudaStreamSynchronize(s), "autotune");
  int rc = check_status(ctx);
  if (rc) return rc;
  db->scan_cfg = R.scan_choice;
  db->tc_ring = R.tc_ring_choice;
  db->tc_limbs = R.tc_limbs_choice;
  db->tc_pair = R.tc_pair_choice;
  db->forms = tuned;
  // captured single-query graphs hold the launch forms of their capture
  for (auto &gr : db->graphs)
    if (gr.exec) cudaGraphExecDestroy(gr.exec);
  db->graphs.clear();
  tune::build_table(db->engines, R.batch, np, R.engine_ms);
  for (int i = 0; i < np; i++) R.engine[i] = db->engines.engine[i];
  if (report) *report = R;
  return OPIR_OK;
}

int opir_set_graphs(opir_ctx *ctx, int enable) {
  if (!ctx) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  ctx->graphs = enable != 0;
  if (ctx->rns) ctx->rns->set_graphs(enable != 0);
  return OPIR_OK;
}

int opir_set_timing(opir_ctx *ctx, int enable) {
  if (!ctx) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (ctx->rns) ctx->rns->set_timing(enable != 0);
  ctx->timing = enable != 0;
  ctx->stage_valid = false;
  return OPIR_OK;
}

int opir_stage_times(opir_ctx *ctx, float *ms6) {
  if (!ctx || !ms6) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (ctx->rns)
    return ctx->rns->stage_times(ms6) ? OPIR_OK : ctx->fail(OPIR_ERR_STATE, "no timed query");
  if (!ctx->timing || !ctx->stage_valid) return ctx->fail(OPIR_ERR_STATE, "no timed query");
  int rc = collect_times(ctx);
  if (rc) return rc;
  std::memcpy(ms6, ctx->stage_ms, sizeof ctx->stage_ms);
  return OPIR_OK;
}

uint64_t opir_launch_count(const opir_ctx *ctx) {
  return ctx ? ctx->launches + (ctx->rns ? ctx->rns->launches() : 0) : 0;
}

int opir_sync(opir_ctx *ctx) {
  if (!ctx) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  return check_status(ctx);
}

int opir_ntt(opir_ctx *ctx, int mod, int inverse, uint64_t *polys, uint64_t count) {
  RNS_DISPATCH(polys ? ctx->rns->ntt(mod, inverse != 0, polys, count, ctx->stream) : OPIR_ERR_ARG)
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
  RNS_UNSUPPORTED("opir_ntt_device")
  if (!ctx || !d_polys || (mod != 0 && mod != 1)) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  launch_ntt(mod ? ctx->Mp.tab : ctx->Mq.tab, d_polys, count, inverse != 0, ctx->stream);
  ctx->launches++;
  CK(cudaGetLastError(), "ntt launch");
  return OPIR_OK;
}

// Test hook of the bounded-wait failure path (async.cuh): the single-query
// scans of this context's synchronous calls withhold one pipeline stage in
// their first CTA and give up waiting for it after `polls` polls (0: off).
int opir_debug_withhold_scan_stage(opir_ctx *ctx, uint32_t polls) {
  RNS_UNSUPPORTED("the scan test hook")
  if (!ctx) return OPIR_ERR_ARG;
  if (polls > (1u << 20))
    return ctx->fail(OPIR_ERR_ARG, "at most 2^20 polls (the production limit is 2^22)");
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  CK(cudaMemcpy(ctx->status.as<uint32_t>() + 1, &polls, sizeof polls, cudaMemcpyHostToDevice),
     "set scan test hook");
  return OPIR_OK;
}

// Test hook: the first dimension of `batch` queries whose n1 leaves the
// caller gives directly (leaves[b][n1][2][N], coefficient form), on the
// engine this batch size uses; out[b][n_rest][2][N] in coefficient form, as
// make_query_trace's first_dim.  Tests drive the products with operands that
// no query expansion produces: the limb-range extremes of the tensor engine.
int opir_debug_first_dim(opir_ctx *ctx, uint32_t db_id, uint32_t batch, const uint64_t *leaves,
                         uint64_t *out) {
  RNS_UNSUPPORTED("the first-dimension test hook")
  if (!ctx || !leaves || !out || !batch) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (serving_active(ctx)) return ctx->fail(OPIR_ERR_STATE, "serving is active");
  Db *db = find_db(ctx, db_id);
  if (!db) return ctx->fail(OPIR_ERR_UNKNOWN_DB, "unknown database %u", db_id);
  if (!db->dbs.p) return ctx->fail(OPIR_ERR_STATE, "database has no data");
  cudaSetDevice(ctx->device);
  const size_t CTW = 2 * (size_t)kN;
  const size_t n1 = db->shape.fst_dim_sz, nr = db->shape.other_dim_sz;
  cudaStream_t s = ctx->stream;
  Workspace &W = ctx->ws;
  int rc = ensure_workspace(ctx, *db, (int)batch, W);
  if (rc) return rc;
  DevBuf dl;
  CK(dl.alloc(batch * n1 * CTW * 8), "alloc leaves");
  CK(cudaMemcpyAsync(dl.p, leaves, batch * n1 * CTW * 8, cudaMemcpyHostToDevice, s),
     "upload leaves");
  const PipeEnv E{&W, s, ctx->status.as<uint32_t>(), false, false};
  rc = enqueue_first_dim(ctx, *db, W, dl.as<uint64_t>(), n1 * CTW, (int)batch, false, E);
  if (rc) return rc;
  launch_ntt_groups(ctx->Mq.tab, W.res.as<uint64_t>(), (int)(nr * 2), (int)batch, nr * CTW,
                    true, s, false);
  ctx->launches++;
  CK(cudaGetLastError(), "first dimension launches");
  CK(cudaMemcpyAsync(out, W.res.p, batch * nr * CTW * 8, cudaMemcpyDeviceToHost, s),
     "download first dimension");
  CK(cudaStreamSynchronize(s), "first dimension");
  return check_status(ctx);
}

// save_resp_to_stream (server.cpp:581-633) for responses the caller holds:
// the bit packing of the pipeline's last kernel without its modulus switch.
int opir_pack_response(opir_ctx *ctx, const uint64_t *resps, uint32_t count, uint8_t *packed) {
  RNS_DISPATCH(resps && packed && count ? ctx->rns->pack_response(resps, count, packed, ctx->stream) : OPIR_ERR_ARG)
  if (!ctx || !resps || !packed || !count) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  const size_t in_bytes = (size_t)count * 2 * kN * 8, out_bytes = (size_t)count * ctx->resp_bytes;
  DevBuf din, dout;
  CK(din.alloc(in_bytes), "alloc");
  CK(dout.alloc(out_bytes), "alloc");
  CK(cudaMemcpyAsync(din.p, resps, in_bytes, cudaMemcpyHostToDevice, ctx->stream), "upload");
  launch_pack_response(din.as<uint64_t>(), 2 * (size_t)kN, dout.as<uint8_t>(), ctx->resp_bytes,
                       (int)count, ctx->C, ctx->stream);
  ctx->launches++;
  CK(cudaGetLastError(), "pack launch");
  CK(cudaMemcpyAsync(packed, dout.p, out_bytes, cudaMemcpyDeviceToHost, ctx->stream), "download");
  CK(cudaStreamSynchronize(ctx->stream), "pack");
  return OPIR_OK;
}

// other_dim_mux (server.cpp:295-334): one folding level of `count`
// ciphertexts with one RGSW selection ciphertext, on the device.
int opir_other_dim_mux(opir_ctx *ctx, uint64_t *result, uint64_t count, const uint64_t *sel) {
  RNS_UNSUPPORTED("other_dim_mux")
  if (!ctx || !result || !sel) return OPIR_ERR_ARG;
  if (count < 2 || count % 2 || count / 2 > 0x7fffffff)
    return ctx->fail(OPIR_ERR_ARG, "other_dim_mux folds an even number (>= 2) of ciphertexts");
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  const size_t CTW = 2 * (size_t)kN;
  const size_t res_bytes = count * CTW * 8, sel_bytes = 2 * (size_t)ctx->prm.gsw_l * CTW * 8;
  DevBuf dres, dsel;
  CK(dres.alloc(res_bytes), "alloc");
  CK(dsel.alloc(sel_bytes), "alloc");
  CK(cudaMemcpyAsync(dres.p, result, res_bytes, cudaMemcpyHostToDevice, ctx->stream), "upload");
  CK(cudaMemcpyAsync(dsel.p, sel, sel_bytes, cudaMemcpyHostToDevice, ctx->stream), "upload");
  // the folds work on ciphertexts in NTT form
  launch_ntt(ctx->Mq.tab, dres.as<uint64_t>(), count * 2, false, ctx->stream);
  launch_fold(dres.as<uint64_t>(), count * CTW, dsel.as<uint64_t>(), 2 * (size_t)ctx->prm.gsw_l * CTW,
              (int)(count / 2), 1, ctx->Mq.tab, ctx->C, ctx->stream);
  launch_ntt(ctx->Mq.tab, dres.as<uint64_t>(), count, true, ctx->stream);
  ctx->launches += 3;
  CK(cudaGetLastError(), "fold launch");
  CK(cudaMemcpyAsync(result, dres.p, res_bytes / 2, cudaMemcpyDeviceToHost, ctx->stream),
     "download");
  CK(cudaStreamSynchronize(ctx->stream), "other_dim_mux");
  return OPIR_OK;
}

}  // extern "C"


// ===========================================================================
// Serving: continuous batching (no counterpart in the reference, which
// answers one make_query call at a time).  A worker thread takes submitted
// queries from per-database FIFOs (serve_core.h), forms a batch whenever a
// lane (stream + workspace) is free and the dispatch rule allows, and runs
// the whole pipeline for it; up to cfg.lanes batches are on the device at
// once, so a batch's transfers and kernels overlap the previous one's.
// ===========================================================================
namespace {

void CUDART_CB lane_done_cb(void *arg) {
  // runs on a CUDA runtime thread: no CUDA calls, no lock held by anyone
  // across a CUDA call
  Lane *L = static_cast<Lane *>(arg);
  L->finished.store(true);
  L->owner->wake();
}

// (ctx->mu and S.mu held)
void fail_ticket(Serving &S, uint64_t ticket, int rc, double t) {
  auto it = S.tickets.find(ticket);
  if (it == S.tickets.end()) return;
  it->second.state = 2;
  it->second.rc = rc;
  it->second.t_done = t;
  it->second.query.clear();
  S.failed++;
}

// (ctx->mu and S.mu held)
int dispatch(opir_ctx *ctx, Serving &S, Lane &L) {
  std::vector<serve::Pending> reqs = S.queue.pop_batch(S.cfg.max_batch);
  if (reqs.empty()) return OPIR_OK;
  const double t = now_s();
  Db *db = find_db(ctx, reqs[0].db);
  std::vector<serve::Pending> ok;
  std::vector<uint64_t> ids;
  for (const auto &r : reqs) {
    auto it = ctx->clients.find(r.client);
    const bool servable = db && it != ctx->clients.end() && it->second->has_galois &&
                          it->second->levels >= (uint32_t)db->h &&
                          (db->ndim == 1 || it->second->has_gsw);
    if (!servable) {
      fail_ticket(S, r.ticket, db ? OPIR_ERR_UNKNOWN_CLIENT : OPIR_ERR_UNKNOWN_DB, t);
      continue;
    }
    ok.push_back(r);
    ids.push_back(r.client);
  }
  S.done_cv.notify_all();
  if (ok.empty()) return OPIR_OK;
  const int n = (int)ok.size();
  const size_t CTB = 2 * (size_t)kN * 8;
  Workspace &W = L.ws;
  int rc = OPIR_OK;
  auto fail_all = [&](int code) {
    for (const auto &r : ok) fail_ticket(S, r.ticket, code, now_s());
    S.done_cv.notify_all();
    return code;
  };
  if (W.queries.alloc(n * CTB) != cudaSuccess || W.resp.alloc(n * CTB) != cudaSuccess ||
      W.packed.alloc(n * ctx->resp_bytes + 16) != cudaSuccess ||
      W.h_in.alloc(n * CTB) != cudaSuccess ||
      W.h_out.alloc(n * (CTB + ctx->resp_bytes)) != cudaSuccess) {
    cudaGetLastError();
    ctx->fail(OPIR_ERR_OOM, "serving lane buffers");
    return fail_all(OPIR_ERR_OOM);
  }
  for (int j = 0; j < n; j++) {
    Ticket &tk = S.tickets[ok[j].ticket];
    std::memcpy(static_cast<uint8_t *>(W.h_in.p) + j * CTB, tk.query.data(), CTB);
    tk.query.clear();
    tk.query.shrink_to_fit();
    tk.state = 1;
  }
  if (cudaMemcpyAsync(W.queries.p, W.h_in.p, n * CTB, cudaMemcpyHostToDevice, L.stream) !=
      cudaSuccess)
    return fail_all(ctx->cuda_fail(cudaGetLastError(), "upload queries"));
  const PipeEnv E{&W, L.stream, L.status.as<uint32_t>(), false, true};
  rc = run_pipeline(ctx, *db, n, ids.data(), W.queries.as<uint64_t>(), W.resp.as<uint64_t>(),
                    W.packed.as<uint8_t>(), nullptr, E);
  if (rc) return fail_all(rc);
  uint8_t *h_resp = static_cast<uint8_t *>(W.h_out.p);
  if (cudaMemcpyAsync(h_resp, W.resp.p, n * CTB, cudaMemcpyDeviceToHost, L.stream) != cudaSuccess ||
      cudaMemcpyAsync(h_resp + n * CTB, W.packed.p, n * ctx->resp_bytes, cudaMemcpyDeviceToHost,
                      L.stream) != cudaSuccess ||
      cudaMemcpyAsync(L.h_status.p, L.status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                      L.stream) != cudaSuccess ||
      cudaEventRecord(L.done, L.stream) != cudaSuccess ||
      cudaLaunchHostFunc(L.stream, lane_done_cb, &L) != cudaSuccess) {
    // the batch may still run: wait for it before the buffers are reused
    cudaStreamSynchronize(L.stream);
    if (ctx->key_budget)
      for (uint64_t id : ids) ctx->lru.unpin(id);
    return fail_all(ctx->cuda_fail(cudaGetLastError(), "serving batch"));
  }
  for (uint64_t id : ids) ctx->clients[id]->inflight++;
  L.busy = true;
  L.finished = false;
  L.db = ok[0].db;
  L.reqs = std::move(ok);
  L.clients = std::move(ids);
  S.batches++;
  S.batched_queries += n;
  return OPIR_OK;
}

// (ctx->mu and S.mu held; the lane's stream has passed its callback)
void complete_lane(opir_ctx *ctx, Serving &S, Lane &L) {
  const int n = (int)L.reqs.size();
  const size_t CTB = 2 * (size_t)kN * 8;
  const uint32_t st = *static_cast<const uint32_t *>(L.h_status.p);
  int rc = OPIR_OK;
  if (st) {
    rc = OPIR_ERR_TIMEOUT;
    cudaMemsetAsync(L.status.p, 0, sizeof(uint32_t), L.stream);
  }
  const double t = now_s();
  const uint8_t *h_resp = static_cast<const uint8_t *>(L.ws.h_out.p);
  const uint8_t *h_packed = h_resp + n * CTB;
  for (int j = 0; j < n; j++) {
    auto it = S.tickets.find(L.reqs[j].ticket);
    if (it == S.tickets.end()) continue;
    Ticket &tk = it->second;
    tk.state = 2;
    tk.rc = rc;
    tk.t_done = t;
    if (rc) {
      S.failed++;
      continue;
    }
    tk.resp.resize(2 * kN);
    std::memcpy(tk.resp.data(), h_resp + j * CTB, CTB);
    tk.packed.assign(h_packed + j * ctx->resp_bytes, h_packed + (j + 1) * ctx->resp_bytes);
    S.completed++;
    S.lat_ms.push_back((t - tk.t_submit) * 1e3);
    S.t_last = t;
  }
  for (uint64_t id : L.clients) {
    auto it = ctx->clients.find(id);
    if (it != ctx->clients.end() && it->second->inflight > 0) it->second->inflight--;
    if (ctx->key_budget) ctx->lru.unpin(id);
  }
  L.busy = false;
  L.finished = false;
  L.reqs.clear();
  L.clients.clear();
  S.done_cv.notify_all();
}

void serve_loop(opir_ctx *ctx) {
  Serving &S = *ctx->serving;
  cudaSetDevice(ctx->device);
  const double max_wait = S.cfg.max_wait_us * 1e-6;
  for (;;) {
    uint64_t seen;
    {
      std::lock_guard<std::mutex> g(S.wake_mu);
      seen = S.wake_seq;
    }
    bool act = false;
    double timeout = 0.01;
    {
      std::lock_guard<std::mutex> g(S.mu);
      int busy = 0, idle = 0;
      bool finished = false;
      for (auto &L : S.lanes) {
        if (L->busy) {
          busy++;
          finished |= L->finished.load();
        } else {
          idle++;
        }
      }
      const double wait = S.queue.size() ? now_s() - S.queue.oldest() : 0.0;
      act = finished || serve::should_dispatch(S.queue.size(), S.cfg.max_batch, busy, idle,
                                               S.stop ? 1e30 : wait, max_wait);
      if (!act && S.stop && !S.queue.size() && !busy) return;
      // until a submission, a finished batch, stop, or the oldest request's deadline
      if (S.queue.size() && busy) timeout = std::max(0.0, max_wait - wait);
    }
    if (!act) {
      std::unique_lock<std::mutex> lk(S.wake_mu);
      S.wake_cv.wait_for(lk, std::chrono::duration<double>(timeout + 2e-5),
                         [&] { return S.wake_seq != seen; });
      continue;
    }
    std::lock_guard<std::mutex> g(ctx->mu);
    std::lock_guard<std::mutex> g2(S.mu);
    for (auto &L : S.lanes)
      if (L->busy && L->finished.load()) complete_lane(ctx, S, *L);
    for (;;) {
      int busy = 0, idle = 0;
      Lane *free_lane = nullptr;
      for (auto &L : S.lanes) {
        if (L->busy) {
          busy++;
        } else {
          idle++;
          if (!free_lane) free_lane = L.get();
        }
      }
      const double wait = S.queue.size() ? now_s() - S.queue.oldest() : 0.0;
      if (!serve::should_dispatch(S.queue.size(), S.cfg.max_batch, busy, idle,
                                  S.stop ? 1e30 : wait, max_wait))
        break;
      dispatch(ctx, S, *free_lane);
    }
  }
}

// Size a lane's buffers for max_batch queries on every resident database
// (and build the tensor-core limb planes), so that no batch allocates --
// freeing device memory would synchronise the device under the worker's locks.
int presize_lane(opir_ctx *ctx, Lane &L, int max_batch) {
  const size_t CTB = 2 * (size_t)kN * 8;
  Workspace &W = L.ws;
  for (auto &kv : ctx->dbs) {
    Db &db = *kv.second;
    int rc = ensure_workspace(ctx, db, max_batch, W);
    if (rc) return rc;
    const int n1 = (int)db.shape.fst_dim_sz, nr = (int)db.shape.other_dim_sz;
    bool tensor = false;  // any batch size up to max_batch on the tensor engine
    for (int b = 2; b <= max_batch && !tensor; b++)
      tensor = engine_for(ctx, db, b) == OPIR_ENGINE_TENSOR;
    if (tensor) {
      CK(W.ql.alloc(tc_query_limb_bytes(n1, max_batch)), "alloc query limbs");
      if (!db.dbl_valid) {
        CK(db.dbl.alloc(tc_db_limb_bytes(n1, nr)), "alloc database limb plane");
        launch_db_limbs(db.dbs.as<uint64_t>(), db.dbl.as<uint16_t>(), n1, nr, L.stream);
        ctx->launches++;
        CK(cudaStreamSynchronize(L.stream), "database limb plane");
        db.dbl_valid = true;
      }
    }
  }
  CK(W.queries.alloc(max_batch * CTB), "alloc queries");
  CK(W.resp.alloc(max_batch * CTB), "alloc response");
  CK(W.packed.alloc(max_batch * ctx->resp_bytes + 16), "alloc packed");
  CK(W.h_in.alloc(max_batch * CTB), "alloc pinned");
  CK(W.h_out.alloc(max_batch * (CTB + ctx->resp_bytes)), "alloc pinned");
  return OPIR_OK;
}

}  // namespace

extern "C" {

int opir_serve_start(opir_ctx *ctx, const opir_serve_config *cfg) {
  RNS_UNSUPPORTED("serving")
  if (!ctx || !cfg || !cfg->max_batch || cfg->lanes < 1 || cfg->lanes > 4) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (serving_active(ctx)) return ctx->fail(OPIR_ERR_STATE, "serving is already active");
  cudaSetDevice(ctx->device);
  // queued synchronous work may still read key slots that a lane would refill
  CK(cudaStreamSynchronize(ctx->stream), "sync");
  auto S = std::make_unique<Serving>();
  S->cfg = *cfg;
  for (uint32_t i = 0; i < cfg->lanes; i++) {
    auto L = std::make_unique<Lane>();
    L->owner = S.get();
    CK(cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking), "lane stream");
    CK(cudaEventCreateWithFlags(&L->done, cudaEventDisableTiming), "lane event");
    CK(L->status.alloc(kStatusWords * sizeof(uint32_t)), "lane status");
    CK(cudaMemset(L->status.p, 0, kStatusWords * sizeof(uint32_t)), "lane status");
    CK(L->h_status.alloc(sizeof(uint32_t)), "lane status");
    const int rc = presize_lane(ctx, *L, (int)cfg->max_batch);
    if (rc) return rc;
    S->lanes.push_back(std::move(L));
  }
  S->active = true;
  ctx->serving = std::move(S);
  ctx->serving->worker = std::thread(serve_loop, ctx);
  return OPIR_OK;
}

int opir_serve_stop(opir_ctx *ctx) {
  if (!ctx) return OPIR_ERR_ARG;
  Serving *S;
  {
    std::lock_guard<std::mutex> g(ctx->mu);
    if (!serving_active(ctx)) return OPIR_OK;
    S = ctx->serving.get();
  }
  {
    std::lock_guard<std::mutex> g(S->mu);
    S->stop = true;
  }
  S->wake();
  if (S->worker.joinable()) S->worker.join();
  std::lock_guard<std::mutex> g(ctx->mu);
  S->active = false;
  return OPIR_OK;
}

int opir_submit(opir_ctx *ctx, uint32_t db_id, uint64_t client_id, const uint64_t *query,
                uint64_t *ticket) {
  if (!ctx || !query || !ticket) return OPIR_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (!serving_active(ctx)) return ctx->fail(OPIR_ERR_STATE, "serving is not active");
  Db *db = find_db(ctx, db_id);
  if (!db) return ctx->fail(OPIR_ERR_UNKNOWN_DB, "unknown database %u", db_id);
  auto it = ctx->clients.find(client_id);
  if (it == ctx->clients.end() || !it->second->has_galois ||
      (db->ndim > 1 && !it->second->has_gsw))
    return ctx->fail(OPIR_ERR_UNKNOWN_CLIENT, "no keys for client %llu",
                     (unsigned long long)client_id);
  if (it->second->levels < (uint32_t)db->h)
    return ctx->fail(OPIR_ERR_ARG, "client %llu has %u Galois levels, database needs %d",
                     (unsigned long long)client_id, it->second->levels, db->h);
  Serving &S = *ctx->serving;
  {
    std::lock_guard<std::mutex> g2(S.mu);
    if (S.stop) return ctx->fail(OPIR_ERR_STATE, "serving is stopping");
    const uint64_t id = S.next_ticket++;
    Ticket &tk = S.tickets[id];
    tk.db = db_id;
    tk.client = client_id;
    tk.query.assign(query, query + 2 * (size_t)kN);
    tk.t_submit = now_s();
    if (!S.submitted) S.t_first = tk.t_submit;
    S.submitted++;
    S.queue.push(serve::Pending{id, db_id, client_id, tk.t_submit});
    *ticket = id;
  }
  S.wake();
  return OPIR_OK;
}

static int take_ticket(opir_ctx *ctx, Serving &S, uint64_t ticket, uint64_t *resp,
                       uint8_t *packed) {
  auto it = S.tickets.find(ticket);
  Ticket &tk = it->second;
  const int rc = tk.rc;
  if (!rc) {
    if (resp) std::memcpy(resp, tk.resp.data(), 2 * (size_t)kN * 8);
    if (packed) std::memcpy(packed, tk.packed.data(), ctx->resp_bytes);
  }
  S.tickets.erase(it);
  return rc;
}

int opir_poll(opir_ctx *ctx, uint64_t ticket, uint64_t *resp, uint8_t *packed, int *done) {
  if (!ctx || !done) return OPIR_ERR_ARG;
  *done = 0;
  Serving *S = ctx->serving.get();
  if (!S) return OPIR_ERR_STATE;
  std::lock_guard<std::mutex> g(S->mu);
  auto it = S->tickets.find(ticket);
  if (it == S->tickets.end()) return OPIR_ERR_ARG;
  if (it->second.state != 2) return OPIR_OK;
  *done = 1;
  return take_ticket(ctx, *S, ticket, resp, packed);
}

int opir_wait(opir_ctx *ctx, uint64_t ticket, uint32_t timeout_ms, uint64_t *resp,
              uint8_t *packed) {
  if (!ctx) return OPIR_ERR_ARG;
  Serving *S = ctx->serving.get();
  if (!S) return OPIR_ERR_STATE;
  std::unique_lock<std::mutex> lk(S->mu);
  const bool ready = S->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] {
    auto it = S->tickets.find(ticket);
    return it == S->tickets.end() || it->second.state == 2;
  });
  if (S->tickets.find(ticket) == S->tickets.end()) return OPIR_ERR_ARG;
  if (!ready) return OPIR_ERR_TIMEOUT;
  return take_ticket(ctx, *S, ticket, resp, packed);
}

int opir_serve_stats_get(opir_ctx *ctx, opir_serve_stats *out) {
  if (!ctx || !out) return OPIR_ERR_ARG;
  Serving *S = ctx->serving.get();
  if (!S) return OPIR_ERR_STATE;
  std::lock_guard<std::mutex> g(S->mu);
  std::memset(out, 0, sizeof *out);
  out->submitted = S->submitted;
  out->completed = S->completed;
  out->failed = S->failed;
  out->batches = S->batches;
  out->queued = S->queue.size();
  out->mean_batch = S->batches ? (double)S->batched_queries / (double)S->batches : 0.0;
  out->p50_ms = serve::percentile(S->lat_ms, 50);
  out->p99_ms = serve::percentile(S->lat_ms, 99);
  out->max_ms = serve::percentile(S->lat_ms, 100);
  double sum = 0;
  for (double v : S->lat_ms) sum += v;
  out->mean_ms = S->lat_ms.empty() ? 0.0 : sum / (double)S->lat_ms.size();
  const double span = S->t_last - S->t_first;
  out->queries_per_s = span > 0 ? (double)S->completed / span : 0.0;
  return OPIR_OK;
}

}  // extern "C"

// ===========================================================================
// First dimension without allocation
//
// For callers that must not allocate device memory during a call: a request
// thread with a latency budget (cudaMalloc/cudaFree synchronise the device)
// or a host process whose device memory is reserved up front by another
// allocator.  The query operand of the scan lives in the file-scope array
// below instead of context workspace.  Every GPU that loads this library
// holds the array until the process exits.
// ===========================================================================

// Room for the transposed query operand: n1 * N * 16 bytes, so n1 <= 512.
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;  // 16 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

extern "C" int opir_first_dim_noalloc(opir_ctx *ctx, uint32_t db_id, const uint64_t *d_fst_cts,
                                      uint64_t *d_out) {
  RNS_UNSUPPORTED("the allocation-free first dimension")
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
  // The host-side symbol is not a device address: look the array up once per
  // context, with the context's device current (a context never outlives the
  // CUDA context its device buffers live in, so the address stays valid).
  if (!ctx->noalloc_scratch) {
    void *p = nullptr;
    CK(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(static scratch)");
    ctx->noalloc_scratch = p;
  }
  uint4 *qs = static_cast<uint4 *>(ctx->noalloc_scratch);
  cudaStream_t s = ctx->stream;
  const size_t CTW = 2 * (size_t)kN;
  // One query, so this is the plain streaming scan (engine_for picks it for
  // batch 1 too); the batched engines' operand buffers and the tensor
  // engine's limb planes, which are allocated on demand, are never touched.
  // The operand is fully rewritten before the scan reads it: nothing to clear.
  launch_query_prep(d_fst_cts, n1 * CTW, qs, (size_t)kN * n1, (int)n1, 1, ctx->Mq.tab, s);
  launch_scan(db->dbs.as<uint64_t>(), qs, (size_t)kN * n1, d_out, nr * CTW, (int)n1, (int)nr, 1,
              ctx->C, ctx->Mq.tab.mu_lo, ctx->Mq.tab.mu_hi, ctx->status.as<uint32_t>(), s,
              db->scan_cfg);
  launch_ntt(ctx->Mq.tab, d_out, nr * 2, true, s);
  ctx->launches += 3;
  CK(cudaGetLastError(), "first dimension launch");
  return OPIR_OK;
}
