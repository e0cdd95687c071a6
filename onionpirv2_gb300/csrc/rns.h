// rns.h -- the multi-modulus server query path (rns_mod_cnt > 1, and any
// power-of-two degree N <= 4096), behind the same C ABI as the N = 2048,
// one-prime path.  capi.cu hands a context created by opir_ctx_create_rns
// to an RnsServer; every supported entry point dispatches to it.
//
// Reference: the PolyDegree = 4096, CoeffMods = {60, 60, 60} presets of
// src/includes/database_constants.h:13-172, decomp_rlwe with CRT composition
// (src/gsw_eval.cpp:108-182), mod_switch_to_next_inplace before the small-q
// switch (src/server.cpp:567-570), RNS key switching in apply_galois_inplace
// (server.cpp:409) and the rest of PirServer::make_query (server.cpp:520-579).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/onionpir_gpu.h"
#include "kernels.h"

namespace opir {

constexpr int kRnsMaxPrimes = 2;  // ciphertext primes
constexpr int kRnsMaxDegree = 4096;

// Per-modulus constants and the scalars of the parameter set, by value to
// every kernel.  Modulus index m: 0 .. R-1 ciphertext primes, R = p.
struct RnsMod {
  uint64_t q, mu_lo, mu_hi;  // floor(2^128 / q)
  uint64_t n_inv, n_inv_s;   // N^-1 mod q and its Shoup companion
};
struct RnsConsts {
  int n, logn, R;
  RnsMod m[kRnsMaxPrimes + 1];
  const ulonglong2 *fwd;  // [R+1][N] {psi^brv(i), companion}
  const ulonglong2 *inv;  // [R+1][N] {psi^-brv(i), companion}
  uint64_t t;
  uint64_t p_half;                              // p >> 1
  uint64_t p_half_mod[kRnsMaxPrimes];           // (p >> 1) mod q_i
  uint64_t p_inv[kRnsMaxPrimes], p_inv_s[kRnsMaxPrimes];        // p^-1 mod q_i
  uint64_t last_half;                           // q_{R-1} >> 1
  uint64_t last_half_mod[kRnsMaxPrimes];        // (q_{R-1} >> 1) mod q_i
  uint64_t last_inv[kRnsMaxPrimes], last_inv_s[kRnsMaxPrimes];  // q_{R-1}^-1 mod q_i
  uint64_t two128[kRnsMaxPrimes];               // 2^128 mod q_i
  uint64_t ms_mant;                             // (double)small_q / (double)q_0 == mant 2^-shift
  int ms_shift, small_w;
  int l, b, l_key, b_key;
};

// Device buffer owned by the multi-modulus path.
struct RnsBuf {
  void *p = nullptr;
  size_t bytes = 0;
  RnsBuf() = default;
  RnsBuf(const RnsBuf &) = delete;
  RnsBuf &operator=(const RnsBuf &) = delete;
  ~RnsBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t n) {
    if (p && n <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    const cudaError_t e = cudaMalloc(&p, n ? n : 16);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  uint64_t *u64() const { return static_cast<uint64_t *>(p); }
};

struct RnsTrace {
  uint64_t *leaves = nullptr, *gsw = nullptr, *first_dim = nullptr;
};

class RnsServer {
 public:
  // opir_ctx_create_rns: checks the parameter set, builds the NTT tables
  static int create(const opir_rns_params &p, int device, std::unique_ptr<RnsServer> *out,
                    std::string *err);
  ~RnsServer();

  int db_create(const opir_db_shape &shape, uint32_t *id);
  int db_destroy(uint32_t id);
  int db_fill_synthetic(uint32_t id, uint64_t seed, cudaStream_t s);
  int db_upload_aligned(uint32_t id, const uint64_t *aligned, cudaStream_t s);
  int set_galois_key(uint64_t client, const uint64_t *keys, uint32_t levels, cudaStream_t s);
  int set_gsw_key(uint64_t client, const uint64_t *rows, cudaStream_t s);
  int erase_client(uint64_t client);
  // one query [2][R][N] (host) -> resp [2][N] mod small_q and packed bytes (host)
  int make_query(uint32_t db, uint64_t client, const uint64_t *query, uint64_t *resp,
                 uint8_t *packed, const RnsTrace *trace, cudaStream_t s);
  // `batch` queries [batch][2][R][N] of clients `clients` (host) -> resps
  // [batch][2][N], packed [batch][bytes]: the queries spread over kLanes
  // lanes that run concurrently, each query the pipeline make_query runs
  int make_query_batch(uint32_t db, uint32_t batch, const uint64_t *clients,
                       const uint64_t *queries, uint64_t *resps, uint8_t *packed,
                       cudaStream_t s);
  int ntt(int mod, bool inverse, uint64_t *polys, uint64_t count, cudaStream_t s);
  int pack_response(const uint64_t *resps, uint32_t count, uint8_t *packed, cudaStream_t s);
  uint64_t response_bytes() const { return resp_bytes_; }
  uint64_t launches() const { return launches_; }
  void set_timing(bool on) { timing_ = on; }
  // replay each (database, client, workspace) query as a CUDA graph
  void set_graphs(bool on);
  bool stage_times(float *ms6) const;
  const std::string &error() const { return err_; }

 private:
  struct Db {
    opir_db_shape shape{};
    uint64_t num_pt = 0;
    int ndim = 1, u = 1, h = 0;
    RnsBuf dbs;  // [R N][n1][n_rest]
  };
  struct Client {
    RnsBuf galois, gsw;
    uint32_t levels = 0;
    bool has_galois = false, has_gsw = false;
  };
  // One query's device workspace, bounded-wait status words and pinned,
  // device-mapped staging [query][response][packed bytes][status word] (the
  // first expansion level reads the query and the last kernels write the rest
  // across the host link themselves: no copy-engine transfers).  Lane 0 is
  // the synchronous call's, on the caller's stream; a batch runs lanes 0 ..
  // kLanes-1 at once, lanes 1 .. on streams of their own, so that the
  // latency-bound tree stages of different queries overlap.
  struct Lane {
    RnsBuf exp0_, exp1_, lift_, acc_, s0_, gsw_, digits_, qn_, scan_qs_, res_, e_, status_;
    void *h_io_ = nullptr;
    uint8_t *d_io_ = nullptr;  // the device address of h_io_
    cudaStream_t stream = nullptr;  // lanes 1 ..: owned
    ~Lane();
  };
  static constexpr int kLanes = 8;
  RnsServer() = default;
  int fail(int code, const std::string &msg);
  int cuda_fail(cudaError_t e, const char *what);
  int prepare_lane(Lane &L);  // staging and status words of a lane
  int ensure_workspace(Lane &L, const Db &db);
  int check_query(Db &db, uint64_t client, Client **cl);
  // copy the query into the lane's staging and launch its pipeline on s
  int start_query(Lane &L, Db &db, Client &cl, const uint64_t *query, const RnsTrace *trace,
                  bool timed, cudaStream_t s);
  // wait for the lane, check its status word, copy the response out
  int finish_query(Lane &L, uint64_t *resp, uint8_t *packed, cudaStream_t s);
  // every kernel of one query, on stream s (captured into a graph or launched)
  int enqueue_query(Lane &L, Db &db, Client &cl, const RnsTrace *trace, bool timed,
                    cudaStream_t s);
  void ntt_launch(const uint64_t *src, size_t src_stride, uint64_t *dst, size_t dst_stride,
                  int polys, int groups, int period, bool inverse, cudaStream_t s);

  opir_rns_params prm_{};
  int device_ = 0;
  RnsConsts C_{};
  RnsBuf fwd_, inv_;
  std::map<uint32_t, std::unique_ptr<Db>> dbs_;
  uint32_t next_db_ = 1;
  std::map<uint64_t, std::unique_ptr<Client>> clients_;
  // workspace (grown on demand)
  // the first dimension on the one-modulus streaming scan, once per prime:
  // its constants (q, 2^30 and 2^60 mod q with Shoup companions) and Barrett
  // mu per prime, its operand (30-bit halves per prime, slot and k) and its
  // bounded-wait status words
  Consts scan_c_[kRnsMaxPrimes] = {};
  uint64_t scan_mu_[kRnsMaxPrimes][2] = {};
  RnsBuf coeffs_;
  Lane lanes_[kLanes];
  uint64_t resp_bytes_ = 0;
  size_t io_resp_off_ = 0, io_packed_off_ = 0, io_status_off_ = 0;  // within a lane's staging
  uint64_t launches_ = 0;
  bool timing_ = false, stage_valid_ = false;
  // the synchronous query as CUDA graphs: executables keyed by every pointer
  // and shape their kernel parameters hold; the least recently used of
  // kMaxGraphs is replaced on a miss
  struct Graph {
    std::vector<uint64_t> key;
    cudaGraphExec_t exec = nullptr;
    uint64_t used = 0, launches = 0;
  };
  static constexpr int kMaxGraphs = 16;
  bool graphs_ = true;
  std::vector<Graph> graphs_cache_;
  uint64_t graph_clock_ = 0;
  void clear_graphs();
  cudaEvent_t ev_[8] = {};  // stage boundaries 0-5, scan kernel 6-7
  std::string err_;
};

}  // namespace opir
