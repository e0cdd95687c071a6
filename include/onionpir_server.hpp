// onionpir_server.hpp -- header-only C++ PirServer over the GB300 C ABI.
//
// Keeps the method names and meaning of the reference class
// (src/includes/server.h:13-51): the constructor takes the parameter set,
// gen_data / push_database_chunk fill the database, set_client_galois_key /
// set_client_gsw_key register a client, make_query answers a query and
// save_resp_to_stream writes the packed response.  Errors are thrown as the
// reference's exception types: std::invalid_argument for bad arguments,
// std::out_of_range for an unknown client (std::map::at in the reference),
// std::runtime_error for device failures.  SEAL objects are replaced by plain
// arrays (ciphertext = uint64_t[2][N], coefficient form, mod q); SEAL wire
// decoding is not part of this header.
#pragma once

#include <cstdint>
#include <ostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "onionpir_gpu.h"
#include "onionpir_params.hpp"

namespace onionpir {

class PirServer {
 public:
  explicit PirServer(const PirParams &p, int device = 0) : params_(p) {
    opir_params gp{};
    gp.poly_degree = p.poly_degree;
    gp.coeff_modulus = p.q;
    gp.special_modulus = p.p;
    gp.plain_modulus = p.t;
    gp.small_modulus = p.small_q;
    gp.gsw_l = p.l;
    gp.gsw_base_log2 = p.base_log2;
    gp.gsw_l_key = p.l_key;
    gp.gsw_base_log2_key = p.base_log2_key;
    const int rc = opir_ctx_create(&gp, device, &ctx_);
    if (rc != OPIR_OK) throw std::invalid_argument("opir_ctx_create failed: " + std::to_string(rc));
    opir_db_shape sh{p.fst_dim_sz, p.other_dim_sz, p.entry_size, p.entries_per_pt,
                     p.bits_per_coeff};
    check(opir_db_create(ctx_, &sh, &db_));
    resp_bytes_ = opir_response_bytes(ctx_);
  }
  ~PirServer() { opir_ctx_destroy(ctx_); }
  PirServer(const PirServer &) = delete;
  PirServer &operator=(const PirServer &) = delete;

  // server.cpp:47-78 (entries derived from `seed` instead of /dev/urandom)
  void gen_data(uint64_t seed) { check(opir_db_fill_synthetic(ctx_, db_, seed)); }

  // server.cpp:635-701: fst_dim_sz * entries_per_pt entries of at most
  // entry_size bytes (shorter ones are zero-padded)
  void push_database_chunk(const std::vector<Entry> &chunk, size_t chunk_idx) {
    const size_t n = (size_t)params_.fst_dim_sz * params_.entries_per_pt;
    if (chunk.size() != n) throw std::invalid_argument("chunk must hold fst_dim_sz entries");
    std::vector<uint8_t> flat(n * params_.entry_size, 0);
    for (size_t i = 0; i < n; ++i) {
      if (chunk[i].size() > params_.entry_size)
        throw std::invalid_argument("Entry size is too large");
      std::copy(chunk[i].begin(), chunk[i].end(), flat.begin() + i * params_.entry_size);
    }
    check(opir_db_push_chunk(ctx_, db_, flat.data(), n, chunk_idx));
  }

  // server.cpp:503-517: the entry read back from the device database
  Entry direct_get_entry(size_t entry_idx) const {
    Entry e(params_.entry_size);
    check(opir_db_get_entry(ctx_, db_, entry_idx, e.data()));
    return e;
  }

  // server.cpp:480-484; keys [levels][2][2][N] in NTT form
  void set_client_galois_key(size_t client_id, const std::vector<uint64_t> &keys) {
    const size_t per = 4 * (size_t)params_.poly_degree;
    if (keys.empty() || keys.size() % per) throw std::invalid_argument("bad Galois key size");
    check(opir_set_galois_key(ctx_, client_id, keys.data(), (uint32_t)(keys.size() / per)));
  }
  // server.cpp:486-500; rows [2 l_key][2][N] in coefficient form
  void set_client_gsw_key(size_t client_id, const std::vector<uint64_t> &rows) {
    if (rows.size() != 2 * (size_t)params_.l_key * 2 * params_.poly_degree)
      throw std::invalid_argument("bad RGSW key size");
    check(opir_set_gsw_key(ctx_, client_id, rows.data()));
  }

  // server.cpp:520-579: the response mod small_q
  Ciphertext make_query(size_t client_id, const Ciphertext &query) {
    if (query.size() != 2 * (size_t)params_.poly_degree)
      throw std::invalid_argument("query must be one ciphertext");
    Ciphertext resp(query.size());
    std::vector<uint8_t> packed(resp_bytes_, 0);
    check(opir_make_query(ctx_, db_, client_id, query.data(), resp.data(), packed.data()));
    // the packed bytes are kept only for a query that succeeded
    last_packed_.swap(packed);
    last_resp_ = resp;
    return resp;
  }

  // server.cpp:581-633: writes the packed response; returns its size.  Any
  // response mod small_q is accepted; the last make_query response reuses
  // the bytes the GPU packed with it, others are packed on the GPU.
  size_t save_resp_to_stream(const Ciphertext &response, std::ostream &stream) {
    if (response.size() != 2 * (size_t)params_.poly_degree)
      throw std::invalid_argument("response must be one ciphertext");
    const std::vector<uint8_t> *bytes = &last_packed_;
    std::vector<uint8_t> packed;
    if (response != last_resp_ || last_packed_.empty()) {
      packed.assign(resp_bytes_, 0);
      check(opir_pack_response(ctx_, response.data(), 1, packed.data()));
      bytes = &packed;
    }
    stream.write(reinterpret_cast<const char *>(bytes->data()), (std::streamsize)bytes->size());
    return bytes->size();
  }

  // server.h:39, server.cpp:295-334: folds result = [x || y] to
  // x + RGSW(b) (x) (y - x) with one RGSW selection ciphertext ([2l][2][N],
  // NTT form) and resizes result to its first half, as the reference does.
  void other_dim_mux(std::vector<Ciphertext> &result, const GSWCiphertext &selection_cipher) {
    const size_t ct = 2 * (size_t)params_.poly_degree;
    if (result.empty() || result.size() % 2)
      throw std::invalid_argument("other_dim_mux folds an even number of ciphertexts");
    if (selection_cipher.size() != 2 * (size_t)params_.l * ct)
      throw std::invalid_argument("selection_cipher must be one RGSW ciphertext");
    std::vector<uint64_t> flat(result.size() * ct);
    for (size_t i = 0; i < result.size(); ++i) {
      if (result[i].size() != ct) throw std::invalid_argument("result must hold ciphertexts");
      std::copy(result[i].begin(), result[i].end(), flat.begin() + i * ct);
    }
    check(opir_other_dim_mux(ctx_, flat.data(), result.size(), selection_cipher.data()));
    result.resize(result.size() / 2);
    for (size_t i = 0; i < result.size(); ++i)
      result[i].assign(flat.begin() + i * ct, flat.begin() + (i + 1) * ct);
  }

  // Many queries at once, one pass over the database; each response equals
  // make_query's for the same query.
  std::vector<Ciphertext> make_query_batch(const std::vector<size_t> &client_ids,
                                           const std::vector<Ciphertext> &queries) {
    if (client_ids.size() != queries.size() || queries.empty())
      throw std::invalid_argument("one client id per query");
    const size_t ct = 2 * (size_t)params_.poly_degree;
    std::vector<uint64_t> ids(client_ids.begin(), client_ids.end()), in(queries.size() * ct),
        out(queries.size() * ct);
    for (size_t i = 0; i < queries.size(); ++i) {
      if (queries[i].size() != ct) throw std::invalid_argument("query must be one ciphertext");
      std::copy(queries[i].begin(), queries[i].end(), in.begin() + i * ct);
    }
    check(opir_make_query_batch(ctx_, db_, (uint32_t)ids.size(), ids.data(), in.data(), out.data(),
                                nullptr));
    std::vector<Ciphertext> resps(queries.size());
    for (size_t i = 0; i < queries.size(); ++i)
      resps[i].assign(out.begin() + i * ct, out.begin() + (i + 1) * ct);
    return resps;
  }

  // First-dimension engine of batches (OPIR_ENGINE_*; tensor_min_batch 0 keeps
  // the current crossover) and the device-memory budget for client keys
  // (before the first key is set; 0 = every client resident).
  void set_batch_engine(int engine, uint32_t tensor_min_batch = 0) {
    check(opir_set_batch_engine(ctx_, engine, tensor_min_batch));
  }
  void set_key_budget(uint64_t bytes) { check(opir_set_key_budget(ctx_, bytes)); }
  // Measure the scan tile configurations and the engines at batch sizes
  // 2 .. max_batch on this GPU and adopt the fastest (opir_autotune).
  opir_tune_report autotune(uint32_t max_batch = 64, uint32_t reps = 3) {
    opir_tune_report r{};
    check(opir_autotune(ctx_, db_, max_batch, reps, &r));
    return r;
  }
  uint64_t key_bytes_per_client() const { return opir_key_bytes_per_client(ctx_); }

  // Serving: continuous batching on a worker thread (opir_serve_* in
  // onionpir_gpu.h).  submit() may be called from any thread.
  void serve_start(uint32_t max_batch = 32, uint32_t lanes = 2, uint32_t max_wait_us = 2000) {
    opir_serve_config cfg{max_batch, lanes, max_wait_us};
    check(opir_serve_start(ctx_, &cfg));
  }
  void serve_stop() { check(opir_serve_stop(ctx_)); }
  uint64_t submit(size_t client_id, const Ciphertext &query) {
    if (query.size() != 2 * (size_t)params_.poly_degree)
      throw std::invalid_argument("query must be one ciphertext");
    uint64_t ticket = 0;
    check(opir_submit(ctx_, db_, client_id, query.data(), &ticket));
    return ticket;
  }
  Ciphertext wait(uint64_t ticket, uint32_t timeout_ms = 60000) {
    Ciphertext resp(2 * (size_t)params_.poly_degree);
    check(opir_wait(ctx_, ticket, timeout_ms, resp.data(), nullptr));
    return resp;
  }
  opir_serve_stats serve_stats() {
    opir_serve_stats st{};
    check(opir_serve_stats_get(ctx_, &st));
    return st;
  }

  opir_ctx *ctx() const { return ctx_; }
  uint32_t db_id() const { return db_; }

 private:
  void check(int rc) const {
    if (rc == OPIR_OK) return;
    const std::string msg = opir_last_error(ctx_);
    if (rc == OPIR_ERR_UNKNOWN_CLIENT) throw std::out_of_range(msg);
    if (rc == OPIR_ERR_ARG || rc == OPIR_ERR_UNKNOWN_DB) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
  }
  PirParams params_;
  opir_ctx *ctx_ = nullptr;
  uint32_t db_ = 0;
  uint64_t resp_bytes_ = 0;
  Ciphertext last_resp_;
  std::vector<uint8_t> last_packed_;
};

}  // namespace onionpir
