// test_pir_server.cpp -- the reference's PirTest::test_pir loop
// (src/tests.cpp:40-153) against the C++ PirServer drop-in
// (include/onionpir_server.hpp), with the CPU oracle as the client.
// Success criterion as in the reference (tests.cpp:110-134): the decrypted
// entry equals the database entry; additionally the response must be
// bit-identical to the oracle server's.
#include <cstdio>
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <vector>

#include "onionpir_server.hpp"
#include "opir_oracle.h"

int main() {
  const uint64_t num_entries = 4096, max_fst_dim = 256, seed = 20261203;
  orc_ctx *o = orc_create(num_entries, max_fst_dim, 0, 5, 10, 16, 27, 60, 60);
  orc_params P;
  orc_get_params(o, &P);
  onionpir::PirParams pp;
  pp.q = P.q;
  pp.p = P.p;
  pp.t = P.t;
  pp.small_q = P.small_q;
  pp.l = (uint32_t)P.l;
  pp.base_log2 = (uint32_t)P.base_log2;
  pp.l_key = (uint32_t)P.l_key;
  pp.base_log2_key = (uint32_t)P.base_log2_key;
  pp.fst_dim_sz = (uint32_t)P.n1;
  pp.other_dim_sz = (uint32_t)P.n_rest;
  pp.entry_size = (uint32_t)P.entry_size;
  pp.entries_per_pt = (uint32_t)P.entries_per_pt;
  pp.bits_per_coeff = (uint32_t)P.bits_per_coeff;

  onionpir::PirServer server(pp);
  server.gen_data(seed);
  std::vector<uint64_t> db(P.num_pt * 2048);
  orc_build_db(o, seed, db.data());

  const size_t N = 2048, iters = 13;  // EXPERIMENT_ITERATIONS = 10 + 3 warm-up
  int success = 0, identical = 0;
  std::vector<int8_t> sk(N);
  std::vector<uint64_t> gk(P.h * 4 * N), gsw(2 * P.l_key * 2 * N), gsw_ntt(gsw.size());
  std::vector<uint64_t> query(2 * N), ref(2 * N), ct(2 * N), plain(N);
  std::vector<uint8_t> ref_packed(orc_response_bytes(o)), entry(P.entry_size),
      expect(P.entry_size);
  std::vector<size_t> all_clients;
  std::vector<onionpir::Ciphertext> all_queries, all_resps;
  for (size_t i = 0; i < iters; ++i) {
    const uint64_t client = 1000 + i, idx = (i * 2654435761ULL + 17) % P.num_entries;
    orc_keygen(o, 77 + i, sk.data());
    orc_make_galois_keys(o, sk.data(), 177 + i, gk.data());
    orc_make_gsw_key(o, sk.data(), 277 + i, gsw.data());
    server.set_client_galois_key(client, gk);
    server.set_client_gsw_key(client, gsw);
    orc_make_query(o, sk.data(), 377 + i, idx, query.data());
    const onionpir::Ciphertext resp = server.make_query(client, query);
    all_clients.push_back(client);
    all_queries.push_back(query);
    all_resps.push_back(resp);
    std::stringstream stream;
    const size_t n = server.save_resp_to_stream(resp, stream);
    const std::string bytes = stream.str();
    orc_unpack_response(o, reinterpret_cast<const uint8_t *>(bytes.data()), ct.data());
    int budget = 0;
    orc_decrypt(o, sk.data(), ct.data(), 2, plain.data(), &budget);
    orc_entry_from_plain(o, idx, plain.data(), entry.data());
    orc_gen_entries(o, seed, idx, 1, expect.data());
    const bool ok = n == ref_packed.size() && entry == expect;
    orc_gsw_key_to_ntt(o, gsw.data(), 2 * P.l_key, gsw_ntt.data());
    orc_make_query_server(o, db.data(), gk.data(), gsw_ntt.data(), query.data(), ref.data(),
                          ref_packed.data(), nullptr);
    const bool same = resp == ref && bytes.size() == ref_packed.size() &&
                      std::memcmp(bytes.data(), ref_packed.data(), ref_packed.size()) == 0;
    success += ok;
    identical += same;
    std::printf("query %zu entry %llu: %s, %s, noise budget %d\n", i, (unsigned long long)idx,
                ok ? "Success" : "Failure", same ? "bit-identical" : "DIFFERS", budget);
  }
  bool threw = false;
  try {
    server.make_query(999999, query);
  } catch (const std::out_of_range &) {
    threw = true;
  }
  // the same queries as one batch, and through the serving loop
  const std::vector<onionpir::Ciphertext> batch = server.make_query_batch(all_clients, all_queries);
  int batch_same = 0, served_same = 0;
  for (size_t i = 0; i < iters; ++i) batch_same += batch[i] == all_resps[i];
  server.serve_start(4, 2, 500);
  std::vector<uint64_t> tickets;
  for (size_t i = 0; i < iters; ++i) tickets.push_back(server.submit(all_clients[i], all_queries[i]));
  for (size_t i = 0; i < iters; ++i) served_same += server.wait(tickets[i]) == all_resps[i];
  const opir_serve_stats st = server.serve_stats();
  server.serve_stop();
  std::printf("Success rate: %d/%zu, bit-identical: %d/%zu, unknown client -> out_of_range: %s\n",
              success, iters, identical, iters, threw ? "yes" : "no");
  std::printf("batch == single: %d/%zu, served == single: %d/%zu (%llu batches, p50 %.2f ms)\n",
              batch_same, iters, served_same, iters, (unsigned long long)st.batches, st.p50_ms);
  orc_destroy(o);
  return (success == (int)iters && identical == (int)iters && threw &&
          batch_same == (int)iters && served_same == (int)iters)
             ? 0
             : 1;
}
