// test_pir_server.cpp -- the reference's PirTest::test_pir loop
// (src/tests.cpp:40-153) with the C++ drop-ins on both sides: the GPU
// PirServer (include/onionpir_server.hpp) answers, the CPU PirClient
// (include/onionpir_client.hpp) makes keys and queries and decodes the
// response stream.  Success criterion as in the reference (tests.cpp:110-134):
// the decrypted entry equals the database entry; additionally the response
// must be bit-identical to the oracle server's.
#include <cstdio>
#include <cstring>
#include <sstream>
#include <string>
#include <stdexcept>
#include <vector>

#include "onionpir_client.hpp"
#include "onionpir_server.hpp"
#include "opir_oracle.h"

int main() {
  const uint64_t num_entries = 4096, max_fst_dim = 256, seed = 20261203;
  orc_ctx *o = orc_create(num_entries, max_fst_dim, 0, 5, 10, 16, 27, 60, 60);
  orc_params P;
  orc_get_params(o, &P);
  const onionpir::PirParams pp = onionpir::PirParams::derive(num_entries, max_fst_dim);

  onionpir::PirServer server(pp);
  server.gen_data(seed);
  std::vector<uint64_t> db(P.num_pt * 2048);
  orc_build_db(o, seed, db.data());

  const size_t N = 2048, iters = 13;  // EXPERIMENT_ITERATIONS = 10 + 3 warm-up
  int success = 0, identical = 0;
  std::vector<uint64_t> gsw_ntt(2 * P.l_key * 2 * N), ref(2 * N);
  std::vector<uint8_t> ref_packed(orc_response_bytes(o)), expect(P.entry_size);
  std::vector<size_t> all_clients;
  std::vector<onionpir::Ciphertext> all_queries, all_resps;
  std::vector<std::string> all_bytes;
  for (size_t i = 0; i < iters; ++i) {
    const uint64_t client_id = 1000 + i, idx = (i * 2654435761ULL + 17) % P.num_entries;
    // odd iterations: keys and queries from OS entropy; even: seeded
    const onionpir::PirClient client =
        i % 2 ? onionpir::PirClient(pp, client_id) : onionpir::PirClient(pp, client_id, 77 + i);
    const std::vector<uint64_t> gk = i % 2 ? client.create_galois_keys() : client.create_galois_keys(177 + i);
    const std::vector<uint64_t> gsw =
        i % 2 ? client.generate_gsw_from_key() : client.generate_gsw_from_key(277 + i);
    server.set_client_galois_key(client_id, gk);
    server.set_client_gsw_key(client_id, gsw);
    const onionpir::Ciphertext query =
        i % 2 ? client.fast_generate_query(idx) : client.fast_generate_query(idx, 377 + i);
    const onionpir::Ciphertext resp = server.make_query(client_id, query);
    all_clients.push_back(client_id);
    all_queries.push_back(query);
    all_resps.push_back(resp);
    std::stringstream stream;
    const size_t n = server.save_resp_to_stream(resp, stream);
    const std::string bytes = stream.str();
    all_bytes.push_back(bytes);
    int budget = 0;
    const onionpir::Plaintext plain =
        client.decrypt_mod_q(client.load_resp_from_stream(stream), &budget);
    const onionpir::Entry entry = client.get_entry_from_plaintext(idx, plain);
    orc_gen_entries(o, seed, idx, 1, expect.data());
    const bool ok = n == ref_packed.size() && entry == expect &&
                    server.direct_get_entry(idx) == expect;  // server.cpp:503-517
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
    server.make_query(999999, all_queries[0]);
  } catch (const std::out_of_range &) {
    threw = true;
  }
  // the same queries as one batch, and through the serving loop
  const std::vector<onionpir::Ciphertext> batch = server.make_query_batch(all_clients, all_queries);
  // save_resp_to_stream packs any response: every batch row and served
  // response must stream the bytes of the single query's response
  int batch_same = 0, served_same = 0;
  for (size_t i = 0; i < iters; ++i) {
    std::stringstream st;
    server.save_resp_to_stream(batch[i], st);
    batch_same += batch[i] == all_resps[i] && st.str() == all_bytes[i];
  }
  server.serve_start(4, 2, 500);
  std::vector<uint64_t> tickets;
  for (size_t i = 0; i < iters; ++i) tickets.push_back(server.submit(all_clients[i], all_queries[i]));
  for (size_t i = 0; i < iters; ++i) {
    const onionpir::Ciphertext r = server.wait(tickets[i]);
    std::stringstream st;
    server.save_resp_to_stream(r, st);
    served_same += r == all_resps[i] && st.str() == all_bytes[i];
  }
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
