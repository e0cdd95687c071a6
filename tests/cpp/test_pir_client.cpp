// test_pir_client.cpp -- the header-only C++ client (include/onionpir_client.hpp)
// and parameter derivation (include/onionpir_params.hpp) against the CPU
// oracle, without a GPU:
//   1. PirParams::derive gives the oracle's parameters (pir.cpp:9-112) for
//      a range of database shapes;
//   2. a seeded PirClient's secret key, Galois keys, RGSW(sk) and queries are
//      the oracle client's, word for word;
//   3. the reference's test_pir criterion (tests.cpp:110-134) with the
//      oracle as the server: every decoded entry equals the database entry.
#include <cstdio>
#include <cstring>
#include <sstream>
#include <vector>

#include "onionpir_client.hpp"
#include "opir_oracle.h"

static int failures = 0;
#define CHECK(cond, ...)                 \
  do {                                   \
    if (!(cond)) {                       \
      std::printf("FAIL: " __VA_ARGS__); \
      std::printf("\n");                 \
      failures++;                        \
    }                                    \
  } while (0)

int main() {
  const uint64_t shapes[][2] = {{4096, 256}, {1 << 13, 64},    {1 << 14, 1024}, {1 << 18, 512},
                                {1 << 21, 1024}, {1000, 100}, {16, 4},         {1 << 20, 4096}};
  for (const auto &s : shapes) {
    orc_ctx *o = orc_create(s[0], s[1], 0, 5, 10, 16, 27, 60, 60);
    orc_params P;
    orc_get_params(o, &P);
    const onionpir::PirParams D = onionpir::PirParams::derive(s[0], s[1]);
    const bool same = D.q == P.q && D.p == P.p && D.t == P.t && D.small_q == P.small_q &&
                      D.base_log2 == P.base_log2 && D.base_log2_key == P.base_log2_key &&
                      D.fst_dim_sz == P.n1 && D.other_dim_sz == P.n_rest &&
                      D.entry_size == P.entry_size && D.entries_per_pt == P.entries_per_pt &&
                      D.bits_per_coeff == P.bits_per_coeff && D.ndim() == P.ndim &&
                      D.expan_height() == P.h && D.num_pt() == P.num_pt;
    CHECK(same, "derive(%llu, %llu) differs from the oracle", (unsigned long long)s[0],
          (unsigned long long)s[1]);
    orc_destroy(o);
  }
  std::printf("derive: %zu shapes checked\n", sizeof(shapes) / sizeof(shapes[0]));

  const uint64_t num_entries = 1 << 13, max_fst_dim = 64, db_seed = 5150;
  const size_t N = 2048;
  orc_ctx *o = orc_create(num_entries, max_fst_dim, 0, 5, 10, 16, 27, 60, 60);
  orc_params P;
  orc_get_params(o, &P);
  const onionpir::PirParams params = onionpir::PirParams::derive(num_entries, max_fst_dim);
  std::vector<uint64_t> db(P.num_pt * N);
  orc_build_db(o, db_seed, db.data());

  int ok = 0, identical = 0;
  const int iters = 6;
  std::vector<int8_t> sk(N);
  std::vector<uint64_t> gk(P.h * 4 * N), gsw(2 * P.l_key * 2 * N), q(2 * N), gsw_ntt(gsw.size()),
      resp(2 * N);
  std::vector<uint8_t> packed(orc_response_bytes(o)), expect(P.entry_size);
  for (int i = 0; i < iters; i++) {
    const onionpir::PirClient client(params, 100 + i, 7 + i);
    orc_keygen(o, 7 + i, sk.data());
    orc_make_galois_keys(o, sk.data(), 70 + i, gk.data());
    orc_make_gsw_key(o, sk.data(), 700 + i, gsw.data());
    const uint64_t idx = (i * 2654435761ULL + 3) % P.num_entries;
    orc_make_query(o, sk.data(), 7000 + i, idx, q.data());
    const auto cgk = client.create_galois_keys(70 + i);
    const auto cgsw = client.generate_gsw_from_key(700 + i);
    const auto cq = client.fast_generate_query(idx, 7000 + i);
    const bool same = client.secret_key() == sk && cgk == gk && cgsw == gsw && cq == q;
    identical += same;
    // the oracle answers the client's query; the client decodes the stream
    orc_gsw_key_to_ntt(o, cgsw.data(), 2 * P.l_key, gsw_ntt.data());
    orc_make_query_server(o, db.data(), cgk.data(), gsw_ntt.data(), cq.data(), resp.data(),
                          packed.data(), nullptr);
    std::stringstream stream;
    stream.write(reinterpret_cast<const char *>(packed.data()), (std::streamsize)packed.size());
    const onionpir::Ciphertext ct = client.load_resp_from_stream(stream);
    int budget = 0;
    const onionpir::Plaintext plain = client.decrypt_mod_q(ct, &budget);
    const onionpir::Entry entry = client.get_entry_from_plaintext(idx, plain);
    orc_gen_entries(o, db_seed, idx, 1, expect.data());
    const bool good = entry == expect && ct == resp;
    ok += good;
    std::printf("entry %llu: %s, %s, noise budget %d\n", (unsigned long long)idx,
                good ? "Success" : "Failure", same ? "same as the oracle client" : "DIFFERS", budget);
  }
  orc_destroy(o);
  std::printf("Success rate: %d/%d, same as the oracle client: %d/%d\n", ok, iters, identical,
              iters);
  return failures || ok != iters || identical != iters;
}
