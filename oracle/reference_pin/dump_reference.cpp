// dump_reference.cpp -- runs the unmodified reference server and client
// (chenyue42/OnionPIRv2 src/*.cpp except main.cpp and tests.cpp, built
// against the SEAL 4.1 fork the reference names in README.md:11-18) on one
// query and writes every array that the oracle and the GPU path are compared
// on, so that the SEAL-level conventions the oracle restates (prime order,
// plaintext lift, key-switch rounding, NTT root and order) can be checked
// against the reference itself wherever SEAL is available.
//
// It defines PirTest, the class src/includes/server.h:50 and client.h:55 name
// as friend (the reference's own tests.cpp defines it; that file is not
// linked here), to read the server's database, keys and intermediate results.
//
// Usage: dump_reference OUT_DIR [query_index]
// Writes, little-endian uint64 arrays unless noted:
//   params.txt       key = value lines (N, primes, t, small_q, gadgets, shape)
//   db_aligned.u64   db_aligned_ [R N][num_pt]        (server.cpp:740)
//   galois.u64       [h][R][2][R+1][N] NTT form       (client.cpp:227-241)
//   gsw_ntt.u64      [2 l_key][2][R][N] NTT form      (server.cpp:486-500)
//   query.u64        [2][R][N] seed expanded          (client.cpp:130-209)
//   leaves.u64       [u][2][R][N]                     (server.cpp:383-428)
//   gsw_rows.u64     [ndim-1][2l][2][R][N] NTT form   (gsw_eval.cpp:254-286)
//   first_dim.u64    [n_rest][2][R][N]                (server.cpp:124-175)
//   response.u64     [2][N] mod small_q               (server.cpp:520-579)
//   response.bin     save_resp_to_stream bytes        (server.cpp:581-633)
//   entry.bin        direct_get_entry(query_index)    (server.cpp:503-517)
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "client.h"
#include "pir.h"
#include "server.h"

namespace {

bool write_file(const std::string &path, const void *p, size_t bytes) {
  std::ofstream f(path, std::ios::binary);
  f.write(static_cast<const char *>(p), (std::streamsize)bytes);
  return (bool)f;
}

bool write_u64(const std::string &path, const std::vector<uint64_t> &v) {
  return write_file(path, v.data(), v.size() * sizeof(uint64_t));
}

// both polynomials of a ciphertext, every RNS component: [2][R][N]
void append_ct(std::vector<uint64_t> &out, const seal::Ciphertext &ct) {
  const size_t words = ct.poly_modulus_degree() * ct.coeff_modulus_size();
  for (size_t poly = 0; poly < 2; ++poly)
    out.insert(out.end(), ct.data(poly), ct.data(poly) + words);
}

void append_gsw(std::vector<uint64_t> &out, const GSWCiphertext &g) {
  for (const auto &row : g) out.insert(out.end(), row.begin(), row.end());
}

}  // namespace

class PirTest {
 public:
  static int dump(const std::string &dir, size_t query_index);
};

int PirTest::dump(const std::string &dir, size_t query_index) {
  PirParams P;
  PirServer server(P);
  server.gen_data();
  PirClient client(P);
  const size_t id = client.get_client_id();
  const size_t N = DatabaseConstants::PolyDegree, R = P.get_rns_mod_cnt();
  std::stringstream gk_stream, gsw_stream, q_stream, resp_stream;
  client.create_galois_keys(gk_stream);
  client.write_gsw_to_stream(client.generate_gsw_from_key(), gsw_stream);
  server.set_client_galois_key(id, gk_stream);
  server.set_client_gsw_key(id, gsw_stream);
  query_index %= P.get_num_entries();
  const seal::Ciphertext query_out = client.fast_generate_query(query_index);
  client.write_query_to_stream(query_out, q_stream);
  const std::string qbytes = q_stream.str();

  // ---- parameters
  {
    const auto all = P.get_seal_params().coeff_modulus();  // q_0 .. q_{R-1}, p
    std::ofstream f(dir + "/params.txt");
    f << "poly_degree = " << N << "\nrns = " << R << "\n";
    for (size_t i = 0; i < all.size(); ++i) f << "modulus" << i << " = " << all[i].value() << "\n";
    f << "plain_modulus = " << P.get_plain_mod() << "\nsmall_q = " << P.get_small_q()
      << "\nl = " << P.get_l() << "\nbase_log2 = " << P.get_base_log2() << "\nl_key = "
      << P.get_l_key() << "\nbase_log2_key = " << P.get_base_log2_key()
      << "\nnum_entries = " << P.get_num_entries() << "\nnum_pt = " << P.get_num_pt()
      << "\nentry_size = " << P.get_entry_size() << "\nn1 = " << P.get_fst_dim_sz()
      << "\nn_rest = " << P.get_other_dim_sz() << "\nndim = " << P.get_dims().size()
      << "\nexpan_height = " << P.get_expan_height() << "\nquery_index = " << query_index
      << "\nmax_fst_dim = " << DatabaseConstants::MaxFstDimSz << "\n";
  }
  // ---- database and keys as the server holds them
  std::vector<uint64_t> buf(server.db_aligned_.get(),
                            server.db_aligned_.get() + P.get_num_pt() * N * R);
  if (!write_u64(dir + "/db_aligned.u64", buf)) return 1;
  buf.clear();
  const seal::GaloisKeys &gk = server.client_galois_keys_.at(id);
  for (size_t a = 0; a < P.get_expan_height(); ++a) {
    const uint32_t elt = (uint32_t)(1 + (N >> a));  // client.cpp:235-237
    for (const seal::PublicKey &comp : gk.key(elt))   // one per ciphertext prime
      append_ct(buf, comp.data());
  }
  if (!write_u64(dir + "/galois.u64", buf)) return 1;
  buf.clear();
  GSWCiphertext &gsw_key = server.client_gsw_keys_.at(id);
  append_gsw(buf, gsw_key);
  if (!write_u64(dir + "/gsw_ntt.u64", buf)) return 1;

  // ---- the query as the server receives it (seed expanded)
  seal::Ciphertext query;
  {
    std::stringstream s(qbytes);
    query.load(server.context_, s);
  }
  buf.clear();
  append_ct(buf, query);
  if (!write_u64(dir + "/query.u64", buf)) return 1;

  // ---- every stage of make_query (server.cpp:520-579)
  seal::Ciphertext q_copy = query;
  std::vector<seal::Ciphertext> leaves = server.fast_expand_qry(id, q_copy);
  buf.clear();
  for (const auto &ct : leaves) append_ct(buf, ct);
  if (!write_u64(dir + "/leaves.u64", buf)) return 1;
  const std::vector<size_t> dims = P.get_dims();
  buf.clear();
  for (size_t i = 1; i < dims.size(); ++i) {
    std::vector<seal::Ciphertext> lwe;
    for (size_t k = 0; k < P.get_l(); ++k) lwe.push_back(leaves[dims[0] + (i - 1) * P.get_l() + k]);
    GSWCiphertext g;
    server.key_gsw_.query_to_gsw(lwe, gsw_key, g);
    append_gsw(buf, g);
  }
  if (!write_u64(dir + "/gsw_rows.u64", buf)) return 1;
  std::vector<seal::Ciphertext> sel(leaves.begin(), leaves.begin() + dims[0]);
  const std::vector<seal::Ciphertext> fd = server.evaluate_first_dim(sel);
  buf.clear();
  for (const auto &ct : fd) append_ct(buf, ct);
  if (!write_u64(dir + "/first_dim.u64", buf)) return 1;

  // ---- the whole query through the public method, and the wire bytes
  std::stringstream q_again(qbytes);
  const seal::Ciphertext resp = server.make_query(id, q_again);
  buf.clear();
  append_ct(buf, resp);
  if (!write_u64(dir + "/response.u64", buf)) return 1;
  server.save_resp_to_stream(resp, resp_stream);
  const std::string rbytes = resp_stream.str();
  if (!write_file(dir + "/response.bin", rbytes.data(), rbytes.size())) return 1;
  const Entry entry = server.direct_get_entry(query_index);
  if (!write_file(dir + "/entry.bin", entry.data(), entry.size())) return 1;

  // the reference's own criterion (tests.cpp:110-134), as a sanity check
  std::stringstream back(rbytes);
  const seal::Ciphertext got = client.load_resp_from_stream(back);
  const Entry decoded = client.get_entry_from_plaintext(query_index, client.decrypt_reply(got));
  std::printf("dumped to %s: query %zu, response %zu bytes, decrypted entry %s\n", dir.c_str(),
              query_index, rbytes.size(), decoded == entry ? "matches" : "DIFFERS");
  return decoded == entry ? 0 : 2;
}

int main(int argc, char **argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s OUT_DIR [query_index]\n", argv[0]);
    return 1;
  }
  return PirTest::dump(argv[1], argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1234);
}
