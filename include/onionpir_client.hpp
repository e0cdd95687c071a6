// onionpir_client.hpp -- header-only CPU PirClient for the GB300 PirServer.
//
// Keeps the method names and meaning of the reference class
// (src/includes/client.h:4-53, src/client.cpp): get_query_indices,
// fast_generate_query, create_galois_keys, generate_gsw_from_key,
// load_resp_from_stream, decrypt_mod_q, get_entry_from_plaintext.  SEAL
// objects are replaced by plain arrays in the layouts the server takes:
//   query / response   [2][N]          coefficient form (mod q / mod small_q)
//   Galois keys        [h][2][2][N]    level a (element N/2^a + 1), key poly,
//                                      modulus (0 = q, 1 = p), NTT form
//   RGSW(sk) rows      [2 l_key][2][N] coefficient form mod q
// NTT form is SEAL's negacyclic convention: A[k] = a(psi^(2 brv(k) + 1)) with
// psi the smallest primitive 2N-th root of unity mod the prime.
//
// Randomness.  Every randomised method has two forms: without a seed it
// draws from a ChaCha20 stream (RFC 8439 block function) keyed from the
// operating system's entropy; with a seed it draws from a SplitMix64 stream
// started at (seed ^ method tag).  The seeded form is reproducible and NOT
// cryptographically secure: it exists for tests and benchmarks, and the same
// seed gives the same keys, queries and responses on every machine.
//
// Thread safety: a PirClient is immutable after construction; every method is
// const and may run concurrently.  The NTT tables are shared between clients
// of the same moduli.
#pragma once

#include <array>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <istream>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "onionpir_params.hpp"

namespace onionpir {

using Plaintext = std::vector<uint64_t>;  // [N] coefficients mod t

// ---- random streams -------------------------------------------------------

// SplitMix64: state += golden gamma, output = the finaliser of the state.
class SeededStream {
 public:
  explicit SeededStream(uint64_t seed) : s_(seed) {}
  uint64_t next() {
    uint64_t z = (s_ += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }

 private:
  uint64_t s_;
};

// ChaCha20 keystream (RFC 8439 section 2.3) read as little-endian 64-bit
// words; words 12-13 of the state are a 64-bit block counter, 14-15 the nonce.
class ChaChaStream {
 public:
  ChaChaStream(const std::array<uint32_t, 8> &key, uint64_t nonce = 0) : key_(key), nonce_(nonce) {}
  static ChaChaStream from_os() {
    std::ifstream f("/dev/urandom", std::ios::binary);
    std::array<uint32_t, 8> key{};
    uint64_t nonce = 0;
    if (!f.read(reinterpret_cast<char *>(key.data()), sizeof(key)) ||
        !f.read(reinterpret_cast<char *>(&nonce), sizeof(nonce)))
      throw std::runtime_error("no operating-system entropy (/dev/urandom)");
    return ChaChaStream(key, nonce);
  }
  uint64_t next() {
    if (pos_ == 16) {
      const uint32_t n[3] = {(uint32_t)(ctr_ >> 32), (uint32_t)nonce_, (uint32_t)(nonce_ >> 32)};
      block(key_.data(), (uint32_t)ctr_, n, buf_);
      ctr_++;
      pos_ = 0;
    }
    const uint64_t lo = buf_[pos_], hi = buf_[pos_ + 1];
    pos_ += 2;
    return lo | (hi << 32);
  }
  // The block function: 20 rounds over (constants, key, counter, nonce),
  // plus the input state; out[i] is word i of the serialised block.
  static void block(const uint32_t key[8], uint32_t counter, const uint32_t nonce[3],
                    uint32_t out[16]) {
    uint32_t in[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u};
    for (int i = 0; i < 8; i++) in[4 + i] = key[i];
    in[12] = counter;
    for (int i = 0; i < 3; i++) in[13 + i] = nonce[i];
    uint32_t x[16];
    std::memcpy(x, in, sizeof(x));
    for (int r = 0; r < 10; r++) {
      quarter(x, 0, 4, 8, 12), quarter(x, 1, 5, 9, 13), quarter(x, 2, 6, 10, 14),
          quarter(x, 3, 7, 11, 15);
      quarter(x, 0, 5, 10, 15), quarter(x, 1, 6, 11, 12), quarter(x, 2, 7, 8, 13),
          quarter(x, 3, 4, 9, 14);
    }
    for (int i = 0; i < 16; i++) out[i] = x[i] + in[i];
  }

 private:
  static uint32_t rotl(uint32_t v, int c) { return (v << c) | (v >> (32 - c)); }
  static void quarter(uint32_t *x, int a, int b, int c, int d) {
    x[a] += x[b], x[d] = rotl(x[d] ^ x[a], 16);
    x[c] += x[d], x[b] = rotl(x[b] ^ x[c], 12);
    x[a] += x[b], x[d] = rotl(x[d] ^ x[a], 8);
    x[c] += x[d], x[b] = rotl(x[b] ^ x[c], 7);
  }
  std::array<uint32_t, 8> key_;
  uint64_t nonce_, ctr_ = 0;
  uint32_t buf_[16] = {};
  int pos_ = 16;
};

namespace client_detail {

constexpr uint32_t kN = 2048, kLogN = 11;
using u128 = unsigned __int128;

inline uint64_t brv(uint64_t x, uint32_t bits) {
  uint64_t y = 0;
  for (uint32_t i = 0; i < bits; i++) y = (y << 1) | ((x >> i) & 1);
  return y;
}

// uniform in [0, m): top bitlen(m) bits of a word, rejected until below m
template <class Rng>
inline uint64_t uniform(Rng &r, uint64_t m) {
  const uint32_t b = PirParams::bitlen(m);
  for (;;) {
    const uint64_t v = r.next() >> (64 - b);
    if (v < m) return v;
  }
}
// centred binomial with 21 coin pairs per draw (variance 10.5)
template <class Rng>
inline int64_t cbd(Rng &r) {
  const uint64_t v = r.next();
  return (int64_t)__builtin_popcountll(v & 0x1FFFFF) -
         (int64_t)__builtin_popcountll((v >> 21) & 0x1FFFFF);
}

// Negacyclic NTT mod one prime: Harvey butterflies with Shoup companions,
// lazy in [0, 4q) (forward) and [0, 2q) (inverse), outputs fully reduced.
struct Ntt {
  uint64_t q = 0, n_inv = 0, n_inv_s = 0;
  std::vector<uint64_t> fwd, fwd_s, inv, inv_s;

  static uint64_t shoup(uint64_t w, uint64_t q) { return (uint64_t)(((u128)w << 64) / q); }
  static uint64_t mul_lazy(uint64_t x, uint64_t w, uint64_t ws, uint64_t q) {
    const uint64_t hq = (uint64_t)(((u128)x * ws) >> 64);
    return x * w - hq * q;  // in [0, 2q)
  }
  // smallest primitive 2N-th root of unity mod q
  static uint64_t minimal_root(uint64_t q) {
    const uint64_t two_n = 2 * kN, cof = (q - 1) / two_n;
    uint64_t psi = 0;
    for (uint64_t g = 2; g < q && !psi; g++) {
      const uint64_t c = PirParams::powmod(g, cof, q);
      if (PirParams::powmod(c, kN, q) == q - 1) psi = c;
    }
    if (!psi) throw std::invalid_argument("modulus has no 2N-th root of unity");
    uint64_t best = psi, cur = psi;
    const uint64_t sq = PirParams::mulmod(psi, psi, q);
    for (uint64_t k = 1; k < kN; k++) {
      cur = PirParams::mulmod(cur, sq, q);
      if (cur < best) best = cur;
    }
    return best;
  }
  explicit Ntt(uint64_t modulus) : q(modulus), fwd(kN), fwd_s(kN), inv(kN), inv_s(kN) {
    if ((q - 1) % (2 * kN)) throw std::invalid_argument("modulus is not 1 mod 2N");
    const uint64_t psi = minimal_root(q), psi_inv = PirParams::powmod(psi, q - 2, q);
    for (uint32_t i = 0; i < kN; i++) {
      const uint64_t e = brv(i, kLogN);
      fwd[i] = PirParams::powmod(psi, e, q);
      inv[i] = PirParams::powmod(psi_inv, e, q);
      fwd_s[i] = shoup(fwd[i], q);
      inv_s[i] = shoup(inv[i], q);
    }
    n_inv = PirParams::powmod(kN, q - 2, q);
    n_inv_s = shoup(n_inv, q);
  }
  void forward(uint64_t *a) const {  // inputs < 4q
    const uint64_t q2 = 2 * q;
    for (uint32_t m = 1, t = kN >> 1; m < kN; m <<= 1, t >>= 1) {
      for (uint32_t i = 0; i < m; i++) {
        const uint64_t w = fwd[m + i], ws = fwd_s[m + i];
        uint64_t *x = a + 2 * i * t, *y = x + t;
        for (uint32_t j = 0; j < t; j++) {
          uint64_t u = x[j];
          u -= (u >= q2) ? q2 : 0;
          const uint64_t v = mul_lazy(y[j], w, ws, q);
          x[j] = u + v;
          y[j] = u + q2 - v;
        }
      }
    }
    for (uint32_t i = 0; i < kN; i++) {
      uint64_t r = a[i];
      r -= (r >= q2) ? q2 : 0;
      a[i] = r - ((r >= q) ? q : 0);
    }
  }
  void inverse(uint64_t *a) const {  // inputs < 2q
    const uint64_t q2 = 2 * q;
    for (uint32_t m = kN >> 1, t = 1; m >= 1; m >>= 1, t <<= 1) {
      for (uint32_t i = 0; i < m; i++) {
        const uint64_t w = inv[m + i], ws = inv_s[m + i];
        uint64_t *x = a + 2 * i * t, *y = x + t;
        for (uint32_t j = 0; j < t; j++) {
          const uint64_t u = x[j], v = y[j];
          uint64_t s = u + v;
          x[j] = s - ((s >= q2) ? q2 : 0);
          y[j] = mul_lazy(u + q2 - v, w, ws, q);
        }
      }
    }
    for (uint32_t i = 0; i < kN; i++) {
      const uint64_t r = mul_lazy(a[i], n_inv, n_inv_s, q);
      a[i] = r - ((r >= q) ? q : 0);
    }
  }
};

struct Tables {
  Ntt q, p, small_q;
  Tables(uint64_t mq, uint64_t mp, uint64_t msq) : q(mq), p(mp), small_q(msq) {}
};

// one table set per (q, p, small_q), shared by every client of those moduli
inline std::shared_ptr<const Tables> tables_for(uint64_t q, uint64_t p, uint64_t small_q) {
  static std::mutex mu;
  static std::map<std::tuple<uint64_t, uint64_t, uint64_t>, std::weak_ptr<const Tables>> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto &slot = cache[std::make_tuple(q, p, small_q)];
  if (auto t = slot.lock()) return t;
  auto t = std::make_shared<const Tables>(q, p, small_q);
  slot = t;
  return t;
}

inline uint64_t addmod(uint64_t a, uint64_t b, uint64_t q) {
  const uint64_t s = a + b;
  return s >= q ? s - q : s;
}
inline uint64_t negmod(uint64_t a, uint64_t q) { return a ? q - a : 0; }
inline uint64_t signed_mod(int64_t v, uint64_t q) {
  return v >= 0 ? (uint64_t)v % q : negmod((uint64_t)(-v) % q, q);
}

}  // namespace client_detail

class PirClient {
 public:
  static constexpr uint32_t N = client_detail::kN;

  // A client with a fresh ternary secret key from operating-system entropy.
  PirClient(const PirParams &params, size_t client_id) : PirClient(params, client_id, NoKey{}) {
    ChaChaStream r = ChaChaStream::from_os();
    keygen(r);
  }
  // A client whose secret key is derived from `secret_seed` (reproducible,
  // not secure: tests and benchmarks).
  PirClient(const PirParams &params, size_t client_id, uint64_t secret_seed)
      : PirClient(params, client_id, NoKey{}) {
    SeededStream r(secret_seed ^ kTagSecret);
    keygen(r);
  }

  size_t get_client_id() const { return client_id_; }
  const PirParams &params() const { return P_; }
  const std::vector<int8_t> &secret_key() const { return sk_; }  // coefficients in {-1, 0, 1}

  // client.cpp:33-35
  size_t get_database_plain_index(size_t entry_index) const {
    return entry_index / P_.entries_per_pt;
  }
  // client.cpp:38-53: digit of the first dimension, then one bit per further
  // dimension, most significant first
  std::vector<size_t> get_query_indices(size_t plaintext_index) const {
    std::vector<size_t> idx{plaintext_index % P_.fst_dim_sz};
    size_t row = plaintext_index / P_.fst_dim_sz, remain = P_.other_dim_sz;
    for (uint32_t i = 1; i < P_.ndim(); i++) {
      remain /= 2;
      idx.push_back(row / remain);
      row %= remain;
    }
    return idx;
  }

  // fast_generate_query + add_gsw_to_query (client.cpp:130-209): a BFV
  // encryption of Delta * 2^-h at slot brv(idx0, h), plus for every further
  // dimension whose bit is 1 the gadget values B^(l-1-k) * 2^-h mod q at
  // slots brv(n1 + (i-1) l + k, h).
  Ciphertext fast_generate_query(size_t entry_index) const {
    ChaChaStream r = ChaChaStream::from_os();
    return make_query(r, entry_index);
  }
  Ciphertext fast_generate_query(size_t entry_index, uint64_t seed) const {
    SeededStream r(seed ^ kTagQuery);
    return make_query(r, entry_index);
  }

  // create_galois_keys (client.cpp:227-241) for the elements N/2^a + 1,
  // a < expansion height; layout [h][2][2][N], NTT form:
  //   k1 = a,  k0 = -a s + e + [modulus q] (p mod q) sigma_g(s).
  std::vector<uint64_t> create_galois_keys() const {
    ChaChaStream r = ChaChaStream::from_os();
    return galois_keys(r);
  }
  std::vector<uint64_t> create_galois_keys(uint64_t seed) const {
    SeededStream r(seed ^ kTagGalois);
    return galois_keys(r);
  }

  // generate_gsw_from_key (client.cpp:17-31, gsw_eval.cpp:339-405): RGSW(s)
  // under the key gadget B_key^(l_key-1-j); rows j < l_key carry g_j s in
  // c0, rows j >= l_key in c1.  Layout [2 l_key][2][N], coefficient form.
  std::vector<uint64_t> generate_gsw_from_key() const {
    ChaChaStream r = ChaChaStream::from_os();
    return gsw_key(r);
  }
  std::vector<uint64_t> generate_gsw_from_key(uint64_t seed) const {
    SeededStream r(seed ^ kTagGsw);
    return gsw_key(r);
  }

  // load_resp_from_stream (client.cpp:364-412): 2N coefficients of
  // ceil(log2 small_q) bits, LSB first in every byte.
  Ciphertext load_resp_from_stream(std::istream &stream) const {
    std::vector<uint8_t> bytes(response_bytes());
    if (!stream.read(reinterpret_cast<char *>(bytes.data()), (std::streamsize)bytes.size()))
      throw std::runtime_error("unexpected end of response stream");
    return unpack_response(bytes.data());
  }
  Ciphertext unpack_response(const uint8_t *bytes) const {
    const uint32_t w = PirParams::bitlen(P_.small_q);
    Ciphertext ct(2 * N);
    uint64_t bit = 0;
    for (uint32_t i = 0; i < 2 * N; i++) {
      uint64_t v = 0;
      for (uint32_t j = 0; j < w; j++, bit++) v |= (uint64_t)((bytes[bit >> 3] >> (bit & 7)) & 1) << j;
      ct[i] = v;
    }
    return ct;
  }
  size_t response_bytes() const { return ((size_t)2 * N * PirParams::bitlen(P_.small_q) + 7) / 8; }

  // decrypt_mod_q (client.cpp:415-479): round(t (c0 + c1 s) / small_q) mod t,
  // the secret key taken to small_q (sk_mod_switch, client.cpp:482-512).
  // `noise_budget`, if given, receives bitlen(small_q) - bitlen(|t·phase|) - 1.
  Plaintext decrypt_mod_q(const Ciphertext &ct, int *noise_budget = nullptr) const {
    return decrypt(ct, T_->small_q, sk_small_q_, noise_budget);
  }
  // decrypt_ct: the same at the ciphertext modulus q (an unswitched response)
  Plaintext decrypt_ct(const Ciphertext &ct, int *noise_budget = nullptr) const {
    return decrypt(ct, T_->q, sk_q_, noise_budget);
  }
  Plaintext decrypt_reply(const Ciphertext &reply, int *noise_budget = nullptr) const {
    return decrypt_mod_q(reply, noise_budget);
  }

  // get_entry_from_plaintext (client.cpp:255-287): entry_size bytes read
  // LSB first from bits_per_coeff-bit coefficients.
  Entry get_entry_from_plaintext(size_t entry_index, const Plaintext &plain) const {
    const uint64_t bpc = P_.bits_per_coeff;
    const uint64_t start = (entry_index % P_.entries_per_pt) * (uint64_t)P_.entry_size * 8;
    uint64_t ci = start / bpc;
    client_detail::u128 buf = plain[ci] >> (start % bpc);
    uint64_t have = bpc - start % bpc;
    Entry out(P_.entry_size);
    for (size_t n = 0; n < out.size();) {
      if (have >= 8) {
        out[n++] = (uint8_t)(buf & 0xFF);
        buf >>= 8;
        have -= 8;
      } else {
        ci++;
        buf |= (client_detail::u128)(ci < N ? plain[ci] : 0) << have;
        have += bpc;
      }
    }
    return out;
  }

 private:
  static constexpr uint64_t kTagSecret = 0x5EC12E7ULL, kTagGalois = 0x6A101500ULL,
                            kTagGsw = 0x65500000ULL, kTagQuery = 0x90E2700ULL;

  struct NoKey {};
  PirClient(const PirParams &params, size_t client_id, NoKey) : P_(params), client_id_(client_id) {
    if (P_.poly_degree != N) throw std::invalid_argument("poly_degree must be 2048");
    if (!P_.q || !P_.p || !P_.t || !P_.small_q || !P_.fst_dim_sz || !P_.other_dim_sz)
      throw std::invalid_argument("incomplete PirParams");
    T_ = client_detail::tables_for(P_.q, P_.p, P_.small_q);
  }

  template <class Rng>
  void keygen(Rng &r) {
    using namespace client_detail;
    sk_.resize(N);
    for (uint32_t i = 0; i < N; i++) sk_[i] = (int8_t)((int)(r.next() % 3) - 1);
    sk_q_.resize(N);
    sk_p_.resize(N);
    sk_small_q_.resize(N);
    for (uint32_t i = 0; i < N; i++) {
      sk_q_[i] = signed_mod(sk_[i], P_.q);
      sk_p_[i] = signed_mod(sk_[i], P_.p);
      sk_small_q_[i] = signed_mod(sk_[i], P_.small_q);
    }
    T_->q.forward(sk_q_.data());
    T_->p.forward(sk_p_.data());
    T_->small_q.forward(sk_small_q_.data());
  }

  // (-a s + e, a) mod q in coefficient form: N uniform draws for a, then N
  // error draws (SEAL encrypt_zero_symmetric semantics)
  template <class Rng>
  void enc_zero(Rng &r, uint64_t *ct) const {
    using namespace client_detail;
    const uint64_t q = P_.q;
    uint64_t *c0 = ct, *c1 = ct + N;
    for (uint32_t i = 0; i < N; i++) c1[i] = uniform(r, q);
    std::memcpy(c0, c1, N * 8);
    T_->q.forward(c0);
    for (uint32_t i = 0; i < N; i++) c0[i] = PirParams::mulmod(c0[i], sk_q_[i], q);
    T_->q.inverse(c0);
    for (uint32_t i = 0; i < N; i++) c0[i] = addmod(negmod(c0[i], q), signed_mod(cbd(r), q), q);
  }

  template <class Rng>
  Ciphertext make_query(Rng &r, size_t entry_index) const {
    using namespace client_detail;
    const uint64_t q = P_.q, t = P_.t;
    const uint32_t h = P_.expan_height();
    const uint64_t pt = get_database_plain_index(entry_index);
    if (pt >= P_.num_pt()) throw std::invalid_argument("entry index out of range");
    const std::vector<size_t> idx = get_query_indices(pt);
    Ciphertext ct(2 * N);
    enc_zero(r, ct.data());
    const uint64_t w = 1ull << h;
    const uint64_t inv_t = PirParams::powmod(w % t, t - 2, t);
    const uint64_t delta_m = (uint64_t)(((u128)q * inv_t + t / 2) / t);  // round(q m / t)
    const uint64_t slot = brv(idx[0], h);
    ct[slot] = addmod(ct[slot], delta_m % q, q);
    const uint64_t inv_q = PirParams::powmod(w % q, q - 2, q);
    uint64_t g = 1;  // B^(l-1-k), k = l-1 .. 0
    std::vector<uint64_t> gadget(P_.l);
    for (int k = (int)P_.l - 1; k >= 0; k--) {
      gadget[k] = g;
      g = (uint64_t)(((u128)g << P_.base_log2) % q);
    }
    for (uint32_t i = 1; i < idx.size(); i++) {
      if (idx[i] != 1) continue;
      for (uint32_t k = 0; k < P_.l; k++) {
        const uint64_t s = brv(P_.fst_dim_sz + (uint64_t)(i - 1) * P_.l + k, h);
        ct[s] = addmod(ct[s], PirParams::mulmod(gadget[k], inv_q, q), q);
      }
    }
    return ct;
  }

  template <class Rng>
  std::vector<uint64_t> galois_keys(Rng &r) const {
    using namespace client_detail;
    const uint32_t h = P_.expan_height();
    std::vector<uint64_t> keys((size_t)h * 4 * N);
    std::vector<int64_t> e(N), sg(N);
    std::vector<uint64_t> em(N), sgm(N);
    const uint64_t f = P_.p % P_.q;
    for (uint32_t lv = 0; lv < h; lv++) {
      const uint64_t g = 1 + (N >> lv);
      for (uint64_t i = 0; i < N; i++) {  // sigma_g(s): x^i -> x^(i g) mod x^N + 1
        const uint64_t j = (i * g) & (2 * N - 1);
        if (j < N)
          sg[j] = sk_[i];
        else
          sg[j - N] = -sk_[i];
      }
      for (uint32_t i = 0; i < N; i++) e[i] = cbd(r);
      for (int m = 0; m < 2; m++) {
        const Ntt &T = m == 0 ? T_->q : T_->p;
        const uint64_t mod = T.q;
        const std::vector<uint64_t> &s = m == 0 ? sk_q_ : sk_p_;
        uint64_t *k0 = keys.data() + ((size_t)(lv * 2 + 0) * 2 + m) * N;
        uint64_t *k1 = keys.data() + ((size_t)(lv * 2 + 1) * 2 + m) * N;
        for (uint32_t i = 0; i < N; i++) em[i] = signed_mod(e[i], mod);
        T.forward(em.data());
        for (uint32_t i = 0; i < N; i++) k1[i] = uniform(r, mod);
        for (uint32_t i = 0; i < N; i++)
          k0[i] = addmod(negmod(PirParams::mulmod(k1[i], s[i], mod), mod), em[i], mod);
        if (m == 0) {
          for (uint32_t i = 0; i < N; i++) sgm[i] = signed_mod(sg[i], mod);
          T.forward(sgm.data());
          for (uint32_t i = 0; i < N; i++)
            k0[i] = addmod(k0[i], PirParams::mulmod(f, sgm[i], mod), mod);
        }
      }
    }
    return keys;
  }

  template <class Rng>
  std::vector<uint64_t> gsw_key(Rng &r) const {
    using namespace client_detail;
    const uint64_t q = P_.q;
    std::vector<uint64_t> rows((size_t)2 * P_.l_key * 2 * N);
    std::vector<uint64_t> gadget(P_.l_key);
    uint64_t g = 1;
    for (int j = (int)P_.l_key - 1; j >= 0; j--) {
      gadget[j] = g;
      g = (uint64_t)(((u128)g << P_.base_log2_key) % q);
    }
    for (uint32_t j = 0; j < 2 * P_.l_key; j++) {
      uint64_t *ct = rows.data() + (size_t)j * 2 * N;
      enc_zero(r, ct);
      uint64_t *dst = ct + (size_t)(j / P_.l_key) * N;
      const uint64_t gj = gadget[j % P_.l_key];
      for (uint32_t i = 0; i < N; i++)
        dst[i] = addmod(dst[i], PirParams::mulmod(gj, signed_mod(sk_[i], q), q), q);
    }
    return rows;
  }

  Plaintext decrypt(const Ciphertext &ct, const client_detail::Ntt &T,
                    const std::vector<uint64_t> &s_ntt, int *noise_budget) const {
    using namespace client_detail;
    if (ct.size() != 2 * N) throw std::invalid_argument("ciphertext must hold 2 N coefficients");
    const uint64_t Q = T.q, t = P_.t;
    std::vector<uint64_t> ph(N);
    for (uint32_t i = 0; i < N; i++) ph[i] = ct[N + i] % Q;
    T.forward(ph.data());
    for (uint32_t i = 0; i < N; i++) ph[i] = PirParams::mulmod(ph[i], s_ntt[i], Q);
    T.inverse(ph.data());
    Plaintext plain(N);
    uint64_t norm = 0;
    for (uint32_t i = 0; i < N; i++) {
      const uint64_t v = addmod(ph[i], ct[i] % Q, Q);
      plain[i] = (uint64_t)((((u128)v * t) + Q / 2) / Q) % t;
      const uint64_t n = PirParams::mulmod(v, t, Q), a = n > Q / 2 ? Q - n : n;
      if (a > norm) norm = a;
    }
    if (noise_budget) {
      const int b = (int)PirParams::bitlen(Q) - (int)PirParams::bitlen(norm) - 1;
      *noise_budget = b > 0 ? b : 0;
    }
    return plain;
  }

  PirParams P_;
  size_t client_id_;
  std::shared_ptr<const client_detail::Tables> T_;
  std::vector<int8_t> sk_;
  std::vector<uint64_t> sk_q_, sk_p_, sk_small_q_;  // NTT form
};

}  // namespace onionpir
