// onionpir_params.hpp -- the parameter set of the C++ PirServer / PirClient
// (header-only, no GPU): PirParams::PirParams (src/pir.cpp:9-112,
// src/includes/pir.h:18-86) for the N = 2048, CoeffMods = {60, 60} presets of
// src/includes/database_constants.h.  Prime selection follows SEAL's
// CoeffModulus::Create (the largest primes below 2^bits that are 1 mod 2N, in
// descending order) and utils::generate_prime (utils.cpp:82-95).
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <vector>

namespace onionpir {

using Ciphertext = std::vector<uint64_t>;  // [2][N], coefficient form
using Entry = std::vector<uint8_t>;
// One RGSW ciphertext (GSWCiphertext, gsw_eval.h:8): 2l rows [row][2][N]
// flattened, NTT form.
using GSWCiphertext = std::vector<uint64_t>;

struct PirParams {
  uint64_t q = 0, p = 0, t = 0, small_q = 0;  // CoeffModulus::Create / generate_prime results
  uint32_t poly_degree = 2048;
  uint32_t l = 5, base_log2 = 12, l_key = 10, base_log2_key = 6;
  uint32_t fst_dim_sz = 0, other_dim_sz = 0;  // PirParams::get_dims()
  uint32_t entry_size = 0, entries_per_pt = 1, bits_per_coeff = 15;

  uint64_t num_pt() const { return (uint64_t)fst_dim_sz * other_dim_sz; }
  uint32_t ndim() const {  // 1 + floor(log2(other_dim_sz)), pir.cpp:89
    uint32_t d = 1;
    while ((2ull << (d - 1)) <= other_dim_sz) d++;
    return d;
  }
  uint32_t expan_height() const {  // pir.h:66-68
    const uint64_t u = fst_dim_sz + (uint64_t)l * (ndim() - 1);
    uint32_t h = 0;
    while ((1ull << h) < u) h++;
    return h;
  }

  // The reference's derivation for `num_entries` entries and a first
  // dimension of at most `max_fst_dim` (DatabaseConstants defaults: GSW_L 5,
  // GSW_L_KEY 10, 16-bit plaintext modulus, 27-bit small_q, entries filling a
  // plaintext when entry_size is 0).
  static PirParams derive(uint64_t num_entries, uint64_t max_fst_dim, uint32_t entry_size = 0,
                          uint32_t l = 5, uint32_t l_key = 10) {
    PirParams P;
    const uint64_t n = P.poly_degree;
    P.t = generate_prime(16);                      // pir.cpp:18
    P.q = ntt_prime(60, n, 0);                     // pir.cpp:22-23
    P.p = ntt_prime(60, n, 1);
    P.small_q = ntt_prime(27, n, 0);               // pir.cpp:40-41
    P.bits_per_coeff = bitlen(P.t) - 1;
    P.entry_size = entry_size ? entry_size : (uint32_t)(P.bits_per_coeff * n / 8);  // pir.cpp:34-38
    P.entries_per_pt = (uint32_t)(P.bits_per_coeff * n / ((uint64_t)P.entry_size * 8));
    if (!P.entries_per_pt) throw std::invalid_argument("entry does not fit a plaintext");
    P.l = l;
    P.l_key = l_key;
    P.base_log2 = (bitlen(P.q) + l - 1) / l;              // pir.cpp:53
    P.base_log2_key = (bitlen(P.q) + l_key - 1) / l_key;  // pir.cpp:54
    const uint64_t need = (num_entries + P.entries_per_pt - 1) / P.entries_per_pt;  // pir.cpp:67
    uint64_t pow2 = 1;
    while (pow2 < need) pow2 <<= 1;
    const uint64_t other = (pow2 + max_fst_dim - 1) / max_fst_dim;  // pir.cpp:70
    const uint64_t first = (need + other - 1) / other;              // pir.cpp:72
    P.fst_dim_sz = (uint32_t)first;
    P.other_dim_sz = (uint32_t)other;
    return P;
  }

  static uint32_t bitlen(uint64_t x) {
    uint32_t b = 0;
    while (x) b++, x >>= 1;
    return b;
  }
  static uint64_t mulmod(uint64_t a, uint64_t b, uint64_t m) {
    return (uint64_t)((unsigned __int128)a * b % m);
  }
  static uint64_t powmod(uint64_t b, uint64_t e, uint64_t m) {
    uint64_t r = 1 % m;
    b %= m;
    for (; e; e >>= 1) {
      if (e & 1) r = mulmod(r, b, m);
      b = mulmod(b, b, m);
    }
    return r;
  }
  static bool is_prime(uint64_t n) {
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
      bool composite = true;
      for (int r = 1; r < s && composite; r++) {
        x = mulmod(x, x, n);
        composite = x != n - 1;
      }
      if (composite) return false;
    }
    return true;
  }
  // utils::generate_prime: the first prime reached from 2^(bits-1) by ++ and |= 1
  static uint64_t generate_prime(uint32_t bits) {
    uint64_t c = 1ull << (bits - 1);
    for (;;) {
      c = (c + 1) | 1;
      if (is_prime(c)) return c;
    }
  }
  // the (rank+1)-th largest prime below 2^bits that is 1 mod 2n
  static uint64_t ntt_prime(uint32_t bits, uint64_t n, int rank) {
    for (uint64_t v = (1ull << bits) - 2 * n + 1; v > (1ull << (bits - 1)); v -= 2 * n)
      if (is_prime(v) && rank-- == 0) return v;
    throw std::invalid_argument("no NTT prime of that size");
  }
};

}  // namespace onionpir
