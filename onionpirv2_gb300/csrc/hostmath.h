// hostmath.h -- host-side number theory shared by the context set-up of the
// single- and multi-modulus paths: modular products, primality, the NTT
// root SEAL builds its tables on, bit reversal and Shoup companions.
#pragma once

#include <cstdint>

namespace opir {
namespace hostmath {

using u128 = unsigned __int128;

inline uint64_t mulmod(uint64_t a, uint64_t b, uint64_t q) { return (uint64_t)(((u128)a * b) % q); }
inline uint64_t powmod(uint64_t b, uint64_t e, uint64_t q) {
  uint64_t r = 1 % q;
  b %= q;
  while (e) {
    if (e & 1) r = mulmod(r, b, q);
    b = mulmod(b, b, q);
    e >>= 1;
  }
  return r;
}
// deterministic Miller-Rabin for 64-bit n
inline bool is_prime(uint64_t n) {
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
inline uint64_t shoup(uint64_t w, uint64_t q) { return (uint64_t)(((u128)w << 64) / q); }
inline unsigned bitlen(uint64_t x) { return x ? 64 - __builtin_clzll(x) : 0; }
inline uint64_t brv(uint64_t x, unsigned bits) {
  uint64_t y = 0;
  for (unsigned i = 0; i < bits; i++) y = (y << 1) | ((x >> i) & 1);
  return y;
}
// smallest primitive two_n-th root of unity mod q (0 if there is none)
inline uint64_t minimal_root(uint64_t q, uint64_t two_n) {
  if ((q - 1) % two_n) return 0;
  const uint64_t cof = (q - 1) / two_n;
  uint64_t psi = 0;
  for (uint64_t g = 2; g < q && !psi; g++) {
    const uint64_t c = powmod(g, cof, q);
    if (powmod(c, two_n / 2, q) == q - 1) psi = c;
  }
  if (!psi) return 0;
  uint64_t best = psi, cur = psi;
  const uint64_t sq = mulmod(psi, psi, q);
  for (uint64_t k = 1; k < two_n / 2; k++) {
    cur = mulmod(cur, sq, q);
    if (cur < best) best = cur;
  }
  return best;
}

}  // namespace hostmath
}  // namespace opir
