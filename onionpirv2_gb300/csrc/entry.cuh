// entry.cuh -- device helpers shared by the single- and multi-modulus paths:
// the x87 modulus switch of mod_switch_inplace (server.cpp:779-801) and the
// seeded synthetic entries of gen_data (utils.cpp:160-172).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace opir {

// (uint64_t)round((long double)x * scale) with the x87 semantics, where
// scale = (double)small_q / (double)q == mant * 2^-shift: the exact product
// x * mant rounded to a 64-bit significand (nearest-even), then scaled by
// 2^-shift and rounded half away from zero.
__device__ __forceinline__ uint64_t mod_switch_x87(uint64_t x, uint64_t mant, int shift) {
  if (x == 0) return 0;
  unsigned __int128 P = (unsigned __int128)x * mant;
  const uint64_t hi = (uint64_t)(P >> 64);
  const int bits = hi ? 128 - __clzll((long long)hi) : 64 - __clzll((long long)(uint64_t)P);
  if (bits > 64) {
    const int sh = bits - 64;
    unsigned __int128 keep = P >> sh;
    const unsigned __int128 rem = P & ((((unsigned __int128)1) << sh) - 1);
    const unsigned __int128 half = ((unsigned __int128)1) << (sh - 1);
    if (rem > half || (rem == half && (keep & 1))) keep += 1;
    P = keep << sh;
  }
  return (uint64_t)((P + (((unsigned __int128)1) << (shift - 1))) >> shift);
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// byte j of synthetic entry e: 8-byte big-endian index, then seeded bytes
__device__ __forceinline__ uint32_t gen_entry_byte(uint64_t seed, uint64_t e, uint64_t j) {
  if (j < 8) return (uint32_t)((e >> (8 * (7 - j))) & 0xFF);
  const uint64_t w = mix64(seed * 0x9E3779B97F4A7C15ULL + e * 0xD1B54A32D192ED03ULL + ((j - 8) >> 3));
  return (uint32_t)((w >> (8 * ((j - 8) & 7))) & 0xFF);
}

}  // namespace opir
