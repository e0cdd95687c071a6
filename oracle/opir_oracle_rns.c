/*
 * opir_oracle_rns.c -- CPU oracle of the multi-modulus OnionPIRv2 server
 * path (R = 1 or 2 ciphertext primes, any power-of-two N up to 4096).
 *
 * TEST INFRASTRUCTURE ONLY (see opir_oracle_rns.h for the parity status).
 * Every function names the reference code it restates; the SEAL primitives
 * (RNS NTTs, Galois automorphism with RNS key switching, CRT composition,
 * divide-and-round by the last prime, BFV encryption) are restated from the
 * mathematics of BFV/RGSW and the public description of SEAL 4.1.  The
 * seeded randomness and its draw order are those of opir_oracle.c, so that
 * at N = 2048, R = 1 both oracles give the same keys, queries and responses.
 */
#include "opir_oracle_rns.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

#define MAXM (ORR_MAX_RNS + 2) /* data primes, p, small_q */

/* ------------------------------------------------------------------------ */
/* modular arithmetic                                                        */
/* ------------------------------------------------------------------------ */

static inline uint64_t mulmod(uint64_t a, uint64_t b, uint64_t q) {
  return (uint64_t)(((u128)a * b) % q);
}
static uint64_t powmod(uint64_t b, uint64_t e, uint64_t q) {
  uint64_t r = 1 % q;
  b %= q;
  while (e) {
    if (e & 1) r = mulmod(r, b, q);
    b = mulmod(b, b, q);
    e >>= 1;
  }
  return r;
}
static inline uint64_t addmod(uint64_t a, uint64_t b, uint64_t q) {
  uint64_t s = a + b;
  return s >= q ? s - q : s;
}
static inline uint64_t submod(uint64_t a, uint64_t b, uint64_t q) { return a >= b ? a - b : a + q - b; }
static inline uint64_t negmod(uint64_t a, uint64_t q) { return a ? q - a : 0; }
static inline uint64_t shoup(uint64_t w, uint64_t q) { return (uint64_t)(((u128)w << 64) / q); }
static inline uint64_t mul_shoup(uint64_t x, uint64_t w, uint64_t ws, uint64_t q) {
  uint64_t hq = (uint64_t)(((u128)x * ws) >> 64);
  uint64_t r = x * w - hq * q;
  return r >= q ? r - q : r;
}
static unsigned bitlen64(uint64_t x) { return x ? 64 - (unsigned)__builtin_clzll(x) : 0; }
static unsigned bitlen128(u128 x) {
  uint64_t hi = (uint64_t)(x >> 64);
  return hi ? 64 + bitlen64(hi) : bitlen64((uint64_t)x);
}
static uint64_t brv(uint64_t x, unsigned bits) {
  uint64_t y = 0;
  for (unsigned i = 0; i < bits; i++) {
    y = (y << 1) | (x & 1);
    x >>= 1;
  }
  return y;
}
static uint64_t next_pow2(uint64_t n) {
  uint64_t p = 1;
  while (p < n) p <<= 1;
  return p;
}
static uint64_t roundup_div(uint64_t a, uint64_t b) { return (a + b - 1) / b; }
static unsigned ceil_log2(uint64_t x) {
  unsigned c = 0;
  while ((1ULL << c) < x) c++;
  return c;
}

static int is_prime(uint64_t n) {
  static const uint64_t bases[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
  if (n < 2) return 0;
  for (size_t i = 0; i < 12; i++) {
    if (n == bases[i]) return 1;
    if (n % bases[i] == 0) return 0;
  }
  uint64_t d = n - 1;
  int s = 0;
  while (!(d & 1)) d >>= 1, s++;
  for (size_t i = 0; i < 12; i++) {
    uint64_t x = powmod(bases[i], d, n);
    if (x == 1 || x == n - 1) continue;
    int comp = 1;
    for (int r = 1; r < s && comp; r++) {
      x = mulmod(x, x, n);
      if (x == n - 1) comp = 0;
    }
    if (comp) return 0;
  }
  return 1;
}

/* utils::generate_prime (utils.cpp:82-95) */
static uint64_t generate_prime(uint64_t bits) {
  uint64_t c = 1ULL << (bits - 1);
  do {
    c++;
    c |= 1;
  } while (!is_prime(c));
  return c;
}

/* SEAL CoeffModulus::Create(n, bit_sizes) (pir.cpp:23,40): per bit size, the
 * largest primes below 2^b that are 1 mod 2n, in descending order. */
static int coeff_modulus_create(uint64_t n, const uint64_t *bits, size_t count, uint64_t *out) {
  for (size_t i = 0; i < count; i++) {
    size_t rank = 0;
    for (size_t j = 0; j < i; j++) rank += bits[j] == bits[i];
    const uint64_t b = bits[i], step = 2 * n, lower = 1ULL << (b - 1);
    uint64_t v = (b == 64 ? 0 : (1ULL << b)) - step + 1;
    size_t found = 0;
    for (;;) {
      if (v <= lower) return -1;
      if (is_prime(v)) {
        if (found == rank) break;
        found++;
      }
      v -= step;
    }
    out[i] = v;
  }
  return 0;
}

/* smallest primitive 2n-th root of unity mod q */
static uint64_t minimal_root(uint64_t q, uint64_t two_n) {
  const uint64_t cof = (q - 1) / two_n;
  uint64_t psi = 0;
  for (uint64_t g = 2; g < q && !psi; g++) {
    uint64_t c = powmod(g, cof, q);
    if (powmod(c, two_n / 2, q) == q - 1) psi = c;
  }
  if (!psi) return 0;
  uint64_t best = psi, sq = mulmod(psi, psi, q), cur = psi;
  for (uint64_t k = 1; k < two_n / 2; k++) {
    cur = mulmod(cur, sq, q);
    if (cur < best) best = cur;
  }
  return best;
}

/* ------------------------------------------------------------------------ */
/* NTT per prime (SEAL ntt_negacyclic_harvey ordering: A[k] = a(psi^(2brv(k)+1))) */
/* ------------------------------------------------------------------------ */

typedef struct {
  uint64_t q, psi, n_inv, n_inv_s;
  uint64_t *fwd, *fwd_s, *inv, *inv_s; /* psi^brv(i), psi^-brv(i), Shoup companions */
  u128 two128; /* 2^128 mod q */
} rntt_t;

static void rntt_init(rntt_t *T, uint64_t q, uint64_t n, unsigned logn) {
  T->q = q;
  T->psi = minimal_root(q, 2 * n);
  T->fwd = (uint64_t *)malloc(4 * n * sizeof(uint64_t));
  T->fwd_s = T->fwd + n;
  T->inv = T->fwd + 2 * n;
  T->inv_s = T->fwd + 3 * n;
  const uint64_t psi_inv = powmod(T->psi, q - 2, q);
  for (uint64_t i = 0; i < n; i++) {
    const uint64_t e = brv(i, logn);
    T->fwd[i] = powmod(T->psi, e, q);
    T->inv[i] = powmod(psi_inv, e, q);
    T->fwd_s[i] = shoup(T->fwd[i], q);
    T->inv_s[i] = shoup(T->inv[i], q);
  }
  T->n_inv = powmod(n % q, q - 2, q);
  T->n_inv_s = shoup(T->n_inv, q);
  const uint64_t t64 = (uint64_t)(((u128)1 << 64) % q);
  T->two128 = mulmod(t64, t64, q);
}

static void rntt_fwd1(const rntt_t *T, uint64_t n, uint64_t *a) {
  const uint64_t q = T->q;
  size_t t = n;
  for (size_t m = 1; m < n; m <<= 1) {
    t >>= 1;
    for (size_t i = 0; i < m; i++) {
      const uint64_t w = T->fwd[m + i], ws = T->fwd_s[m + i];
      uint64_t *x = a + 2 * i * t, *y = x + t;
      for (size_t j = 0; j < t; j++) {
        const uint64_t u = x[j], v = mul_shoup(y[j], w, ws, q);
        x[j] = addmod(u, v, q);
        y[j] = submod(u, v, q);
      }
    }
  }
}

static void rntt_inv1(const rntt_t *T, uint64_t n, uint64_t *a) {
  const uint64_t q = T->q;
  size_t t = 1;
  for (size_t m = n >> 1; m >= 1; m >>= 1) {
    for (size_t i = 0; i < m; i++) {
      const uint64_t w = T->inv[m + i], ws = T->inv_s[m + i];
      uint64_t *x = a + 2 * i * t, *y = x + t;
      for (size_t j = 0; j < t; j++) {
        const uint64_t u = x[j], v = y[j];
        x[j] = addmod(u, v, q);
        y[j] = mul_shoup(submod(u, v, q), w, ws, q);
      }
    }
    t <<= 1;
  }
  for (size_t i = 0; i < n; i++) a[i] = mul_shoup(a[i], T->n_inv, T->n_inv_s, q);
}

/* ------------------------------------------------------------------------ */
/* context                                                                    */
/* ------------------------------------------------------------------------ */

struct orr_ctx {
  orr_params P;
  rntt_t nt[MAXM];                     /* q_0 .. q_{R-1}, p, small_q */
  uint64_t gadget[ORR_MAX_RNS][64];    /* B^(l-1-j) mod q_i (utils.cpp:61-74) */
  uint64_t gadget_key[ORR_MAX_RNS][64];
  uint64_t p_inv[ORR_MAX_RNS];         /* p^-1 mod q_i */
  uint64_t last_inv[ORR_MAX_RNS];      /* q_{R-1}^-1 mod q_i */
  uint64_t delta[ORR_MAX_RNS];         /* floor(Q / t) mod q_i */
  uint64_t q_mod_t;                    /* Q mod t */
};

#define NN (ctx->P.n)
#define RR (ctx->P.rns)

orr_ctx *orr_create(uint64_t n, uint64_t num_entries, uint64_t max_fst_dim, uint64_t entry_size,
                    uint64_t l, uint64_t l_key, uint64_t plain_bits, uint64_t small_q_width,
                    const uint64_t *coeff_bits, uint64_t coeff_count) {
  if (coeff_count < 2 || coeff_count > ORR_MAX_RNS + 1 || n < 16 || n > 4096 || (n & (n - 1)) ||
      !l || !l_key || l > 64 || l_key > 64 || !max_fst_dim)
    return NULL;
  orr_ctx *c = (orr_ctx *)calloc(1, sizeof(orr_ctx));
  if (!c) return NULL;
  orr_params *P = &c->P;
  P->n = n;
  P->logn = ceil_log2(n);
  P->rns = coeff_count - 1;
  uint64_t mods[ORR_MAX_RNS + 1];
  if (coeff_modulus_create(n, coeff_bits, coeff_count, mods)) goto fail; /* pir.cpp:22-23 */
  for (uint64_t i = 0; i < P->rns; i++) P->q[i] = mods[i];
  P->p = mods[P->rns];
  P->t = generate_prime(plain_bits); /* pir.cpp:18 */
  {
    uint64_t sb[2] = {small_q_width, coeff_bits[coeff_count - 1]}, sq[2];
    if (coeff_modulus_create(n, sb, 2, sq)) goto fail; /* pir.cpp:40-41 */
    P->small_q = sq[0];
  }
  P->small_q_width = (uint64_t)ceil(log2((double)P->small_q)); /* server.cpp:587-588 */
  P->bits_per_coeff = bitlen64(P->t) - 1;
  P->entry_size = entry_size ? entry_size : P->bits_per_coeff * n / 8; /* pir.cpp:34-38 */
  P->entries_per_pt = P->bits_per_coeff * n / (P->entry_size * 8);
  if (!P->entries_per_pt) goto fail;
  P->l = l;
  P->l_key = l_key;
  {
    uint64_t logq = 0; /* the special prime does not count (pir.cpp:46-48) */
    for (uint64_t i = 0; i < P->rns; i++) logq += bitlen64(P->q[i]);
    P->base_log2 = (logq + l - 1) / l;             /* pir.cpp:53 */
    P->base_log2_key = (logq + l_key - 1) / l_key; /* pir.cpp:54 */
    if (P->base_log2 >= 64 || P->base_log2_key >= 64) goto fail;
  }
  {
    const uint64_t need = roundup_div(num_entries, P->entries_per_pt); /* pir.cpp:67 */
    const uint64_t other = roundup_div(next_pow2(need), max_fst_dim); /* pir.cpp:70 */
    const uint64_t first = roundup_div(need, other);                  /* pir.cpp:72 */
    P->num_pt = first * other;
    P->num_entries = P->num_pt * P->entries_per_pt;
    P->n1 = first;
    P->n_rest = other;
    P->ndim = 1 + (uint64_t)log2((double)other); /* pir.cpp:89 */
  }
  P->u = P->n1 + P->l * (P->ndim - 1);
  P->h = ceil_log2(P->u); /* pir.h:66-68 */
  {
    double scale = (double)P->small_q / (double)P->q[0]; /* server.cpp:790-795 */
    int e;
    double m = frexp(scale, &e);
    P->ms_mant = (uint64_t)ldexp(m, 53);
    P->ms_exp = (int64_t)e - 53;
  }
  for (uint64_t i = 0; i < P->rns; i++) rntt_init(&c->nt[i], P->q[i], n, (unsigned)P->logn);
  rntt_init(&c->nt[P->rns], P->p, n, (unsigned)P->logn);
  rntt_init(&c->nt[P->rns + 1], P->small_q, n, (unsigned)P->logn);
  for (uint64_t i = 0; i < P->rns; i++) {
    const uint64_t q = P->q[i];
    u128 pw = 1;
    for (int j = (int)l - 1; j >= 0; j--) {
      c->gadget[i][j] = (uint64_t)pw;
      pw = (pw << P->base_log2) % q;
    }
    pw = 1;
    for (int j = (int)l_key - 1; j >= 0; j--) {
      c->gadget_key[i][j] = (uint64_t)pw;
      pw = (pw << P->base_log2_key) % q;
    }
    c->p_inv[i] = powmod(P->p % q, q - 2, q);
    c->last_inv[i] = powmod(P->q[P->rns - 1] % q, q - 2, q);
  }
  {
    /* Q = prod q_i < 2^120 (R <= 2) */
    u128 Q = 1;
    for (uint64_t i = 0; i < P->rns; i++) Q *= P->q[i];
    const u128 D = Q / P->t;
    c->q_mod_t = (uint64_t)(Q % P->t);
    for (uint64_t i = 0; i < P->rns; i++) c->delta[i] = (uint64_t)(D % P->q[i]);
  }
  return c;
fail:
  free(c);
  return NULL;
}

void orr_destroy(orr_ctx *ctx) {
  if (!ctx) return;
  for (int i = 0; i < MAXM; i++) free(ctx->nt[i].fwd);
  free(ctx);
}
void orr_get_params(const orr_ctx *ctx, orr_params *out) { *out = ctx->P; }

void orr_ntt_fwd(const orr_ctx *ctx, int mod, uint64_t *a, size_t count) {
#pragma omp parallel for schedule(static) if (count > 8)
  for (long i = 0; i < (long)count; i++) rntt_fwd1(&ctx->nt[mod], NN, a + (size_t)i * NN);
}
void orr_ntt_inv(const orr_ctx *ctx, int mod, uint64_t *a, size_t count) {
#pragma omp parallel for schedule(static) if (count > 8)
  for (long i = 0; i < (long)count; i++) rntt_inv1(&ctx->nt[mod], NN, a + (size_t)i * NN);
}

/* forward / inverse NTT of every prime block of `polys` [R] polynomials */
static void rns_fwd(const orr_ctx *ctx, uint64_t *poly) {
  for (uint64_t i = 0; i < RR; i++) rntt_fwd1(&ctx->nt[i], NN, poly + i * NN);
}
static void rns_inv(const orr_ctx *ctx, uint64_t *poly) {
  for (uint64_t i = 0; i < RR; i++) rntt_inv1(&ctx->nt[i], NN, poly + i * NN);
}

/* ------------------------------------------------------------------------ */
/* seeded randomness (the generator and draw order of opir_oracle.c)         */
/* ------------------------------------------------------------------------ */

static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
typedef struct {
  uint64_t s;
} rng_t;
static inline uint64_t rng_next(rng_t *r) { return mix64(r->s += 0x9E3779B97F4A7C15ULL); }
static uint64_t rng_uniform(rng_t *r, uint64_t q) {
  const unsigned b = bitlen64(q);
  for (;;) {
    const uint64_t v = rng_next(r) >> (64 - b);
    if (v < q) return v;
  }
}
static int64_t rng_cbd(rng_t *r) {
  const uint64_t v = rng_next(r);
  return (int64_t)__builtin_popcountll(v & 0x1FFFFF) -
         (int64_t)__builtin_popcountll((v >> 21) & 0x1FFFFF);
}
static inline uint64_t small_mod(int64_t v, uint64_t q) {
  return v >= 0 ? (uint64_t)v % q : negmod((uint64_t)(-v) % q, q);
}

/* ------------------------------------------------------------------------ */
/* database (server.cpp:47-78, 635-748; utils.cpp:98-104, 160-172)          */
/* ------------------------------------------------------------------------ */

void orr_gen_entries(const orr_ctx *ctx, uint64_t seed, uint64_t first, uint64_t count,
                     uint8_t *out) {
  const uint64_t es = ctx->P.entry_size;
#pragma omp parallel for schedule(static) if (count > 64)
  for (long k = 0; k < (long)count; k++) {
    const uint64_t e = first + (uint64_t)k;
    uint8_t *o = out + (size_t)k * es;
    for (int i = 0; i < 8; i++) o[7 - i] = (uint8_t)(e >> (8 * i));
    for (uint64_t j = 8; j < es; j++) {
      const uint64_t w =
          mix64(seed * 0x9E3779B97F4A7C15ULL + e * 0xD1B54A32D192ED03ULL + ((j - 8) >> 3));
      o[j] = (uint8_t)(w >> (8 * ((j - 8) & 7)));
    }
  }
}

/* push_database_chunk byte packing (server.cpp:649-700) */
static void pack_plaintext(const orr_ctx *ctx, const uint8_t *entries, uint64_t *pt) {
  const orr_params *P = &ctx->P;
  const uint64_t bpc = P->bits_per_coeff;
  const u128 mask = ((u128)1 << bpc) - 1;
  memset(pt, 0, NN * sizeof(uint64_t));
  size_t index = 0;
  u128 buf = 0;
  uint64_t off = 0;
  for (uint64_t k = 0; k < P->entries_per_pt * P->entry_size; k++) {
    buf += (u128)entries[k] << off;
    off += 8;
    while (off >= bpc) {
      pt[index++] = (uint64_t)(buf & mask);
      buf >>= bpc;
      off -= bpc;
    }
  }
  if (off > 0) pt[index++] = (uint64_t)(buf & mask);
}

/* gen_data + preprocess_ntt + realign_db (server.cpp:47-78, 703-748).  The
 * plaintext is lifted centred to every prime (v >= (t+1)/2 -> v + q_i - t,
 * SEAL's plain_upper_half_increment) and transformed per prime;
 * db_aligned[(i N + c) num_pt + pt]. */
void orr_build_db(const orr_ctx *ctx, uint64_t seed, uint64_t *db) {
  const orr_params *P = &ctx->P;
  const uint64_t np = P->num_pt, thr = (P->t + 1) >> 1;
#pragma omp parallel for schedule(dynamic, 4)
  for (long pt = 0; pt < (long)np; pt++) {
    uint8_t *ent = (uint8_t *)malloc(P->entries_per_pt * P->entry_size);
    uint64_t *coeffs = (uint64_t *)malloc(NN * 8), *lift = (uint64_t *)malloc(NN * 8);
    orr_gen_entries(ctx, seed, (uint64_t)pt * P->entries_per_pt, P->entries_per_pt, ent);
    pack_plaintext(ctx, ent, coeffs);
    for (uint64_t i = 0; i < RR; i++) {
      const uint64_t inc = P->q[i] - P->t;
      for (uint64_t c = 0; c < NN; c++) lift[c] = coeffs[c] >= thr ? coeffs[c] + inc : coeffs[c];
      rntt_fwd1(&ctx->nt[i], NN, lift);
      for (uint64_t c = 0; c < NN; c++) db[(i * NN + c) * np + (uint64_t)pt] = lift[c];
    }
    free(ent);
    free(coeffs);
    free(lift);
  }
}

/* ------------------------------------------------------------------------ */
/* client (client.cpp)                                                        */
/* ------------------------------------------------------------------------ */

void orr_keygen(const orr_ctx *ctx, uint64_t seed, int8_t *sk) {
  rng_t r = {seed ^ 0x5EC12E7ULL};
  for (uint64_t i = 0; i < NN; i++) sk[i] = (int8_t)((int)(rng_next(&r) % 3) - 1);
}

/* a * b mod (x^N + 1, modulus `mod`), coefficient form */
static void polymul(const orr_ctx *ctx, int mod, const uint64_t *a, const uint64_t *b,
                    uint64_t *out) {
  const rntt_t *T = &ctx->nt[mod];
  uint64_t *A = (uint64_t *)malloc(2 * NN * 8), *B = A + NN;
  memcpy(A, a, NN * 8);
  memcpy(B, b, NN * 8);
  rntt_fwd1(T, NN, A);
  rntt_fwd1(T, NN, B);
  for (uint64_t i = 0; i < NN; i++) A[i] = mulmod(A[i], B[i], T->q);
  rntt_inv1(T, NN, A);
  memcpy(out, A, NN * 8);
  free(A);
}

/* Symmetric RLWE encryption of zero over the ciphertext primes (SEAL
 * encrypt_zero_symmetric): a_i uniform per prime, one error polynomial e,
 * ct[0][i] = -a_i s + e, ct[1][i] = a_i (coefficient form, [2][R][N]). */
static void enc_zero(const orr_ctx *ctx, const int8_t *sk, rng_t *r, uint64_t *ct) {
  const uint64_t n = NN, R = RR;
  uint64_t *s = (uint64_t *)malloc(2 * n * 8), *as = s + n;
  for (uint64_t i = 0; i < R; i++)
    for (uint64_t c = 0; c < n; c++) ct[(R + i) * n + c] = rng_uniform(r, ctx->P.q[i]);
  int64_t *e = (int64_t *)malloc(n * 8);
  for (uint64_t i = 0; i < R; i++) {
    const uint64_t q = ctx->P.q[i];
    for (uint64_t c = 0; c < n; c++) s[c] = small_mod(sk[c], q);
    polymul(ctx, (int)i, ct + (R + i) * n, s, as);
    for (uint64_t c = 0; c < n; c++) {
      if (i == 0) e[c] = rng_cbd(r);
      ct[i * n + c] = addmod(negmod(as[c], q), small_mod(e[c], q), q);
    }
  }
  free(e);
  free(s);
}

/* KeyGenerator::create_galois_keys for elements 1 + (N >> a), a < h
 * (client.cpp:227-241), with SEAL's RNS key-switching key layout: for
 * decomposition prime j and modulus m in {q_0 .. q_{R-1}, p} (NTT form)
 *   k1 = a,  k0 = -a s + e_j + [m == q_j] (p mod q_j) sigma_g(s). */
void orr_make_galois_keys(const orr_ctx *ctx, const int8_t *sk, uint64_t seed, uint64_t *keys) {
  const orr_params *P = &ctx->P;
  const uint64_t n = NN, R = RR, M = R + 1;
  rng_t r = {seed ^ 0x6A101500ULL};
  int64_t *sg = (int64_t *)malloc(n * 8), *e = (int64_t *)malloc(n * 8);
  uint64_t *sm = (uint64_t *)malloc(4 * n * 8), *sgm = sm + n, *em = sm + 2 * n, *a = sm + 3 * n;
  for (uint64_t lv = 0; lv < P->h; lv++) {
    const uint64_t g = 1 + (n >> lv);
    for (uint64_t i = 0; i < n; i++) {
      const uint64_t j = (i * g) & (2 * n - 1);
      if (j < n)
        sg[j] = sk[i];
      else
        sg[j - n] = -sk[i];
    }
    for (uint64_t j = 0; j < R; j++) {
      for (uint64_t i = 0; i < n; i++) e[i] = rng_cbd(&r);
      for (uint64_t m = 0; m < M; m++) {
        const rntt_t *T = &ctx->nt[m];
        const uint64_t q = T->q;
        uint64_t *k0 = keys + (((lv * R + j) * 2 + 0) * M + m) * n;
        uint64_t *k1 = keys + (((lv * R + j) * 2 + 1) * M + m) * n;
        for (uint64_t i = 0; i < n; i++) {
          sm[i] = small_mod(sk[i], q);
          em[i] = small_mod(e[i], q);
        }
        rntt_fwd1(T, n, sm);
        rntt_fwd1(T, n, em);
        for (uint64_t i = 0; i < n; i++) a[i] = rng_uniform(&r, q);
        for (uint64_t i = 0; i < n; i++) {
          k1[i] = a[i];
          k0[i] = addmod(negmod(mulmod(a[i], sm[i], q), q), em[i], q);
        }
        if (m == j) {
          for (uint64_t i = 0; i < n; i++) sgm[i] = small_mod(sg[i], q);
          rntt_fwd1(T, n, sgm);
          const uint64_t f = P->p % q;
          for (uint64_t i = 0; i < n; i++) k0[i] = addmod(k0[i], mulmod(f, sgm[i], q), q);
        }
      }
    }
  }
  free(sg);
  free(e);
  free(sm);
}

/* RGSW(sk) with the key gadget (client.cpp:17-31, gsw_eval.cpp:339-405),
 * coefficient form [2 l_key][2][R][N]:
 *   rows j <  l_key: (-a s + e + g_j s, a),  rows j >= l_key: (-a s + e, a + g_j s),
 * g_j = B_key^(l_key-1-j) mod q_i per prime. */
void orr_make_gsw_key(const orr_ctx *ctx, const int8_t *sk, uint64_t seed, uint64_t *rows) {
  const orr_params *P = &ctx->P;
  const uint64_t n = NN, R = RR;
  rng_t r = {seed ^ 0x65500000ULL};
  for (uint64_t j = 0; j < 2 * P->l_key; j++) {
    uint64_t *ct = rows + j * 2 * R * n;
    enc_zero(ctx, sk, &r, ct);
    const uint64_t half = j / P->l_key, lvl = j % P->l_key;
    for (uint64_t i = 0; i < R; i++) {
      const uint64_t q = P->q[i], g = ctx->gadget_key[i][lvl];
      uint64_t *dst = ct + (half * R + i) * n;
      for (uint64_t c = 0; c < n; c++) dst[c] = addmod(dst[c], mulmod(g, small_mod(sk[c], q), q), q);
    }
  }
}

static void query_indices(const orr_ctx *ctx, uint64_t pt_index, uint64_t *idx) {
  const orr_params *P = &ctx->P;
  uint64_t row = pt_index / P->n1, remain = P->num_pt / P->n1;
  idx[0] = pt_index % P->n1;
  for (uint64_t i = 1; i < P->ndim; i++) {
    remain /= 2;
    idx[i] = row / remain;
    row %= remain;
  }
}

/* fast_generate_query + add_gsw_to_query (client.cpp:130-209): BFV symmetric
 * encryption of (2^h)^-1 mod t at slot brv(idx0, h), with SEAL's scaling
 * Delta m = m floor(Q/t) + floor((m (Q mod t) + (t+1)/2) / t); then the
 * further dimensions' gadget values B^(l-1-k) (2^h)^-1 mod q_i added. */
void orr_make_query(const orr_ctx *ctx, const int8_t *sk, uint64_t seed, uint64_t entry_index,
                    uint64_t *ct) {
  const orr_params *P = &ctx->P;
  const uint64_t n = NN, R = RR, t = P->t, w = 1ULL << P->h;
  uint64_t idx[64];
  query_indices(ctx, entry_index / P->entries_per_pt, idx);
  rng_t r = {seed ^ 0x90E2700ULL};
  enc_zero(ctx, sk, &r, ct);
  const uint64_t m = powmod(w % t, t - 2, t);
  const uint64_t slot = brv(idx[0], (unsigned)P->h);
  const uint64_t fix = (uint64_t)(((u128)m * ctx->q_mod_t + ((t + 1) >> 1)) / t);
  for (uint64_t i = 0; i < R; i++) {
    const uint64_t q = P->q[i];
    const uint64_t dm = (uint64_t)(((u128)m * ctx->delta[i] + fix) % q);
    ct[i * n + slot] = addmod(ct[i * n + slot], dm, q);
  }
  for (uint64_t d = 1; d < P->ndim; d++) {
    if (idx[d] != 1) continue;
    for (uint64_t k = 0; k < P->l; k++) {
      const uint64_t rv = brv(P->n1 + (d - 1) * P->l + k, (unsigned)P->h);
      for (uint64_t i = 0; i < R; i++) {
        const uint64_t q = P->q[i];
        const uint64_t coef = mulmod(ctx->gadget[i][k], powmod(w % q, q - 2, q), q);
        ct[i * n + rv] = addmod(ct[i * n + rv], coef, q);
      }
    }
  }
}

/* decrypt_mod_q + invariant noise budget (client.cpp:458-479) of a response
 * [2][N] mod small_q. */
void orr_decrypt_small(const orr_ctx *ctx, const int8_t *sk, const uint64_t *ct, uint64_t *plain,
                       int *noise_budget) {
  const uint64_t n = NN, Q = ctx->P.small_q, t = ctx->P.t;
  const int mod = (int)RR + 1;
  uint64_t *c0 = (uint64_t *)calloc(4 * n, 8), *c1 = c0 + n, *s = c0 + 2 * n, *ph = c0 + 3 * n;
  for (uint64_t i = 0; i < n; i++) {
    c0[i] = ct[i] % Q;
    c1[i] = ct[n + i] % Q;
    s[i] = small_mod(sk[i], Q);
  }
  polymul(ctx, mod, c1, s, ph);
  uint64_t norm = 0;
  for (uint64_t i = 0; i < n; i++) {
    const uint64_t v0 = addmod(ph[i], c0[i], Q);
    plain[i] = (uint64_t)((((u128)v0 * t) + Q / 2) / Q) % t;
    const uint64_t v = mulmod(v0, t, Q);
    const uint64_t a = v > Q / 2 ? Q - v : v;
    if (a > norm) norm = a;
  }
  if (noise_budget) {
    const int b = (int)bitlen64(Q) - (int)bitlen64(norm) - 1;
    *noise_budget = b > 0 ? b : 0;
  }
  free(c0);
}

/* get_entry_from_plaintext (client.cpp:255-287) */
void orr_entry_from_plain(const orr_ctx *ctx, uint64_t entry_index, const uint64_t *plain,
                          uint8_t *entry) {
  const orr_params *P = &ctx->P;
  const uint64_t start = (entry_index % P->entries_per_pt) * P->entry_size * 8, bpc = P->bits_per_coeff;
  uint64_t ci = start / bpc, off = start % bpc, k = 0;
  u128 buf = plain[ci] >> off;
  uint64_t have = bpc - off;
  while (k < P->entry_size) {
    if (have >= 8) {
      entry[k++] = (uint8_t)(buf & 0xFF);
      buf >>= 8;
      have -= 8;
    } else {
      ci++;
      buf |= (u128)(ci < NN ? plain[ci] : 0) << have;
      have += bpc;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* server                                                                     */
/* ------------------------------------------------------------------------ */

/* x -> x^g on one polynomial mod q, coefficient form */
static void automorph(const orr_ctx *ctx, const uint64_t *in, uint64_t g, uint64_t q, uint64_t *out) {
  const uint64_t n = NN;
  for (uint64_t i = 0; i < n; i++) {
    const uint64_t j = (i * g) & (2 * n - 1);
    if (j < n)
      out[j] = in[i];
    else
      out[j - n] = negmod(in[i], q);
  }
}

/* Evaluator::apply_galois_inplace (server.cpp:409) with SEAL's RNS key
 * switching: T = sigma_g(c1); for every decomposition prime j the component
 * T mod q_j is lifted to every key modulus m (T_j mod m), transformed and
 * multiplied with key[j][k][m]; the sums X_k over j are brought back to
 * coefficient form and divided by p with rounding:
 *   ks_k,i = (x_i + p/2 - ((x_p + p/2) mod p)) p^-1 mod q_i,
 * out = (sigma_g(c0) + ks_0, ks_1). */
void orr_apply_galois(const orr_ctx *ctx, const uint64_t *ct, uint64_t g, const uint64_t *key,
                      uint64_t *out) {
  const uint64_t n = NN, R = RR, M = R + 1, p = ctx->P.p, ph = p >> 1;
  uint64_t *s0 = (uint64_t *)malloc(2 * R * n * 8), *T = s0 + R * n;
  uint64_t *lift = (uint64_t *)malloc(R * M * n * 8);
  uint64_t *acc = (uint64_t *)malloc(2 * M * n * 8);
  for (uint64_t i = 0; i < R; i++) {
    automorph(ctx, ct + i * n, g, ctx->P.q[i], s0 + i * n);
    automorph(ctx, ct + (R + i) * n, g, ctx->P.q[i], T + i * n);
  }
  for (uint64_t j = 0; j < R; j++)
    for (uint64_t m = 0; m < M; m++) {
      uint64_t *d = lift + (j * M + m) * n;
      for (uint64_t c = 0; c < n; c++) d[c] = T[j * n + c] % ctx->nt[m].q;
      rntt_fwd1(&ctx->nt[m], n, d);
    }
  for (uint64_t k = 0; k < 2; k++)
    for (uint64_t m = 0; m < M; m++) {
      const uint64_t q = ctx->nt[m].q;
      uint64_t *a = acc + (k * M + m) * n;
      for (uint64_t c = 0; c < n; c++) {
        u128 s = 0;
        for (uint64_t j = 0; j < R; j++)
          s += (u128)lift[(j * M + m) * n + c] * key[((j * 2 + k) * M + m) * n + c];
        a[c] = (uint64_t)(s % q);
      }
      rntt_inv1(&ctx->nt[m], n, a);
    }
  for (uint64_t k = 0; k < 2; k++) {
    const uint64_t *xp = acc + (k * M + R) * n;
    for (uint64_t i = 0; i < R; i++) {
      const uint64_t q = ctx->P.q[i];
      const uint64_t *xq = acc + (k * M + i) * n;
      for (uint64_t c = 0; c < n; c++) {
        const uint64_t rr = addmod(xp[c], ph, p);
        uint64_t v = submod(addmod(xq[c], ph % q, q), rr % q, q);
        v = mulmod(v, ctx->p_inv[i], q);
        if (k == 0)
          out[i * n + c] = addmod(s0[i * n + c], v, q);
        else
          out[(R + i) * n + c] = v;
      }
    }
  }
  free(s0);
  free(lift);
  free(acc);
}

/* utils::shift_polynomial (utils.cpp:6-40) with index = -k, every prime */
static void neg_shift(const orr_ctx *ctx, const uint64_t *ct, uint64_t k, uint64_t *out) {
  const uint64_t n = NN, R = RR, shift = (uint64_t)(-(int64_t)k);
  for (uint64_t poly = 0; poly < 2; poly++)
    for (uint64_t i = 0; i < R; i++) {
      const uint64_t q = ctx->P.q[i];
      const uint64_t *in = ct + (poly * R + i) * n;
      uint64_t *o = out + (poly * R + i) * n;
      uint64_t raw = shift;
      for (uint64_t c = 0; c < n; c++, raw++) {
        const uint64_t index = raw & (n - 1);
        o[index] = (!(raw & n) || !in[c]) ? in[c] : q - in[c];
      }
    }
}

/* fast_expand_qry (server.cpp:383-428) */
void orr_expand(const orr_ctx *ctx, const uint64_t *query, const uint64_t *galois_keys,
                uint64_t *leaves) {
  const orr_params *P = &ctx->P;
  const uint64_t n = NN, R = RR, h = P->h, w = 1ULL << h, u = P->u, CT = 2 * R * n;
  const uint64_t key_words = R * 2 * (R + 1) * n;
  uint64_t *cur = (uint64_t *)malloc(w * CT * 8), *nxt = (uint64_t *)malloc(w * CT * 8);
  memcpy(cur, query, CT * 8);
  for (uint64_t a = 0; a < h; a++) {
    const uint64_t k = 1ULL << a;
    const uint64_t *key = galois_keys + a * key_words;
#pragma omp parallel for schedule(dynamic, 1)
    for (long ii = 0; ii < (long)k; ii++) {
      const uint64_t i = k + (uint64_t)ii;
      if (i * w / k - w >= u) continue;
      const uint64_t *ci = cur + (uint64_t)ii * CT;
      uint64_t *even = nxt + 2 * (uint64_t)ii * CT, *odd = even + CT;
      uint64_t *cp = (uint64_t *)malloc(2 * CT * 8), *diff = cp + CT;
      orr_apply_galois(ctx, ci, n / k + 1, key, cp);
      for (uint64_t poly = 0; poly < 2; poly++)
        for (uint64_t r = 0; r < R; r++) {
          const uint64_t q = P->q[r], off = (poly * R + r) * n;
          for (uint64_t c = 0; c < n; c++) {
            even[off + c] = addmod(ci[off + c], cp[off + c], q);
            diff[off + c] = submod(ci[off + c], cp[off + c], q);
          }
        }
      neg_shift(ctx, diff, k, odd);
      free(cp);
    }
    uint64_t *tmp = cur;
    cur = nxt;
    nxt = tmp;
  }
  memcpy(leaves, cur, u * CT * 8);
  free(cur);
  free(nxt);
}

/* gsw_ntt_negacyclic_harvey (gsw_eval.cpp:15-31): rows [2][R][N] to NTT form */
void orr_gsw_to_ntt(const orr_ctx *ctx, const uint64_t *rows_coeff, uint64_t rows,
                    uint64_t *rows_ntt) {
  const uint64_t n = NN, R = RR;
  memcpy(rows_ntt, rows_coeff, rows * 2 * R * n * 8);
#pragma omp parallel for schedule(static) if (rows > 4)
  for (long j = 0; j < (long)(rows * 2); j++) rns_fwd(ctx, rows_ntt + (uint64_t)j * R * n);
}

/* decomp_rlwe (gsw_eval.cpp:108-182; decomp_rlwe_single_mod 184-224 when
 * R = 1): each coefficient's residues are composed by CRT into the integer
 * X in [0, Q); digit (X >> (p b)) & (2^b - 1) for p = l-1 .. 0 is the same
 * small value in every prime.  Output [poly][l][R][N] in that order. */
void orr_decompose(const orr_ctx *ctx, const uint64_t *ct, uint64_t l, uint64_t base_log2,
                   uint64_t *digits) {
  const uint64_t n = NN, R = RR;
  const u128 mask = ((u128)1 << base_log2) - 1;
  for (uint64_t poly = 0; poly < 2; poly++)
    for (uint64_t c = 0; c < n; c++) {
      u128 X;
      if (R == 1) {
        X = ct[poly * n + c];
      } else {
        /* X = x_1 + q_1 ((x_0 - x_1) q_1^-1 mod q_0) */
        const uint64_t q0 = ctx->P.q[0], q1 = ctx->P.q[1];
        const uint64_t x0 = ct[(poly * R + 0) * n + c], x1 = ct[(poly * R + 1) * n + c];
        const uint64_t d = mulmod(submod(x0, x1 % q0, q0), ctx->last_inv[0], q0);
        X = (u128)x1 + (u128)q1 * d;
      }
      for (uint64_t pp = l; pp-- > 0;) {
        const uint64_t j = poly * l + (l - 1 - pp);
        const uint64_t v = (uint64_t)((X >> (pp * base_log2)) & mask);
        for (uint64_t i = 0; i < R; i++) digits[(j * R + i) * n + c] = v;
      }
    }
}

/* GSWEval::external_product (gsw_eval.cpp:33-106): decompose, NTT every
 * digit polynomial per prime, sum_j digit_j * gsw[j][k] in 128 bits, reduce
 * per prime.  Output [2][R][N] in NTT form. */
void orr_ext_product(const orr_ctx *ctx, const uint64_t *gsw, uint64_t l, uint64_t base_log2,
                     const uint64_t *ct, uint64_t *out) {
  const uint64_t n = NN, R = RR;
  uint64_t *d = (uint64_t *)malloc(2 * l * R * n * 8);
  orr_decompose(ctx, ct, l, base_log2, d);
  for (uint64_t j = 0; j < 2 * l; j++) rns_fwd(ctx, d + j * R * n);
  for (uint64_t k = 0; k < 2; k++)
    for (uint64_t i = 0; i < R; i++) {
      const uint64_t q = ctx->P.q[i];
      for (uint64_t c = 0; c < n; c++) {
        u128 s = 0;
        for (uint64_t j = 0; j < 2 * l; j++)
          s += (u128)d[(j * R + i) * n + c] * gsw[((j * 2 + k) * R + i) * n + c];
        out[(k * R + i) * n + c] = (uint64_t)(s % q);
      }
    }
  free(d);
}

/* GSWEval::query_to_gsw (gsw_eval.cpp:254-286) */
void orr_query_to_gsw(const orr_ctx *ctx, const uint64_t *cts, const uint64_t *key,
                      uint64_t *out) {
  const orr_params *P = &ctx->P;
  const uint64_t CT = 2 * RR * NN;
  for (uint64_t i = 0; i < P->l; i++) {
    memcpy(out + i * CT, cts + i * CT, CT * 8);
    rns_fwd(ctx, out + i * CT);
    rns_fwd(ctx, out + i * CT + RR * NN);
  }
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)P->l; i++)
    orr_ext_product(ctx, key, P->l_key, P->base_log2_key, cts + (uint64_t)i * CT,
                    out + (P->l + (uint64_t)i) * CT);
}

/* evaluate_first_dim (server.cpp:124-175) + mat_mat_128 (matrix.cpp:220-235)
 * + delay_modulus (server.cpp:178-293) per slot c of every prime; exact sums
 * (returns how many uint128 sums of the reference would have wrapped). */
int orr_first_dim(const orr_ctx *ctx, const uint64_t *db, const uint64_t *fst, uint64_t *out) {
  const orr_params *P = &ctx->P;
  const uint64_t n = NN, R = RR, n1 = P->n1, nr = P->n_rest, np = P->num_pt, CT = 2 * R * n;
  uint64_t *qn = (uint64_t *)malloc(n1 * CT * 8);
  memcpy(qn, fst, n1 * CT * 8);
#pragma omp parallel for schedule(static)
  for (long k = 0; k < (long)(2 * n1); k++) rns_fwd(ctx, qn + (uint64_t)k * R * n);
  long wraps = 0;
#pragma omp parallel for schedule(static) reduction(+ : wraps)
  for (long cc = 0; cc < (long)(R * n); cc++) {
    const uint64_t i = (uint64_t)cc / n, c = (uint64_t)cc % n, q = P->q[i];
    const uint64_t *A = db + (uint64_t)cc * np;
    for (uint64_t row = 0; row < nr; row++) {
      u128 t0 = 0, t1 = 0;
      uint64_t w0 = 0, w1 = 0;
      for (uint64_t k = 0; k < n1; k++) {
        const uint64_t a = A[row * n1 + k];
        const u128 p0 = (u128)a * qn[k * CT + i * n + c], p1 = (u128)a * qn[k * CT + (R + i) * n + c];
        t0 += p0;
        w0 += t0 < p0;
        t1 += p1;
        w1 += t1 < p1;
      }
      wraps += (long)(w0 + w1);
      const u128 two128 = ctx->nt[i].two128;
      out[row * CT + i * n + c] = (uint64_t)((t0 % q + (u128)(w0 % q) * two128) % q);
      out[row * CT + (R + i) * n + c] = (uint64_t)((t1 % q + (u128)(w1 % q) * two128) % q);
    }
  }
#pragma omp parallel for schedule(static)
  for (long k = 0; k < (long)(2 * nr); k++) rns_inv(ctx, out + (uint64_t)k * R * n);
  free(qn);
  return (int)(wraps > 0x7fffffff ? 0x7fffffff : wraps);
}

/* other_dim_mux (server.cpp:295-334): x_i += INTT(RGSW (x) (x_{i+half} - x_i)) */
void orr_other_dim_mux(const orr_ctx *ctx, uint64_t *res, uint64_t count, const uint64_t *gsw) {
  const orr_params *P = &ctx->P;
  const uint64_t n = NN, R = RR, CT = 2 * R * n, half = count / 2;
#pragma omp parallel for schedule(dynamic, 1)
  for (long ii = 0; ii < (long)half; ii++) {
    uint64_t *x = res + (uint64_t)ii * CT;
    const uint64_t *y = res + (half + (uint64_t)ii) * CT;
    uint64_t *diff = (uint64_t *)malloc(2 * CT * 8), *e = diff + CT;
    for (uint64_t poly = 0; poly < 2; poly++)
      for (uint64_t i = 0; i < R; i++) {
        const uint64_t off = (poly * R + i) * n;
        for (uint64_t c = 0; c < n; c++) diff[off + c] = submod(y[off + c], x[off + c], P->q[i]);
      }
    orr_ext_product(ctx, gsw, P->l, P->base_log2, diff, e);
    rns_inv(ctx, e);
    rns_inv(ctx, e + R * n);
    for (uint64_t poly = 0; poly < 2; poly++)
      for (uint64_t i = 0; i < R; i++) {
        const uint64_t off = (poly * R + i) * n;
        for (uint64_t c = 0; c < n; c++) x[off + c] = addmod(x[off + c], e[off + c], P->q[i]);
      }
    free(diff);
  }
}

/* Evaluator::mod_switch_to_next_inplace (server.cpp:567-570) for BFV: SEAL's
 * divide-and-round by the last prime q_L, per remaining prime q_i:
 *   r = (x_L + q_L/2) mod q_L,  x_i' = (x_i + q_L/2 - r) q_L^-1 mod q_i. */
void orr_mod_switch_next(const orr_ctx *ctx, const uint64_t *ct, uint64_t *out) {
  const uint64_t n = NN, R = RR, qL = ctx->P.q[R - 1], h = qL >> 1;
  for (uint64_t poly = 0; poly < 2; poly++)
    for (uint64_t i = 0; i + 1 < R; i++) {
      const uint64_t q = ctx->P.q[i];
      for (uint64_t c = 0; c < n; c++) {
        const uint64_t r = addmod(ct[(poly * R + R - 1) * n + c], h, qL);
        const uint64_t v = submod(addmod(ct[(poly * R + i) * n + c], h % q, q), r % q, q);
        out[(poly * (R - 1) + i) * n + c] = mulmod(v, ctx->last_inv[i], q);
      }
    }
}

/* mod_switch_inplace (server.cpp:779-801): the x87 long-double product and
 * round(), emulated in integers as in opir_oracle.c. */
uint64_t orr_mod_switch_coeff(const orr_ctx *ctx, uint64_t x) {
  const uint64_t M = ctx->P.ms_mant;
  const int64_t E = ctx->P.ms_exp;
  if (x == 0) return 0;
  u128 P = (u128)x * M;
  const unsigned b = bitlen128(P);
  if (b > 64) {
    const unsigned sh = b - 64;
    u128 keep = P >> sh;
    const u128 rem = P & (((u128)1 << sh) - 1), half = (u128)1 << (sh - 1);
    if (rem > half || (rem == half && (keep & 1))) keep++;
    P = keep << sh;
  }
  if (E >= 0) return (uint64_t)(P << E);
  const unsigned s = (unsigned)(-E);
  if (s >= 127) return 0;
  return (uint64_t)((P + ((u128)1 << (s - 1))) >> s);
}

uint64_t orr_response_bytes(const orr_ctx *ctx) {
  return (2 * NN * ctx->P.small_q_width + 7) / 8;
}

/* save_resp_to_stream (server.cpp:581-633) */
uint64_t orr_pack_response(const orr_ctx *ctx, const uint64_t *ct, uint8_t *out) {
  const uint64_t w = ctx->P.small_q_width, nbytes = orr_response_bytes(ctx);
  memset(out, 0, nbytes);
  uint64_t bit = 0;
  for (uint64_t i = 0; i < 2 * NN; i++) {
    const uint64_t v = ct[i] & ((1ULL << w) - 1);
    for (uint64_t j = 0; j < w; j++, bit++) out[bit >> 3] |= (uint8_t)(((v >> j) & 1) << (bit & 7));
  }
  return nbytes;
}

/* PirServer::make_query (server.cpp:520-579) + save_resp_to_stream */
int orr_make_query_server(const orr_ctx *ctx, const uint64_t *db, const uint64_t *galois_keys,
                          const uint64_t *gsw_key_ntt, const uint64_t *query, uint64_t *resp,
                          uint8_t *packed) {
  const orr_params *P = &ctx->P;
  const uint64_t n = NN, R = RR, CT = 2 * R * n, dims = P->ndim;
  uint64_t *leaves = (uint64_t *)malloc(P->u * CT * 8);
  orr_expand(ctx, query, galois_keys, leaves);
  uint64_t *gsw = (uint64_t *)malloc((dims > 1 ? dims - 1 : 1) * 2 * P->l * CT * 8);
  for (uint64_t d = 1; d < dims; d++)
    orr_query_to_gsw(ctx, leaves + (P->n1 + (d - 1) * P->l) * CT, gsw_key_ntt,
                     gsw + (d - 1) * 2 * P->l * CT);
  uint64_t *res = (uint64_t *)malloc(P->n_rest * CT * 8);
  const int wraps = orr_first_dim(ctx, db, leaves, res);
  uint64_t cnt = P->n_rest;
  for (uint64_t d = 1; d < dims; d++) {
    orr_other_dim_mux(ctx, res, cnt, gsw + (d - 1) * 2 * P->l * CT);
    cnt /= 2;
  }
  /* to the first prime (server.cpp:567-570), then to small_q */
  uint64_t *one = (uint64_t *)malloc(2 * n * 8);
  if (R > 1)
    orr_mod_switch_next(ctx, res, one);
  else
    memcpy(one, res, 2 * n * 8);
  for (uint64_t c = 0; c < 2 * n; c++) resp[c] = orr_mod_switch_coeff(ctx, one[c]);
  if (packed) orr_pack_response(ctx, resp, packed);
  free(one);
  free(leaves);
  free(gsw);
  free(res);
  return wraps;
}
