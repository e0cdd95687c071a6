/*
 * opir_oracle.c -- CPU oracle for the OnionPIRv2 server query path.
 *
 * TEST INFRASTRUCTURE ONLY (see opir_oracle.h for the parity status).  Every
 * function names the reference code it restates.  SEAL primitives the
 * reference calls (NTT, Galois automorphism + key switching, Barrett
 * reduction, prime generation, BFV encryption/decryption) are restated from
 * the mathematics of BFV/RGSW and the public description of SEAL 4.1.
 *
 * Built with -O3 (and -fopenmp where available) so that it can also serve as
 * the timed CPU baseline of the same algorithm.
 */
#include "opir_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

#define N ORC_N
#define LOGN ORC_LOGN

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
static inline uint64_t submod(uint64_t a, uint64_t b, uint64_t q) {
  return a >= b ? a - b : a + q - b;
}
static inline uint64_t negmod(uint64_t a, uint64_t q) { return a ? q - a : 0; }

/* Shoup companion floor(w * 2^64 / q) */
static inline uint64_t shoup(uint64_t w, uint64_t q) { return (uint64_t)(((u128)w << 64) / q); }

/* w*x mod q with precomputed companion, result in [0, q) */
static inline uint64_t mul_shoup(uint64_t x, uint64_t w, uint64_t ws, uint64_t q) {
  uint64_t hq = (uint64_t)(((u128)x * ws) >> 64);
  uint64_t r = x * w - hq * q;
  return r >= q ? r - q : r;
}

typedef struct {
  uint64_t q, mu_lo, mu_hi; /* mu = floor(2^128 / q) */
  uint64_t r64;             /* 2^64 mod q */
  uint64_t r128;            /* 2^128 mod q */
} barrett_t;

static void barrett_init(barrett_t *b, uint64_t q) {
  u128 mu = (~(u128)0) / q; /* == floor(2^128/q) since q is odd */
  b->q = q;
  b->mu_lo = (uint64_t)mu;
  b->mu_hi = (uint64_t)(mu >> 64);
  b->r64 = (uint64_t)(((u128)1 << 64) % q);
  b->r128 = mulmod(b->r64, b->r64, q);
}

/* Exact x mod q for x < 2^125 (the role of SEAL's barrett_reduce_128 in
 * gsw_eval.cpp:100, server.cpp:222-227, matrix.h:92).  q_hat below equals
 * floor(x * mu / 2^128) exactly, which is >= floor(x/q) - 1, so one
 * conditional subtraction finishes. */
static inline uint64_t barrett128(u128 x, const barrett_t *b) {
  uint64_t lo = (uint64_t)x, hi = (uint64_t)(x >> 64);
  u128 t = ((u128)lo * b->mu_lo) >> 64;
  u128 m1 = (u128)lo * b->mu_hi + (u128)hi * b->mu_lo + t;
  uint64_t qhat = hi * b->mu_hi + (uint64_t)(m1 >> 64);
  uint64_t r = lo - qhat * b->q;
  return r >= b->q ? r - b->q : r;
}

/* Exact x mod q for any 128-bit x. */
static inline uint64_t reduce128_full(u128 x, const barrett_t *b) {
  uint64_t hi = (uint64_t)(x >> 64), lo = (uint64_t)x;
  uint64_t hr = hi % b->q;
  return barrett128((u128)hr * b->r64 + lo, b);
}

uint64_t orc_barrett_reduce_128(uint64_t lo, uint64_t hi, uint64_t q) {
  barrett_t b;
  barrett_init(&b, q);
  return reduce128_full(((u128)hi << 64) | lo, &b);
}

/* ------------------------------------------------------------------------ */
/* primes (utils.cpp:82-95; SEAL CoeffModulus::Create called at pir.cpp:23,40) */
/* ------------------------------------------------------------------------ */

int orc_is_prime(uint64_t n) {
  static const uint64_t bases[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
  if (n < 2) return 0;
  for (size_t i = 0; i < sizeof(bases) / sizeof(bases[0]); i++) {
    if (n == bases[i]) return 1;
    if (n % bases[i] == 0) return 0;
  }
  uint64_t d = n - 1;
  int s = 0;
  while (!(d & 1)) {
    d >>= 1;
    s++;
  }
  for (size_t i = 0; i < sizeof(bases) / sizeof(bases[0]); i++) {
    uint64_t x = powmod(bases[i], d, n);
    if (x == 1 || x == n - 1) continue;
    int comp = 1;
    for (int r = 1; r < s; r++) {
      x = mulmod(x, x, n);
      if (x == n - 1) {
        comp = 0;
        break;
      }
    }
    if (comp) return 0;
  }
  return 1;
}

/* utils::generate_prime: smallest prime reached by candidate++, |= 1 from
 * 2^(bits-1) (utils.cpp:82-95). */
uint64_t orc_generate_prime(uint64_t bit_width) {
  if (bit_width < 2) return 0;
  uint64_t c = 1ULL << (bit_width - 1);
  do {
    c++;
    c |= 1;
  } while (!orc_is_prime(c));
  return c;
}

/* CoeffModulus::Create(n, bit_sizes): for every distinct bit size b, the
 * largest primes below 2^b that are 1 mod 2n, in descending order, handed
 * out to the requests of that size in the order the requests appear. */
int orc_coeff_modulus_create(uint64_t n, const uint64_t *bits, size_t count, uint64_t *out) {
  for (size_t i = 0; i < count; i++) {
    size_t rank = 0;
    for (size_t j = 0; j < i; j++)
      if (bits[j] == bits[i]) rank++;
    uint64_t b = bits[i];
    uint64_t step = 2 * n;
    uint64_t lower = 1ULL << (b - 1);
    uint64_t v = (b == 64 ? 0 : (1ULL << b)) - step + 1;
    size_t found = 0;
    for (;;) {
      if (v <= lower) return -1;
      if (orc_is_prime(v)) {
        if (found == rank) break;
        found++;
      }
      v -= step;
    }
    out[i] = v;
  }
  return 0;
}

/* Smallest primitive 2n-th root of unity mod q (the root SEAL's NTT tables
 * are built on). */
uint64_t orc_minimal_root(uint64_t q, uint64_t two_n) {
  uint64_t cof = (q - 1) / two_n;
  uint64_t psi = 0;
  for (uint64_t g = 2; g < q; g++) {
    uint64_t c = powmod(g, cof, q);
    if (powmod(c, two_n / 2, q) == q - 1) {
      psi = c;
      break;
    }
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
/* NTT tables and transforms                                                  */
/* ------------------------------------------------------------------------ */

typedef struct {
  uint64_t q, psi, n_inv, n_inv_s;
  uint64_t fwd[N], fwd_s[N]; /* psi^brv(i)  */
  uint64_t inv[N], inv_s[N]; /* psi^-brv(i) */
  barrett_t br;
} ntt_t;

static inline uint64_t brv(uint64_t x, unsigned bits) {
  uint64_t y = 0;
  for (unsigned i = 0; i < bits; i++) {
    y = (y << 1) | (x & 1);
    x >>= 1;
  }
  return y;
}

static void ntt_init(ntt_t *T, uint64_t q) {
  T->q = q;
  T->psi = orc_minimal_root(q, 2 * N);
  uint64_t psi_inv = powmod(T->psi, q - 2, q);
  for (uint64_t i = 0; i < N; i++) {
    uint64_t e = brv(i, LOGN);
    T->fwd[i] = powmod(T->psi, e, q);
    T->inv[i] = powmod(psi_inv, e, q);
    T->fwd_s[i] = shoup(T->fwd[i], q);
    T->inv_s[i] = shoup(T->inv[i], q);
  }
  T->n_inv = powmod(N, q - 2, q);
  T->n_inv_s = shoup(T->n_inv, q);
  barrett_init(&T->br, q);
}

/* Forward negacyclic NTT (Cooley-Tukey, bit-reversed output): on return
 * a[k] = A(psi^(2*brv(k)+1)).  This is the transform SEAL's
 * ntt_negacyclic_harvey computes (gsw_eval.cpp:24,28,248), with every output
 * fully reduced. */
static void ntt_fwd1(const ntt_t *T, uint64_t *a) {
  const uint64_t q = T->q;
  size_t t = N;
  for (size_t m = 1; m < N; m <<= 1) {
    t >>= 1;
    for (size_t i = 0; i < m; i++) {
      const uint64_t w = T->fwd[m + i], ws = T->fwd_s[m + i];
      uint64_t *x = a + 2 * i * t, *y = x + t;
      for (size_t j = 0; j < t; j++) {
        uint64_t u = x[j], v = mul_shoup(y[j], w, ws, q);
        x[j] = addmod(u, v, q);
        y[j] = submod(u, v, q);
      }
    }
  }
}

/* Inverse of ntt_fwd1 (Gentleman-Sande), outputs fully reduced
 * (SEAL inverse_ntt_negacyclic_harvey, server.cpp:239,290,325). */
static void ntt_inv1(const ntt_t *T, uint64_t *a) {
  const uint64_t q = T->q;
  size_t t = 1;
  for (size_t m = N >> 1; m >= 1; m >>= 1) {
    for (size_t i = 0; i < m; i++) {
      const uint64_t w = T->inv[m + i], ws = T->inv_s[m + i];
      uint64_t *x = a + 2 * i * t, *y = x + t;
      for (size_t j = 0; j < t; j++) {
        uint64_t u = x[j], v = y[j];
        x[j] = addmod(u, v, q);
        y[j] = mul_shoup(submod(u, v, q), w, ws, q);
      }
    }
    t <<= 1;
  }
  for (size_t i = 0; i < N; i++) a[i] = mul_shoup(a[i], T->n_inv, T->n_inv_s, q);
}

/* ------------------------------------------------------------------------ */
/* context                                                                    */
/* ------------------------------------------------------------------------ */

struct orc_ctx {
  orc_params P;
  ntt_t nt[3]; /* q, p, small_q */
  uint64_t gadget[64];     /* data gadget  B^(l-1) .. B^0 mod q   (utils.cpp:61-74) */
  uint64_t gadget_key[64]; /* key gadget   */
  uint64_t p_half, p_inv_q, p_inv_q_s;
};

static uint64_t next_pow2(uint64_t n) {
  uint64_t p = 1;
  while (p < n) p <<= 1;
  return p;
}
static uint64_t roundup_div(uint64_t a, uint64_t b) { return (a + b - 1) / b; }
static unsigned bitlen64(uint64_t x) {
  unsigned b = 0;
  while (x) {
    b++;
    x >>= 1;
  }
  return b;
}
static unsigned ceil_log2(uint64_t x) {
  unsigned c = 0;
  while ((1ULL << c) < x) c++;
  return c;
}

/* PirParams::PirParams (pir.cpp:29-95) and init_seal_params (pir.cpp:9-27). */
orc_ctx *orc_create(uint64_t num_entries, uint64_t max_fst_dim, uint64_t entry_size,
                    uint64_t l, uint64_t l_key, uint64_t plain_bits, uint64_t small_q_width,
                    uint64_t coeff_bits0, uint64_t coeff_bits1) {
  orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
  if (!c) return NULL;
  orc_params *P = &c->P;
  P->poly_degree = N;
  P->t = orc_generate_prime(plain_bits); /* pir.cpp:18 */
  uint64_t bits[2] = {coeff_bits0, coeff_bits1}, mods[2];
  if (orc_coeff_modulus_create(N, bits, 2, mods)) goto fail;
  P->q = mods[0];
  P->p = mods[1];
  uint64_t sq_bits[2] = {small_q_width, coeff_bits1}, sq[2];
  if (orc_coeff_modulus_create(N, sq_bits, 2, sq)) goto fail; /* pir.cpp:40-41 */
  P->small_q = sq[0];
  P->small_q_width = (uint64_t)ceil(log2((double)P->small_q)); /* server.cpp:587-588 */
  P->bits_per_coeff = bitlen64(P->t) - 1;                        /* pir.cpp:97-99 */
  P->entry_size = entry_size ? entry_size : P->bits_per_coeff * N / 8; /* pir.cpp:34-38 */
  P->entries_per_pt = P->bits_per_coeff * N / (P->entry_size * 8);     /* pir.cpp:105-112 */
  if (P->entries_per_pt == 0) goto fail;
  P->l = l;
  P->l_key = l_key;
  {
    uint64_t logq = bitlen64(P->q); /* only q counts: the last prime is special */
    P->base_log2 = (logq + l - 1) / l;         /* pir.cpp:53 */
    P->base_log2_key = (logq + l_key - 1) / l_key; /* pir.cpp:54 */
  }
  {
    uint64_t num_pt_required = roundup_div(num_entries, P->entries_per_pt); /* pir.cpp:67 */
    uint64_t other = roundup_div(next_pow2(num_pt_required), max_fst_dim); /* pir.cpp:70 */
    uint64_t first = roundup_div(num_pt_required, other);                  /* pir.cpp:72 */
    P->num_pt = first * other;
    P->num_entries = P->num_pt * P->entries_per_pt;
    P->n1 = first;
    P->n_rest = other;
    P->ndim = 1 + (uint64_t)log2((double)other); /* pir.cpp:89 */
  }
  P->u = P->n1 + P->l * (P->ndim - 1);
  P->h = ceil_log2(P->u); /* pir.h:66-68 */
  {
    double scale = (double)P->small_q / (double)P->q; /* server.cpp:795 */
    int e;
    double m = frexp(scale, &e);
    P->ms_mant = (uint64_t)ldexp(m, 53);
    P->ms_exp = (int64_t)e - 53;
  }
  ntt_init(&c->nt[0], P->q);
  ntt_init(&c->nt[1], P->p);
  ntt_init(&c->nt[2], P->small_q);
  for (int i = 0; i < 64; i++) c->gadget[i] = c->gadget_key[i] = 0;
  {
    u128 pw = 1;
    for (int j = (int)l - 1; j >= 0; j--) {
      c->gadget[j] = (uint64_t)pw;
      pw = (pw << P->base_log2) % P->q;
    }
    pw = 1;
    for (int j = (int)l_key - 1; j >= 0; j--) {
      c->gadget_key[j] = (uint64_t)pw;
      pw = (pw << P->base_log2_key) % P->q;
    }
  }
  c->p_half = P->p >> 1;
  c->p_inv_q = powmod(P->p % P->q, P->q - 2, P->q);
  c->p_inv_q_s = shoup(c->p_inv_q, P->q);
  return c;
fail:
  free(c);
  return NULL;
}

void orc_destroy(orc_ctx *ctx) { free(ctx); }
void orc_get_params(const orc_ctx *ctx, orc_params *out) { *out = ctx->P; }

int orc_set_threads(int n) {
#ifdef _OPENMP
  int prev = omp_get_max_threads();
  if (n > 0) omp_set_num_threads(n);
  return prev;
#else
  (void)n;
  return 1;
#endif
}

void orc_ntt_fwd(const orc_ctx *ctx, int mod, uint64_t *a, size_t count) {
  const ntt_t *T = &ctx->nt[mod];
#pragma omp parallel for schedule(static) if (count > 8)
  for (long i = 0; i < (long)count; i++) ntt_fwd1(T, a + (size_t)i * N);
}
void orc_ntt_inv(const orc_ctx *ctx, int mod, uint64_t *a, size_t count) {
  const ntt_t *T = &ctx->nt[mod];
#pragma omp parallel for schedule(static) if (count > 8)
  for (long i = 0; i < (long)count; i++) ntt_inv1(T, a + (size_t)i * N);
}
void orc_ntt_tables(const orc_ctx *ctx, int mod, uint64_t *fwd, uint64_t *inv, uint64_t *psi,
                    uint64_t *n_inv) {
  const ntt_t *T = &ctx->nt[mod];
  if (fwd) memcpy(fwd, T->fwd, sizeof(T->fwd));
  if (inv) memcpy(inv, T->inv, sizeof(T->inv));
  if (psi) *psi = T->psi;
  if (n_inv) *n_inv = T->n_inv;
}

/* ------------------------------------------------------------------------ */
/* deterministic randomness (replaces /dev/urandom and SEAL's PRNG)           */
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
  unsigned b = bitlen64(q);
  for (;;) {
    uint64_t v = rng_next(r) >> (64 - b);
    if (v < q) return v;
  }
}
/* centered binomial, eta = 21 (sigma ~ 3.24, SEAL's default error width) */
static int64_t rng_cbd(rng_t *r) {
  uint64_t v = rng_next(r);
  return (int64_t)__builtin_popcountll(v & 0x1FFFFF) -
         (int64_t)__builtin_popcountll((v >> 21) & 0x1FFFFF);
}

/* Entry byte stream: bytes 0..7 are the entry index big-endian
 * (utils.cpp:98-104); the rest are seeded pseudo-random bytes in place of
 * /dev/urandom (utils.cpp:160-172). */
static inline uint64_t entry_word(uint64_t seed, uint64_t entry, uint64_t i) {
  return mix64(seed * 0x9E3779B97F4A7C15ULL + entry * 0xD1B54A32D192ED03ULL + i);
}

void orc_gen_entries(const orc_ctx *ctx, uint64_t seed, uint64_t first_entry, uint64_t count,
                     uint8_t *out) {
  const uint64_t es = ctx->P.entry_size;
#pragma omp parallel for schedule(static) if (count > 64)
  for (long k = 0; k < (long)count; k++) {
    uint64_t e = first_entry + (uint64_t)k;
    uint8_t *o = out + (size_t)k * es;
    for (int i = 0; i < 8; i++) o[7 - i] = (uint8_t)(e >> (8 * i));
    for (uint64_t j = 8; j < es; j++) {
      uint64_t w = entry_word(seed, e, (j - 8) >> 3);
      o[j] = (uint8_t)(w >> (8 * ((j - 8) & 7)));
    }
  }
}

/* push_database_chunk byte packing (server.cpp:649-700): bytes LSB-first into
 * bits_per_coeff-bit coefficients, remainder into one extra coefficient. */
void orc_pack_plaintexts(const orc_ctx *ctx, const uint8_t *entries, uint64_t num_pt,
                         uint64_t *coeffs) {
  const orc_params *P = &ctx->P;
  const uint64_t bpc = P->bits_per_coeff, epp = P->entries_per_pt, es = P->entry_size;
  const u128 mask = ((u128)1 << bpc) - 1;
#pragma omp parallel for schedule(static) if (num_pt > 16)
  for (long i = 0; i < (long)num_pt; i++) {
    uint64_t *pt = coeffs + (size_t)i * N;
    memset(pt, 0, N * sizeof(uint64_t));
    size_t index = 0;
    u128 buf = 0;
    uint64_t off = 0;
    for (uint64_t j = (uint64_t)i * epp; j < ((uint64_t)i + 1) * epp; j++) {
      const uint8_t *e = entries + j * es;
      for (uint64_t k = 0; k < es; k++) {
        buf += (u128)e[k] << off;
        off += 8;
        while (off >= bpc) {
          pt[index++] = (uint64_t)(buf & mask);
          buf >>= bpc;
          off -= bpc;
        }
      }
    }
    if (off > 0) pt[index++] = (uint64_t)(buf & mask);
  }
}

/* Evaluator::transform_to_ntt_inplace(Plaintext, first_parms_id)
 * (server.cpp:709): plain coefficients are lifted to Z_q centred (values
 * >= (t+1)/2 become v + q - t), then forward NTT mod q. */
void orc_plain_to_ntt(const orc_ctx *ctx, uint64_t *coeffs, uint64_t num_pt) {
  const orc_params *P = &ctx->P;
  const uint64_t thr = (P->t + 1) >> 1, inc = P->q - P->t;
  const ntt_t *T = &ctx->nt[0];
#pragma omp parallel for schedule(static) if (num_pt > 8)
  for (long i = 0; i < (long)num_pt; i++) {
    uint64_t *pt = coeffs + (size_t)i * N;
    for (size_t c = 0; c < N; c++)
      if (pt[c] >= thr) pt[c] += inc;
    ntt_fwd1(T, pt);
  }
}

/* realign_db (server.cpp:722-748): db_aligned[c*num_pt + pt] */
void orc_realign(const orc_ctx *ctx, const uint64_t *ntt_pts, uint64_t *db_aligned) {
  const uint64_t np = ctx->P.num_pt;
#pragma omp parallel for schedule(static)
  for (long c = 0; c < N; c++)
    for (uint64_t pt = 0; pt < np; pt++) db_aligned[(size_t)c * np + pt] = ntt_pts[pt * N + c];
}

/* gen_data (server.cpp:47-78) with seeded entries. */
void orc_build_db(const orc_ctx *ctx, uint64_t seed, uint64_t *db_aligned) {
  const orc_params *P = &ctx->P;
  const uint64_t chunk = 1024;
  uint8_t *ent = (uint8_t *)malloc(chunk * P->entries_per_pt * P->entry_size);
  uint64_t *pts = (uint64_t *)malloc(chunk * N * sizeof(uint64_t));
  for (uint64_t base = 0; base < P->num_pt; base += chunk) {
    uint64_t cnt = P->num_pt - base < chunk ? P->num_pt - base : chunk;
    orc_gen_entries(ctx, seed, base * P->entries_per_pt, cnt * P->entries_per_pt, ent);
    orc_pack_plaintexts(ctx, ent, cnt, pts);
    orc_plain_to_ntt(ctx, pts, cnt);
#pragma omp parallel for schedule(static)
    for (long c = 0; c < N; c++)
      for (uint64_t k = 0; k < cnt; k++)
        db_aligned[(size_t)c * P->num_pt + base + k] = pts[k * N + c];
  }
  free(ent);
  free(pts);
}

/* ------------------------------------------------------------------------ */
/* polynomial helpers                                                        */
/* ------------------------------------------------------------------------ */

/* Galois automorphism x -> x^g on one polynomial in coefficient form. */
static void automorph(const uint64_t *in, uint64_t g, uint64_t q, uint64_t *out) {
  for (uint64_t i = 0; i < N; i++) {
    uint64_t j = (i * g) & (2 * N - 1);
    if (j < N)
      out[j] = in[i];
    else
      out[j - N] = negmod(in[i], q);
  }
}

/* a * b mod (x^N + 1, q_mod), both in coefficient form */
static void polymul(const orc_ctx *ctx, int mod, const uint64_t *a, const uint64_t *b,
                    uint64_t *out) {
  const ntt_t *T = &ctx->nt[mod];
  uint64_t *A = (uint64_t *)malloc(2 * N * sizeof(uint64_t)), *B = A + N;
  memcpy(A, a, N * 8);
  memcpy(B, b, N * 8);
  ntt_fwd1(T, A);
  ntt_fwd1(T, B);
  for (size_t i = 0; i < N; i++) A[i] = mulmod(A[i], B[i], T->q);
  ntt_inv1(T, A);
  memcpy(out, A, N * 8);
  free(A);
}

static void small_to_mod(const int64_t *v, uint64_t q, uint64_t *out) {
  for (size_t i = 0; i < N; i++) out[i] = v[i] >= 0 ? (uint64_t)v[i] % q : negmod((uint64_t)(-v[i]) % q, q);
}

/* ------------------------------------------------------------------------ */
/* client (client.cpp) -- used only to produce queries/keys and to decrypt   */
/* ------------------------------------------------------------------------ */

void orc_keygen(const orc_ctx *ctx, uint64_t seed, int8_t *sk) {
  (void)ctx;
  rng_t r = {seed ^ 0x5EC12E7ULL};
  for (size_t i = 0; i < N; i++) sk[i] = (int8_t)((int)(rng_next(&r) % 3) - 1);
}

/* RLWE encryption of zero under sk mod q (coefficient form):
 * (-a*s + e, a).  SEAL encrypt_zero_symmetric semantics. */
static void enc_zero(const orc_ctx *ctx, int mod, const int8_t *sk, rng_t *r, uint64_t *ct) {
  const uint64_t q = ctx->nt[mod].q;
  int64_t tmp[N];
  uint64_t *s = (uint64_t *)malloc(2 * N * 8), *as = s + N;
  for (size_t i = 0; i < N; i++) tmp[i] = sk[i];
  small_to_mod(tmp, q, s);
  for (size_t i = 0; i < N; i++) ct[N + i] = rng_uniform(r, q);
  polymul(ctx, mod, ct + N, s, as);
  for (size_t i = 0; i < N; i++) {
    int64_t e = rng_cbd(r);
    uint64_t em = e >= 0 ? (uint64_t)e : q - (uint64_t)(-e);
    ct[i] = addmod(negmod(as[i], q), em % q, q);
  }
  free(s);
}

/* KeyGenerator::create_galois_keys for elements 1 + (N >> a), a < h
 * (client.cpp:227-241).  Key for element g, modulus m in {q, p}, NTT form:
 * k1 = a, k0 = -a*s + e + [m == q] (p mod q) * sigma_g(s). */
void orc_make_galois_keys(const orc_ctx *ctx, const int8_t *sk, uint64_t seed, uint64_t *keys) {
  const orc_params *P = &ctx->P;
  rng_t r = {seed ^ 0x6A101500ULL};
  int64_t s_i[N], sg_i[N], e_i[N];
  uint64_t sm[N], sgm[N], em[N], a[N];
  for (size_t i = 0; i < N; i++) s_i[i] = sk[i];
  for (uint64_t lv = 0; lv < P->h; lv++) {
    uint64_t g = 1 + (N >> lv);
    for (uint64_t i = 0; i < N; i++) {
      uint64_t j = (i * g) & (2 * N - 1);
      if (j < N)
        sg_i[j] = s_i[i];
      else
        sg_i[j - N] = -s_i[i];
    }
    for (size_t i = 0; i < N; i++) e_i[i] = rng_cbd(&r);
    for (int m = 0; m < 2; m++) {
      const ntt_t *T = &ctx->nt[m];
      const uint64_t q = T->q;
      uint64_t *k0 = keys + ((lv * 2 + 0) * 2 + (uint64_t)m) * N;
      uint64_t *k1 = keys + ((lv * 2 + 1) * 2 + (uint64_t)m) * N;
      small_to_mod(s_i, q, sm);
      small_to_mod(e_i, q, em);
      ntt_fwd1(T, sm);
      ntt_fwd1(T, em);
      for (size_t i = 0; i < N; i++) a[i] = rng_uniform(&r, q);
      for (size_t i = 0; i < N; i++) {
        k1[i] = a[i];
        k0[i] = addmod(negmod(mulmod(a[i], sm[i], q), q), em[i], q);
      }
      if (m == 0) {
        small_to_mod(sg_i, q, sgm);
        ntt_fwd1(T, sgm);
        uint64_t f = P->p % q;
        for (size_t i = 0; i < N; i++) k0[i] = addmod(k0[i], mulmod(f, sgm[i], q), q);
      }
    }
  }
}

/* RGSW(sk) with the key gadget (client.cpp:17-31, gsw_eval.cpp:339-405):
 * rows j < l_key:  (-a*s + e + g_j*s, a)
 * rows j >= l_key: (-a*s + e, a + g_j*s)          coefficient form mod q. */
void orc_make_gsw_key(const orc_ctx *ctx, const int8_t *sk, uint64_t seed, uint64_t *rows) {
  const orc_params *P = &ctx->P;
  const uint64_t q = P->q;
  rng_t r = {seed ^ 0x65500000ULL};
  uint64_t sm[N];
  int64_t s_i[N];
  for (size_t i = 0; i < N; i++) s_i[i] = sk[i];
  small_to_mod(s_i, q, sm);
  for (uint64_t j = 0; j < 2 * P->l_key; j++) {
    uint64_t *ct = rows + j * 2 * N;
    enc_zero(ctx, 0, sk, &r, ct);
    uint64_t half = j / P->l_key, lvl = j % P->l_key;
    uint64_t g = ctx->gadget_key[lvl];
    uint64_t *dst = ct + half * N;
    for (size_t i = 0; i < N; i++) dst[i] = addmod(dst[i], mulmod(g, sm[i], q), q);
  }
}

/* get_query_indices (client.cpp:38-53) */
void orc_query_indices(const orc_ctx *ctx, uint64_t pt_index, uint64_t *idx) {
  const orc_params *P = &ctx->P;
  uint64_t row = pt_index / P->n1, remain = P->num_pt / P->n1;
  idx[0] = pt_index % P->n1;
  for (uint64_t i = 1; i < P->ndim; i++) {
    remain /= 2;
    idx[i] = row / remain;
    row %= remain;
  }
}

/* fast_generate_query + add_gsw_to_query (client.cpp:130-209).  BFV
 * symmetric encryption with Delta*m = round(q*m/t). */
void orc_make_query(const orc_ctx *ctx, const int8_t *sk, uint64_t seed, uint64_t entry_index,
                    uint64_t *ct) {
  const orc_params *P = &ctx->P;
  const uint64_t q = P->q, t = P->t, w = 1ULL << P->h;
  uint64_t idx[64];
  orc_query_indices(ctx, entry_index / P->entries_per_pt, idx);
  rng_t r = {seed ^ 0x90E2700ULL};
  enc_zero(ctx, 0, sk, &r, ct);
  uint64_t inv_t = powmod(w % t, t - 2, t);
  uint64_t slot = brv(idx[0], (unsigned)P->h);
  uint64_t delta_m = (uint64_t)(((u128)q * inv_t + t / 2) / t);
  ct[slot] = addmod(ct[slot], delta_m % q, q);
  uint64_t inv_q = powmod(w % q, q - 2, q);
  for (uint64_t i = 1; i < P->ndim; i++) {
    if (idx[i] != 1) continue;
    for (uint64_t k = 0; k < P->l; k++) {
      uint64_t pos = P->n1 + (i - 1) * P->l + k;
      uint64_t rv = brv(pos, (unsigned)P->h);
      uint64_t coef = mulmod(ctx->gadget[k], inv_q, q);
      ct[rv] = addmod(ct[rv], coef, q);
    }
  }
}

/* decrypt_mod_q + invariant_noise_budget (client.cpp:458-479), at modulus
 * q (mod = 0) or small_q (mod = 2). */
void orc_decrypt(const orc_ctx *ctx, const int8_t *sk, const uint64_t *ct, int mod,
                 uint64_t *plain, int *noise_budget) {
  const uint64_t Q = ctx->nt[mod].q, t = ctx->P.t;
  uint64_t c0[N], c1[N], s[N], phase[N];
  int64_t s_i[N];
  for (size_t i = 0; i < N; i++) {
    c0[i] = ct[i] % Q;
    c1[i] = ct[N + i] % Q;
    s_i[i] = sk[i];
  }
  small_to_mod(s_i, Q, s);
  polymul(ctx, mod, c1, s, phase);
  uint64_t norm = 0;
  for (size_t i = 0; i < N; i++) {
    uint64_t ph = addmod(phase[i], c0[i], Q);
    plain[i] = (uint64_t)((((u128)ph * t) + Q / 2) / Q) % t;
    uint64_t v = mulmod(ph, t, Q);
    uint64_t a = v > Q / 2 ? Q - v : v;
    if (a > norm) norm = a;
  }
  if (noise_budget) {
    int b = (int)bitlen64(Q) - (int)bitlen64(norm) - 1;
    *noise_budget = b > 0 ? b : 0;
  }
}

/* get_entry_from_plaintext (client.cpp:255-287) */
void orc_entry_from_plain(const orc_ctx *ctx, uint64_t entry_index, const uint64_t *plain,
                          uint8_t *entry) {
  const orc_params *P = &ctx->P;
  uint64_t start = (entry_index % P->entries_per_pt) * P->entry_size * 8;
  uint64_t bpc = P->bits_per_coeff;
  uint64_t ci = start / bpc, off = start % bpc;
  u128 buf = plain[ci] >> off;
  u128 have = bpc - off;
  uint64_t n = 0;
  while (n < P->entry_size) {
    if (have >= 8) {
      entry[n++] = (uint8_t)(buf & 0xFF);
      buf >>= 8;
      have -= 8;
    } else {
      ci++;
      u128 nb = ci < N ? plain[ci] : 0;
      buf |= nb << have;
      have += bpc;
    }
  }
}

/* load_resp_from_stream (client.cpp:364-412) */
void orc_unpack_response(const orc_ctx *ctx, const uint8_t *bytes, uint64_t *ct) {
  const uint64_t w = ctx->P.small_q_width;
  uint64_t bitpos = 0;
  for (size_t i = 0; i < 2 * N; i++) {
    uint64_t v = 0;
    for (uint64_t j = 0; j < w; j++, bitpos++) v |= (uint64_t)((bytes[bitpos >> 3] >> (bitpos & 7)) & 1) << j;
    ct[i] = v;
  }
}

/* ------------------------------------------------------------------------ */
/* server query path                                                          */
/* ------------------------------------------------------------------------ */

/* utils::shift_polynomial / negacyclic_shift_poly_coeffmod (utils.cpp:6-40),
 * called with index = (size_t)(-k) from server.cpp:422.  Zero coefficients
 * stay zero, wrapped non-zero v becomes q - v. */
void orc_negacyclic_shift(const orc_ctx *ctx, const uint64_t *ct, int64_t k, uint64_t *out) {
  const uint64_t q = ctx->P.q;
  const uint64_t shift = (uint64_t)k;
  for (int poly = 0; poly < 2; poly++) {
    const uint64_t *in = ct + poly * N;
    uint64_t *o = out + poly * N;
    if (shift == 0) {
      memcpy(o, in, N * 8);
      continue;
    }
    uint64_t raw = shift;
    for (size_t i = 0; i < N; i++, raw++) {
      uint64_t index = raw & (N - 1);
      if (!(raw & N) || !in[i])
        o[index] = in[i];
      else
        o[index] = q - in[i];
    }
  }
}

/* Evaluator::apply_galois_inplace (server.cpp:409) for a BFV ciphertext in
 * coefficient form with one data prime q and special prime p:
 *   T = sigma_g(c1);  X_k = T * K_k over {q, p} (NTT domain);
 *   ks_k = round(X_k / p) mod q = (x_q + p/2 - ((x_p + p/2) mod p)) * p^-1;
 *   out = (sigma_g(c0) + ks_0, ks_1). */
void orc_apply_galois(const orc_ctx *ctx, const uint64_t *ct, uint64_t g, const uint64_t *key,
                      uint64_t *out) {
  const uint64_t q = ctx->P.q, p = ctx->P.p;
  const ntt_t *Tq = &ctx->nt[0], *Tp = &ctx->nt[1];
  uint64_t *buf = (uint64_t *)malloc(6 * N * 8);
  uint64_t *tq = buf, *tp = buf + N, *aq = buf + 2 * N, *ap = buf + 3 * N, *s0 = buf + 4 * N;
  automorph(ct, g, q, s0);
  automorph(ct + N, g, q, tq);
  for (size_t i = 0; i < N; i++) tp[i] = tq[i] >= p ? tq[i] - p : tq[i];
  ntt_fwd1(Tq, tq);
  ntt_fwd1(Tp, tp);
  const uint64_t ph = ctx->p_half;
  for (int k = 0; k < 2; k++) {
    const uint64_t *kq = key + (2 * k + 0) * N, *kp = key + (2 * k + 1) * N;
    for (size_t i = 0; i < N; i++) {
      aq[i] = mulmod(tq[i], kq[i], q);
      ap[i] = mulmod(tp[i], kp[i], p);
    }
    ntt_inv1(Tq, aq);
    ntt_inv1(Tp, ap);
    for (size_t i = 0; i < N; i++) {
      uint64_t rr = addmod(ap[i], ph, p);
      uint64_t v = submod(addmod(aq[i], ph % q, q), rr % q, q);
      v = mul_shoup(v, ctx->p_inv_q, ctx->p_inv_q_s, q);
      if (k == 0)
        out[i] = addmod(s0[i], v, q);
      else
        out[N + i] = v;
    }
  }
  free(buf);
}

/* fast_expand_qry (server.cpp:383-428): heap-order expansion, root at slot 1,
 * subtrees whose left-most leaf is >= u are skipped.  Returns leaves
 * w .. w+u-1 as u ciphertexts. */
void orc_expand(const orc_ctx *ctx, const uint64_t *query, const uint64_t *galois_keys,
                uint64_t *leaves) {
  const orc_params *P = &ctx->P;
  const uint64_t h = P->h, w = 1ULL << h, u = P->u;
  const size_t CT = 2 * N;
  uint64_t *cur = (uint64_t *)malloc(w * CT * 8), *nxt = (uint64_t *)malloc(w * CT * 8);
  memcpy(cur, query, CT * 8);
  for (uint64_t a = 0; a < h; a++) {
    const uint64_t k = 1ULL << a, first = k; /* nodes [k, 2k) */
    const uint64_t *key = galois_keys + a * 4 * N;
#pragma omp parallel for schedule(dynamic, 1)
    for (long ii = 0; ii < (long)k; ii++) {
      uint64_t i = first + (uint64_t)ii;
      uint64_t left_leaf = i * w / k - w;
      if (left_leaf >= u) continue;
      const uint64_t *ci = cur + (uint64_t)ii * CT;
      uint64_t *c_even = nxt + 2 * (uint64_t)ii * CT, *c_odd = c_even + CT;
      uint64_t *cp = (uint64_t *)malloc(2 * CT * 8), *diff = cp + CT;
      orc_apply_galois(ctx, ci, N / k + 1, key, cp);
      for (size_t j = 0; j < CT; j++) {
        c_even[j] = addmod(ci[j], cp[j], P->q);
        diff[j] = submod(ci[j], cp[j], P->q);
      }
      orc_negacyclic_shift(ctx, diff, -(int64_t)k, c_odd);
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

/* set_client_gsw_key (server.cpp:486-500): rows to NTT form. */
void orc_gsw_key_to_ntt(const orc_ctx *ctx, const uint64_t *rows_coeff, uint64_t rows,
                        uint64_t *rows_ntt) {
  memcpy(rows_ntt, rows_coeff, rows * 2 * N * 8);
  orc_ntt_fwd(ctx, 0, rows_ntt, rows * 2);
}

/* GSWEval::external_product (gsw_eval.cpp:33-106) with
 * decomp_rlwe_single_mod (184-224) and decomp_to_ntt (226-252).  Output in
 * NTT form. */
void orc_ext_product(const orc_ctx *ctx, const uint64_t *gsw, uint64_t l, uint64_t base_log2,
                     const uint64_t *ct, uint64_t *out) {
  const ntt_t *T = &ctx->nt[0];
  const uint64_t mask = (1ULL << base_log2) - 1;
  u128 *acc = (u128 *)calloc(2 * N, sizeof(u128));
  uint64_t *d = (uint64_t *)malloc(N * 8);
  for (uint64_t poly = 0; poly < 2; poly++) {
    for (uint64_t pp = l; pp-- > 0;) {
      uint64_t j = poly * l + (l - 1 - pp);
      uint64_t sh = pp * base_log2;
      for (size_t c = 0; c < N; c++) d[c] = (ct[poly * N + c] >> sh) & mask;
      ntt_fwd1(T, d);
      const uint64_t *g0 = gsw + j * 2 * N, *g1 = g0 + N;
      for (size_t c = 0; c < N; c++) {
        acc[c] += (u128)d[c] * g0[c];
        acc[N + c] += (u128)d[c] * g1[c];
      }
    }
  }
  for (size_t c = 0; c < 2 * N; c++) out[c] = barrett128(acc[c], &T->br);
  free(acc);
  free(d);
}

/* GSWEval::query_to_gsw (gsw_eval.cpp:254-286): rows 0..l-1 = NTT(ct_i),
 * rows l..2l-1 = external_product(key, ct_i) with the key gadget. */
void orc_query_to_gsw(const orc_ctx *ctx, const uint64_t *cts, const uint64_t *key,
                      uint64_t *out) {
  const orc_params *P = &ctx->P;
  const size_t CT = 2 * N;
  for (uint64_t i = 0; i < P->l; i++) {
    memcpy(out + i * CT, cts + i * CT, CT * 8);
    ntt_fwd1(&ctx->nt[0], out + i * CT);
    ntt_fwd1(&ctx->nt[0], out + i * CT + N);
  }
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)P->l; i++)
    orc_ext_product(ctx, key, P->l_key, P->base_log2_key, cts + (size_t)i * CT,
                    out + (P->l + (size_t)i) * CT);
}

/* evaluate_first_dim (server.cpp:124-175): NTT the n1 selection ciphertexts,
 * C[c] = A[c] (n_rest x n1) * B[c] (n1 x 2) per coefficient
 * (matrix.cpp:79-97, 220-235), reduce mod q and INTT each result
 * (delay_modulus, server.cpp:178-293).  Sums are exact: an accumulator that
 * would wrap mod 2^128 in the reference is carried, and the function returns
 * the number of such wraps (0 means bit-identical to the reference loop). */
int orc_first_dim(const orc_ctx *ctx, const uint64_t *db, const uint64_t *fst, uint64_t *out) {
  const orc_params *P = &ctx->P;
  const uint64_t n1 = P->n1, nr = P->n_rest, np = P->num_pt;
  const size_t CT = 2 * N;
  const barrett_t *br = &ctx->nt[0].br;
  uint64_t *qn = (uint64_t *)malloc(n1 * CT * 8);
  memcpy(qn, fst, n1 * CT * 8);
  orc_ntt_fwd(ctx, 0, qn, 2 * n1);
  /* prep_query (server.cpp:80-118): Q[c][k][poly] */
  uint64_t *Q = (uint64_t *)malloc(n1 * CT * 8);
#pragma omp parallel for schedule(static)
  for (long c = 0; c < N; c++)
    for (uint64_t k = 0; k < n1; k++) {
      Q[(size_t)c * 2 * n1 + 2 * k] = qn[k * CT + (size_t)c];
      Q[(size_t)c * 2 * n1 + 2 * k + 1] = qn[k * CT + N + (size_t)c];
    }
  long wraps = 0;
#pragma omp parallel for schedule(static) reduction(+ : wraps)
  for (long c = 0; c < N; c++) {
    const uint64_t *A = db + (size_t)c * np, *B = Q + (size_t)c * 2 * n1;
    for (uint64_t row = 0; row < nr; row++) {
      u128 t0 = 0, t1 = 0;
      uint64_t w0 = 0, w1 = 0;
      const uint64_t *a = A + row * n1;
      for (uint64_t k = 0; k < n1; k++) {
        u128 p0 = (u128)a[k] * B[2 * k], p1 = (u128)a[k] * B[2 * k + 1];
        t0 += p0;
        w0 += t0 < p0;
        t1 += p1;
        w1 += t1 < p1;
      }
      wraps += (long)(w0 + w1);
      uint64_t r0 = addmod(reduce128_full(t0, br), mulmod(w0, br->r128, P->q), P->q);
      uint64_t r1 = addmod(reduce128_full(t1, br), mulmod(w1, br->r128, P->q), P->q);
      out[row * CT + (size_t)c] = r0;
      out[row * CT + N + (size_t)c] = r1;
    }
  }
  orc_ntt_inv(ctx, 0, out, 2 * nr);
  free(qn);
  free(Q);
  return (int)(wraps > 0x7fffffff ? 0x7fffffff : wraps);
}

/* Same as orc_first_dim but with the reference's wrapping uint128 sums
 * (mat_mat_128, matrix.cpp:220-235), for the exact-vs-wrapping tests.  The
 * CPU baseline times orc_make_query_server, whose first dimension is the
 * exact orc_first_dim: the same loop nest plus one carry count per MAC. */
void orc_first_dim_wrapping(const orc_ctx *ctx, const uint64_t *db, const uint64_t *fst,
                            uint64_t *out) {
  const orc_params *P = &ctx->P;
  const uint64_t n1 = P->n1, nr = P->n_rest, np = P->num_pt;
  const size_t CT = 2 * N;
  const barrett_t *br = &ctx->nt[0].br;
  uint64_t *qn = (uint64_t *)malloc(n1 * CT * 8);
  memcpy(qn, fst, n1 * CT * 8);
  orc_ntt_fwd(ctx, 0, qn, 2 * n1);
  uint64_t *Q = (uint64_t *)malloc(n1 * CT * 8);
#pragma omp parallel for schedule(static)
  for (long c = 0; c < N; c++)
    for (uint64_t k = 0; k < n1; k++) {
      Q[(size_t)c * 2 * n1 + 2 * k] = qn[k * CT + (size_t)c];
      Q[(size_t)c * 2 * n1 + 2 * k + 1] = qn[k * CT + N + (size_t)c];
    }
  u128 *inter = (u128 *)malloc(nr * 2 * sizeof(u128) * N);
#pragma omp parallel for schedule(static)
  for (long c = 0; c < N; c++) {
    const uint64_t *A = db + (size_t)c * np, *B = Q + (size_t)c * 2 * n1;
    u128 *C = inter + (size_t)c * 2 * nr;
    for (uint64_t row = 0; row < nr; row++) {
      u128 t0 = 0, t1 = 0;
      const uint64_t *a = A + row * n1;
      for (uint64_t k = 0; k < n1; k++) {
        t0 += a[k] * (u128)B[2 * k];
        t1 += a[k] * (u128)B[2 * k + 1];
      }
      C[2 * row] = t0;
      C[2 * row + 1] = t1;
    }
  }
#pragma omp parallel for schedule(static)
  for (long row = 0; row < (long)nr; row++)
    for (size_t c = 0; c < N; c++) {
      out[(size_t)row * CT + c] = reduce128_full(inter[c * 2 * nr + 2 * (size_t)row], br);
      out[(size_t)row * CT + N + c] = reduce128_full(inter[c * 2 * nr + 2 * (size_t)row + 1], br);
    }
  orc_ntt_inv(ctx, 0, out, 2 * nr);
  free(inter);
  free(qn);
  free(Q);
}

/* other_dim_mux (server.cpp:295-334): result[i] += INTT(RGSW(b) x (y - x)). */
void orc_other_dim_mux(const orc_ctx *ctx, uint64_t *result, uint64_t count, const uint64_t *gsw) {
  const orc_params *P = &ctx->P;
  const uint64_t half = count / 2, q = P->q;
  const size_t CT = 2 * N;
#pragma omp parallel for schedule(dynamic, 1)
  for (long i = 0; i < (long)half; i++) {
    uint64_t *x = result + (size_t)i * CT, *y = result + ((size_t)i + half) * CT;
    for (size_t c = 0; c < CT; c++) y[c] = submod(y[c], x[c], q);
    uint64_t *tmp = (uint64_t *)malloc(CT * 8);
    orc_ext_product(ctx, gsw, P->l, P->base_log2, y, tmp);
    ntt_inv1(&ctx->nt[0], tmp);
    ntt_inv1(&ctx->nt[0], tmp + N);
    for (size_t c = 0; c < CT; c++) x[c] = addmod(x[c], tmp[c], q);
    free(tmp);
  }
}

static unsigned bitlen128(u128 x) {
  uint64_t hi = (uint64_t)(x >> 64);
  return hi ? 64 + bitlen64(hi) : bitlen64((uint64_t)x);
}

/* mod_switch_inplace (server.cpp:779-801): (uint64_t)round((long double)x *
 * (long double)((double)small_q / (double)q)).  The long double product is
 * the x87 64-bit-significand product (round-to-nearest-even), round() is
 * half-away-from-zero; both are done here in integers on x * M * 2^E where
 * M * 2^E is the double scale. */
uint64_t orc_mod_switch_coeff(const orc_ctx *ctx, uint64_t x) {
  const uint64_t M = ctx->P.ms_mant;
  const int64_t E = ctx->P.ms_exp;
  if (x == 0) return 0;
  u128 P = (u128)x * M;
  unsigned b = bitlen128(P);
  if (b > 64) {
    unsigned sh = b - 64;
    u128 keep = P >> sh, rem = P & (((u128)1 << sh) - 1), half = (u128)1 << (sh - 1);
    if (rem > half || (rem == half && (keep & 1))) keep++;
    P = keep << sh;
  }
  if (E >= 0) return (uint64_t)(P << E);
  unsigned s = (unsigned)(-E);
  if (s >= 127) return 0;
  return (uint64_t)((P + ((u128)1 << (s - 1))) >> s);
}

void orc_mod_switch(const orc_ctx *ctx, uint64_t *ct) {
  for (size_t i = 0; i < 2 * N; i++) ct[i] = orc_mod_switch_coeff(ctx, ct[i]);
}

/* x87 long double evaluation of the same expression, where the host has it
 * (x86-64); used by the tests to pin the integer emulation. */
int orc_x87_mod_switch(const orc_ctx *ctx, uint64_t x, uint64_t *out) {
#if defined(__x86_64__) || defined(__i386__)
  const long double scale = (double)ctx->P.small_q / (double)ctx->P.q;
  *out = (uint64_t)roundl((long double)x * scale);
  return 1;
#else
  (void)ctx;
  (void)x;
  (void)out;
  return 0;
#endif
}

uint64_t orc_response_bytes(const orc_ctx *ctx) {
  return (2 * N * ctx->P.small_q_width + 7) / 8;
}

/* save_resp_to_stream (server.cpp:581-633): LSB-first packing of c0 then c1
 * at small_q_width bits, each coefficient masked to that width. */
uint64_t orc_pack_response(const orc_ctx *ctx, const uint64_t *ct, uint8_t *out) {
  const uint64_t w = ctx->P.small_q_width, nbytes = orc_response_bytes(ctx);
  memset(out, 0, nbytes);
  uint64_t bitpos = 0;
  for (size_t i = 0; i < 2 * N; i++) {
    uint64_t v = ct[i] & ((1ULL << w) - 1);
    for (uint64_t j = 0; j < w; j++, bitpos++)
      out[bitpos >> 3] |= (uint8_t)(((v >> j) & 1) << (bitpos & 7));
  }
  return nbytes;
}

static double now_ms(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

/* PirServer::make_query (server.cpp:520-579) followed by save_resp_to_stream.
 * gsw_key_ntt: the client's RGSW(sk) already in NTT form (server.cpp:497).
 * stage_ms (optional, 5 entries): Expand, Convert, First dim, Other dim,
 * Mod switch -- the reference's TIME_START sections.  Returns the number of
 * first-dimension accumulator wraps (see orc_first_dim). */
int orc_make_query_server(const orc_ctx *ctx, const uint64_t *db, const uint64_t *galois_keys,
                          const uint64_t *gsw_key_ntt, const uint64_t *query, uint64_t *resp,
                          uint8_t *packed, double *stage_ms) {
  const orc_params *P = &ctx->P;
  const size_t CT = 2 * N;
  const uint64_t dims = P->ndim;
  double t0 = now_ms();
  uint64_t *leaves = (uint64_t *)malloc(P->u * CT * 8);
  orc_expand(ctx, query, galois_keys, leaves);
  double t1 = now_ms();
  uint64_t *gsw = (uint64_t *)malloc((dims > 1 ? dims - 1 : 1) * 2 * P->l * CT * 8);
  for (uint64_t i = 1; i < dims; i++)
    orc_query_to_gsw(ctx, leaves + (P->n1 + (i - 1) * P->l) * CT, gsw_key_ntt,
                     gsw + (i - 1) * 2 * P->l * CT);
  double t2 = now_ms();
  uint64_t *res = (uint64_t *)malloc(P->n_rest * CT * 8);
  int wraps = orc_first_dim(ctx, db, leaves, res);
  double t3 = now_ms();
  uint64_t cnt = P->n_rest;
  for (uint64_t i = 1; i < dims; i++) {
    orc_other_dim_mux(ctx, res, cnt, gsw + (i - 1) * 2 * P->l * CT);
    cnt /= 2;
  }
  double t4 = now_ms();
  memcpy(resp, res, CT * 8);
  orc_mod_switch(ctx, resp);
  if (packed) orc_pack_response(ctx, resp, packed);
  double t5 = now_ms();
  if (stage_ms) {
    stage_ms[0] = t1 - t0;
    stage_ms[1] = t2 - t1;
    stage_ms[2] = t3 - t2;
    stage_ms[3] = t4 - t3;
    stage_ms[4] = t5 - t4;
  }
  free(leaves);
  free(gsw);
  free(res);
  return wraps;
}
