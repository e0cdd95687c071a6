/*
 * opir_oracle_rns.h -- CPU oracle for the multi-modulus OnionPIRv2 server
 * path (rns_mod_cnt > 1: the PolyDegree = 4096, CoeffMods = {60, 60, 60}
 * presets of src/includes/database_constants.h:13-172).
 *
 * TEST INFRASTRUCTURE ONLY.  A plain-C restatement, generic in the
 * polynomial degree N and the number R (1 or 2) of ciphertext primes, of the
 * reference server (src/server.cpp), the RGSW evaluator with the CRT
 * decomposition (src/gsw_eval.cpp:108-182), the modulus switch to the next
 * level (server.cpp:567-570) and of the client (src/client.cpp), with the
 * SEAL 4.1 primitives restated from BFV/RGSW mathematics.  Only tests, the
 * smoke check and the CPU-baseline leg of the benchmark may load it.
 *
 * Parity status: PARTIALLY PINNED, as the single-modulus oracle
 * (opir_oracle.h).  At N = 2048, R = 1 this file reproduces opir_oracle.c
 * bit for bit (keys, queries, every server stage), which the tests check; at
 * R = 2 what is pinned is the reference's end-to-end criterion (decrypted
 * entry == database entry) and the CRT identities; SEAL's multi-modulus
 * conventions (RNS key-switching decomposition, divide-and-round by the last
 * prime, plaintext lift per prime) are restated from public descriptions.
 *
 * Layouts follow SEAL's in-memory order (poly, then prime, then coefficient):
 *   ciphertext      [2][R][N]           coefficient form
 *   GSW ciphertext  [rows][2][R][N]     gsw_eval.h:8 (NTT form on the server)
 *   aligned DB      [R*N][num_pt]       db_aligned_[c*num_pt + row*n1 + col]
 *   galois keys     [h][R][2][R+1][N]   level a, decomposition prime j, key
 *                                       poly k, modulus (q_0..q_{R-1}, p), NTT
 *   response        [2][N]              mod small_q after both switches
 */
#ifndef OPIR_ORACLE_RNS_H
#define OPIR_ORACLE_RNS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORR_MAX_RNS 2

typedef struct orr_params {
  uint64_t n, logn, rns;           /* N, log2 N, ciphertext primes R */
  uint64_t q[ORR_MAX_RNS];         /* ciphertext primes q_0 .. q_{R-1} */
  uint64_t p;                      /* SEAL special (key-switching) prime */
  uint64_t t, small_q, small_q_width;
  uint64_t l, base_log2, l_key, base_log2_key;
  uint64_t num_entries, num_pt, entry_size, entries_per_pt, bits_per_coeff;
  uint64_t n1, n_rest, ndim, u, h;
  uint64_t ms_mant;                /* (double)small_q / (double)q_0 == ms_mant * 2^ms_exp */
  int64_t ms_exp;
} orr_params;

typedef struct orr_ctx orr_ctx;

/* PirParams (pir.cpp:9-95) for N, plain_bits, small_q_width and
 * coeff_bits[0 .. R] (the last entry is the special prime). */
orr_ctx *orr_create(uint64_t n, uint64_t num_entries, uint64_t max_fst_dim, uint64_t entry_size,
                    uint64_t l, uint64_t l_key, uint64_t plain_bits, uint64_t small_q_width,
                    const uint64_t *coeff_bits, uint64_t coeff_count);
void orr_destroy(orr_ctx *ctx);
void orr_get_params(const orr_ctx *ctx, orr_params *out);

/* negacyclic NTT of `count` polynomials; mod: 0..R-1 = q_i, R = p, R+1 = small_q */
void orr_ntt_fwd(const orr_ctx *ctx, int mod, uint64_t *a, size_t count);
void orr_ntt_inv(const orr_ctx *ctx, int mod, uint64_t *a, size_t count);

/* ---- database ---- */
void orr_gen_entries(const orr_ctx *ctx, uint64_t seed, uint64_t first, uint64_t count,
                     uint8_t *out);
void orr_build_db(const orr_ctx *ctx, uint64_t seed, uint64_t *db_aligned);

/* ---- client ---- */
void orr_keygen(const orr_ctx *ctx, uint64_t seed, int8_t *sk);
void orr_make_galois_keys(const orr_ctx *ctx, const int8_t *sk, uint64_t seed, uint64_t *keys);
void orr_make_gsw_key(const orr_ctx *ctx, const int8_t *sk, uint64_t seed, uint64_t *rows);
void orr_make_query(const orr_ctx *ctx, const int8_t *sk, uint64_t seed, uint64_t entry_index,
                    uint64_t *ct);
void orr_decrypt_small(const orr_ctx *ctx, const int8_t *sk, const uint64_t *ct, uint64_t *plain,
                       int *noise_budget);
void orr_entry_from_plain(const orr_ctx *ctx, uint64_t entry_index, const uint64_t *plain,
                          uint8_t *entry);

/* ---- server ---- */
void orr_apply_galois(const orr_ctx *ctx, const uint64_t *ct, uint64_t galois_elt,
                      const uint64_t *key, uint64_t *out);
void orr_expand(const orr_ctx *ctx, const uint64_t *query, const uint64_t *galois_keys,
                uint64_t *leaves);
void orr_gsw_to_ntt(const orr_ctx *ctx, const uint64_t *rows_coeff, uint64_t rows,
                    uint64_t *rows_ntt);
/* decomp_rlwe (gsw_eval.cpp:108-182): [2l][R][N] digits, coefficient form */
void orr_decompose(const orr_ctx *ctx, const uint64_t *ct, uint64_t l, uint64_t base_log2,
                   uint64_t *digits);
void orr_ext_product(const orr_ctx *ctx, const uint64_t *gsw_ntt, uint64_t l, uint64_t base_log2,
                     const uint64_t *ct, uint64_t *out_ntt);
void orr_query_to_gsw(const orr_ctx *ctx, const uint64_t *cts, const uint64_t *key_ntt,
                      uint64_t *out);
int orr_first_dim(const orr_ctx *ctx, const uint64_t *db_aligned, const uint64_t *fst,
                  uint64_t *out);
void orr_other_dim_mux(const orr_ctx *ctx, uint64_t *result, uint64_t count,
                       const uint64_t *gsw_ntt);
/* Evaluator::mod_switch_to_next_inplace (server.cpp:569): [2][R][N] -> [2][R-1][N] */
void orr_mod_switch_next(const orr_ctx *ctx, const uint64_t *ct, uint64_t *out);
uint64_t orr_mod_switch_coeff(const orr_ctx *ctx, uint64_t x);
uint64_t orr_response_bytes(const orr_ctx *ctx);
uint64_t orr_pack_response(const orr_ctx *ctx, const uint64_t *ct, uint8_t *out);
int orr_make_query_server(const orr_ctx *ctx, const uint64_t *db_aligned,
                          const uint64_t *galois_keys, const uint64_t *gsw_key_ntt,
                          const uint64_t *query, uint64_t *resp, uint8_t *packed);

#ifdef __cplusplus
}
#endif
#endif
