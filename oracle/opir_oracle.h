/*
 * opir_oracle.h -- CPU oracle for the OnionPIRv2 server query path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * server (src/server.cpp), the RGSW evaluator (src/gsw_eval.cpp), the level
 * mat-mat kernel (src/matrix.cpp), the parameter derivation (src/pir.cpp),
 * the client (src/client.cpp) and of the SEAL 4.1 primitives those call,
 * restated from BFV/RGSW mathematics.  Only tests, the smoke check and the
 * CPU-baseline leg of the benchmark may load it; the GPU product never does.
 *
 * Parity status: PARTIALLY PINNED.  The reference ships no golden vectors
 * and cannot be built here (it needs a SEAL 4.1 fork that is not present).
 * What is pinned:
 *   - the reference's own end-to-end criterion (decrypted entry == database
 *     entry, src/tests.cpp:110-134) over seeded queries;
 *   - the x87 long-double rounding of mod_switch_inplace (server.cpp:795-799),
 *     checked against the host's real long double on x86-64;
 *   - mathematical identities of every primitive (NTT round trip and
 *     evaluation semantics, negacyclic convolution, key-switch correctness).
 * What is unpinned: SEAL-internal conventions (prime order, NTT root and
 * ordering, plaintext lift, key-switch rounding), restated from public
 * descriptions of SEAL.
 *
 * Layouts follow the reference (rns_mod_cnt == 1):
 *   ciphertext      [2][N]            poly-major (c0 then c1), coefficient form
 *   GSW ciphertext  [rows][2][N]      gsw_eval.h:8, seal_GSW_vec_to_GSW
 *   aligned DB      [N][num_pt]       db_aligned_[c*num_pt + row*n1 + col]
 *                                      (server.cpp:740)
 *   galois keys     [h][2][2][N]      level a (galois elt N/2^a+1), key poly k,
 *                                      modulus (0 = q, 1 = p), NTT form
 */
#ifndef OPIR_ORACLE_H
#define OPIR_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_N 2048
#define ORC_LOGN 11

typedef struct orc_params {
  uint64_t poly_degree;      /* N */
  uint64_t q;                /* ciphertext modulus q0 (60-bit) */
  uint64_t p;                /* SEAL special (key-switching) prime */
  uint64_t t;                /* plaintext modulus */
  uint64_t small_q;          /* modulus-switching target */
  uint64_t small_q_width;    /* ceil(log2(small_q)) */
  uint64_t l, base_log2;     /* data RGSW gadget */
  uint64_t l_key, base_log2_key;  /* key RGSW gadget */
  uint64_t num_entries;      /* padded */
  uint64_t num_pt;
  uint64_t entry_size;       /* bytes */
  uint64_t entries_per_pt;
  uint64_t bits_per_coeff;
  uint64_t n1;               /* first dimension */
  uint64_t n_rest;           /* other_dim_sz = 2^(ndim-1) */
  uint64_t ndim;
  uint64_t u;                /* useful expansion leaves n1 + l*(ndim-1) */
  uint64_t h;                /* expansion height */
  /* mod-switch constants: (double)small_q/(double)q == m * 2^e, m odd-free 53-bit */
  uint64_t ms_mant;
  int64_t ms_exp;
} orc_params;

typedef struct orc_ctx orc_ctx;

/* ---- context / parameters (pir.cpp:9-95, database_constants.h) ---- */
orc_ctx *orc_create(uint64_t num_entries, uint64_t max_fst_dim, uint64_t entry_size,
                    uint64_t l, uint64_t l_key, uint64_t plain_bits,
                    uint64_t small_q_width, uint64_t coeff_bits0, uint64_t coeff_bits1);
void orc_destroy(orc_ctx *ctx);
void orc_get_params(const orc_ctx *ctx, orc_params *out);
int orc_set_threads(int n);   /* OpenMP threads for the batched loops; returns previous */

/* ---- number theory helpers ---- */
int orc_is_prime(uint64_t n);
uint64_t orc_generate_prime(uint64_t bit_width);                 /* utils.cpp:82-95 */
int orc_coeff_modulus_create(uint64_t n, const uint64_t *bits, size_t count, uint64_t *out);
uint64_t orc_minimal_root(uint64_t q, uint64_t two_n);
uint64_t orc_barrett_reduce_128(uint64_t lo, uint64_t hi, uint64_t q);

/* ---- negacyclic NTT, mod: 0 = q, 1 = p, 2 = small_q ---- */
void orc_ntt_fwd(const orc_ctx *ctx, int mod, uint64_t *a, size_t count);
void orc_ntt_inv(const orc_ctx *ctx, int mod, uint64_t *a, size_t count);
/* twiddle tables as stored (psi^brv(i), psi^-brv(i)), for device upload checks */
void orc_ntt_tables(const orc_ctx *ctx, int mod, uint64_t *fwd, uint64_t *inv, uint64_t *psi,
                    uint64_t *n_inv);

/* ---- database (server.cpp:47-78, 635-748, utils.cpp:98-104,160-172) ---- */
void orc_gen_entries(const orc_ctx *ctx, uint64_t seed, uint64_t first_entry, uint64_t count,
                     uint8_t *out);
void orc_pack_plaintexts(const orc_ctx *ctx, const uint8_t *entries, uint64_t num_pt,
                         uint64_t *coeffs);
void orc_plain_to_ntt(const orc_ctx *ctx, uint64_t *coeffs, uint64_t num_pt);
void orc_realign(const orc_ctx *ctx, const uint64_t *ntt_pts, uint64_t *db_aligned);
void orc_build_db(const orc_ctx *ctx, uint64_t seed, uint64_t *db_aligned);

/* ---- client side (client.cpp) ---- */
void orc_keygen(const orc_ctx *ctx, uint64_t seed, int8_t *sk);
void orc_make_galois_keys(const orc_ctx *ctx, const int8_t *sk, uint64_t seed, uint64_t *keys);
void orc_make_gsw_key(const orc_ctx *ctx, const int8_t *sk, uint64_t seed, uint64_t *rows);
void orc_query_indices(const orc_ctx *ctx, uint64_t pt_index, uint64_t *indices);
void orc_make_query(const orc_ctx *ctx, const int8_t *sk, uint64_t seed, uint64_t entry_index,
                    uint64_t *ct);
void orc_decrypt(const orc_ctx *ctx, const int8_t *sk, const uint64_t *ct, int mod,
                 uint64_t *plain, int *noise_budget);
void orc_entry_from_plain(const orc_ctx *ctx, uint64_t entry_index, const uint64_t *plain,
                          uint8_t *entry);
void orc_unpack_response(const orc_ctx *ctx, const uint8_t *bytes, uint64_t *ct);

/* ---- server query path (server.cpp:295-579, gsw_eval.cpp, utils.cpp) ---- */
void orc_negacyclic_shift(const orc_ctx *ctx, const uint64_t *ct, int64_t k, uint64_t *out);
void orc_apply_galois(const orc_ctx *ctx, const uint64_t *ct, uint64_t galois_elt,
                      const uint64_t *key, uint64_t *out);
void orc_expand(const orc_ctx *ctx, const uint64_t *query, const uint64_t *galois_keys,
                uint64_t *leaves);
void orc_gsw_key_to_ntt(const orc_ctx *ctx, const uint64_t *rows_coeff, uint64_t rows,
                        uint64_t *rows_ntt);
void orc_ext_product(const orc_ctx *ctx, const uint64_t *gsw_ntt, uint64_t l, uint64_t base_log2,
                     const uint64_t *ct, uint64_t *out_ntt);
void orc_query_to_gsw(const orc_ctx *ctx, const uint64_t *cts, const uint64_t *key_gsw_ntt,
                      uint64_t *out);
int orc_first_dim(const orc_ctx *ctx, const uint64_t *db_aligned, const uint64_t *fst_cts,
                  uint64_t *out);
void orc_first_dim_wrapping(const orc_ctx *ctx, const uint64_t *db_aligned,
                            const uint64_t *fst_cts, uint64_t *out);
void orc_other_dim_mux(const orc_ctx *ctx, uint64_t *result, uint64_t count,
                       const uint64_t *gsw_ntt);
void orc_mod_switch(const orc_ctx *ctx, uint64_t *ct);
uint64_t orc_mod_switch_coeff(const orc_ctx *ctx, uint64_t x);
int orc_x87_mod_switch(const orc_ctx *ctx, uint64_t x, uint64_t *out); /* 0 if no x87 */
uint64_t orc_pack_response(const orc_ctx *ctx, const uint64_t *ct, uint8_t *out);
uint64_t orc_response_bytes(const orc_ctx *ctx);
int orc_make_query_server(const orc_ctx *ctx, const uint64_t *db_aligned,
                          const uint64_t *galois_keys, const uint64_t *gsw_key_ntt,
                          const uint64_t *query, uint64_t *resp, uint8_t *packed,
                          double *stage_ms);

#ifdef __cplusplus
}
#endif
#endif
