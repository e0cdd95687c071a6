/*
 * onionpir_client.h -- C ABI of the CPU PirClient (libopir_client.so).
 *
 * The client side of the protocol (src/includes/client.h:4-53): secret key,
 * Galois keys, RGSW(sk), packed queries, response unpacking, decryption at
 * small_q with the noise budget, entry extraction.  No GPU is involved; the
 * library links against nothing but the C++ runtime.  Arrays use the layouts
 * of onionpir_gpu.h, so a client's outputs are the server's inputs:
 *   Galois keys  [h][2][2][N]     NTT form (h = expansion height)
 *   RGSW(sk)     [2 l_key][2][N]  coefficient form mod q
 *   query        [2][N]           coefficient form mod q
 *   response     [2][N]           mod small_q (or the packed bytes)
 *
 * Randomised calls take `const uint64_t *seed`: NULL draws from ChaCha20
 * keyed by the operating system's entropy; a seed gives a reproducible,
 * NOT secure SplitMix64 stream (tests and benchmarks).
 *
 * Every call returns OPIR_OK (0) or a negative status (onionpir_gpu.h's
 * codes: OPIR_ERR_ARG for bad arguments); opir_client_last_error() gives the
 * message of the calling thread's last failure.
 */
#ifndef ONIONPIR_CLIENT_H
#define ONIONPIR_CLIENT_H

#include <stddef.h>
#include <stdint.h>

#include "onionpir_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct opir_client opir_client;

/* PirClient::PirClient (client.cpp:11-16).  `secret_seed` NULL: a fresh key
 * from OS entropy. */
int opir_client_create(const opir_params *params, const opir_db_shape *shape, uint64_t client_id,
                       const uint64_t *secret_seed, opir_client **out);
void opir_client_destroy(opir_client *c);
const char *opir_client_last_error(void);

uint64_t opir_client_id(const opir_client *c);                  /* get_client_id */
uint32_t opir_client_expansion_height(const opir_client *c);    /* Galois key levels */
uint64_t opir_client_response_bytes(const opir_client *c);      /* packed response size */
int opir_client_secret_key(const opir_client *c, int8_t *out);  /* N values in {-1,0,1} */

/* create_galois_keys (client.cpp:227-241): h * 4 * N words */
int opir_client_galois_keys(const opir_client *c, const uint64_t *seed, uint64_t *out);
/* generate_gsw_from_key (client.cpp:17-31): 2 l_key * 2 * N words */
int opir_client_gsw_key(const opir_client *c, const uint64_t *seed, uint64_t *out);
/* fast_generate_query + add_gsw_to_query (client.cpp:130-209): 2 * N words */
int opir_client_query(const opir_client *c, uint64_t entry_index, const uint64_t *seed,
                      uint64_t *out);
/* get_query_indices (client.cpp:38-53): ndim indices */
int opir_client_query_indices(const opir_client *c, uint64_t plaintext_index, uint64_t *out,
                              uint32_t *ndim);

/* load_resp_from_stream (client.cpp:364-412): `nbytes` must be at least
 * opir_client_response_bytes */
int opir_client_unpack_response(const opir_client *c, const uint8_t *bytes, uint64_t nbytes,
                                uint64_t *ct);
/* decrypt_mod_q (client.cpp:415-479); decrypt_ct at q when at_q != 0 */
int opir_client_decrypt(const opir_client *c, const uint64_t *ct, int at_q, uint64_t *plain,
                        int *noise_budget);
/* get_entry_from_plaintext (client.cpp:255-287): entry_size bytes */
int opir_client_entry_from_plaintext(const opir_client *c, uint64_t entry_index,
                                     const uint64_t *plain, uint8_t *entry);
/* unpack + decrypt_mod_q + get_entry_from_plaintext in one call */
int opir_client_decode_response(const opir_client *c, uint64_t entry_index, const uint8_t *bytes,
                                uint64_t nbytes, uint8_t *entry, int *noise_budget);

/* ChaCha20 block function (RFC 8439 section 2.3), for known-answer tests */
void opir_chacha20_block(const uint32_t key[8], uint32_t counter, const uint32_t nonce[3],
                         uint32_t out[16]);

#ifdef __cplusplus
}
#endif
#endif
