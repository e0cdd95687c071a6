// client.cpp -- the C ABI of include/onionpir_client.h over the header-only
// onionpir::PirClient (include/onionpir_client.hpp).  CPU only: built by g++
// into libopir_client.so, which needs no CUDA runtime.
#include <cstring>
#include <exception>
#include <new>
#include <stdexcept>
#include <string>

#include "onionpir_client.h"
#include "onionpir_client.hpp"

struct opir_client {
  onionpir::PirClient impl;
};

namespace {

thread_local std::string g_error;

int fail(int code, const char *msg) {
  g_error = msg;
  return code;
}

// runs `f`, turning exceptions into status codes
template <class F>
int guard(F &&f) {
  try {
    f();
    return OPIR_OK;
  } catch (const std::invalid_argument &e) {
    return fail(OPIR_ERR_ARG, e.what());
  } catch (const std::bad_alloc &) {
    return fail(OPIR_ERR_OOM, "host allocation failed");
  } catch (const std::exception &e) {
    return fail(OPIR_ERR_STATE, e.what());
  }
}

template <class V>
void copy_out(const V &v, typename V::value_type *out) {
  std::memcpy(out, v.data(), v.size() * sizeof(typename V::value_type));
}

}  // namespace

extern "C" {

int opir_client_create(const opir_params *params, const opir_db_shape *shape, uint64_t client_id,
                       const uint64_t *secret_seed, opir_client **out) {
  if (!params || !shape || !out) return fail(OPIR_ERR_ARG, "null argument");
  *out = nullptr;
  return guard([&] {
    onionpir::PirParams P;
    P.poly_degree = params->poly_degree;
    P.q = params->coeff_modulus;
    P.p = params->special_modulus;
    P.t = params->plain_modulus;
    P.small_q = params->small_modulus;
    P.l = params->gsw_l;
    P.base_log2 = params->gsw_base_log2;
    P.l_key = params->gsw_l_key;
    P.base_log2_key = params->gsw_base_log2_key;
    P.fst_dim_sz = shape->fst_dim_sz;
    P.other_dim_sz = shape->other_dim_sz;
    P.entry_size = shape->entry_size;
    P.entries_per_pt = shape->entries_per_pt;
    P.bits_per_coeff = shape->bits_per_coeff;
    if (!P.l || !P.l_key || !P.entries_per_pt || !P.entry_size || !P.bits_per_coeff ||
        (P.other_dim_sz & (P.other_dim_sz - 1)))
      throw std::invalid_argument("bad parameter set");
    *out = secret_seed ? new opir_client{onionpir::PirClient(P, client_id, *secret_seed)}
                       : new opir_client{onionpir::PirClient(P, client_id)};
  });
}

void opir_client_destroy(opir_client *c) { delete c; }
const char *opir_client_last_error(void) { return g_error.c_str(); }

uint64_t opir_client_id(const opir_client *c) { return c ? c->impl.get_client_id() : 0; }
uint32_t opir_client_expansion_height(const opir_client *c) {
  return c ? c->impl.params().expan_height() : 0;
}
uint64_t opir_client_response_bytes(const opir_client *c) {
  return c ? c->impl.response_bytes() : 0;
}
int opir_client_secret_key(const opir_client *c, int8_t *out) {
  if (!c || !out) return fail(OPIR_ERR_ARG, "null argument");
  copy_out(c->impl.secret_key(), out);
  return OPIR_OK;
}

int opir_client_galois_keys(const opir_client *c, const uint64_t *seed, uint64_t *out) {
  if (!c || !out) return fail(OPIR_ERR_ARG, "null argument");
  return guard([&] {
    copy_out(seed ? c->impl.create_galois_keys(*seed) : c->impl.create_galois_keys(), out);
  });
}

int opir_client_gsw_key(const opir_client *c, const uint64_t *seed, uint64_t *out) {
  if (!c || !out) return fail(OPIR_ERR_ARG, "null argument");
  return guard([&] {
    copy_out(seed ? c->impl.generate_gsw_from_key(*seed) : c->impl.generate_gsw_from_key(), out);
  });
}

int opir_client_query(const opir_client *c, uint64_t entry_index, const uint64_t *seed,
                      uint64_t *out) {
  if (!c || !out) return fail(OPIR_ERR_ARG, "null argument");
  return guard([&] {
    copy_out(seed ? c->impl.fast_generate_query(entry_index, *seed)
                  : c->impl.fast_generate_query(entry_index),
             out);
  });
}

int opir_client_query_indices(const opir_client *c, uint64_t plaintext_index, uint64_t *out,
                              uint32_t *ndim) {
  if (!c || !out || !ndim) return fail(OPIR_ERR_ARG, "null argument");
  if (plaintext_index >= c->impl.params().num_pt())
    return fail(OPIR_ERR_ARG, "plaintext index out of range");
  const auto idx = c->impl.get_query_indices(plaintext_index);
  for (size_t i = 0; i < idx.size(); i++) out[i] = idx[i];
  *ndim = (uint32_t)idx.size();
  return OPIR_OK;
}

int opir_client_unpack_response(const opir_client *c, const uint8_t *bytes, uint64_t nbytes,
                                uint64_t *ct) {
  if (!c || !bytes || !ct) return fail(OPIR_ERR_ARG, "null argument");
  if (nbytes < c->impl.response_bytes())
    return fail(OPIR_ERR_ARG, "unexpected end of response stream");
  copy_out(c->impl.unpack_response(bytes), ct);
  return OPIR_OK;
}

int opir_client_decrypt(const opir_client *c, const uint64_t *ct, int at_q, uint64_t *plain,
                        int *noise_budget) {
  if (!c || !ct || !plain) return fail(OPIR_ERR_ARG, "null argument");
  return guard([&] {
    const onionpir::Ciphertext v(ct, ct + 2 * onionpir::PirClient::N);
    copy_out(at_q ? c->impl.decrypt_ct(v, noise_budget) : c->impl.decrypt_mod_q(v, noise_budget),
             plain);
  });
}

int opir_client_entry_from_plaintext(const opir_client *c, uint64_t entry_index,
                                     const uint64_t *plain, uint8_t *entry) {
  if (!c || !plain || !entry) return fail(OPIR_ERR_ARG, "null argument");
  return guard([&] {
    const onionpir::Plaintext v(plain, plain + onionpir::PirClient::N);
    copy_out(c->impl.get_entry_from_plaintext(entry_index, v), entry);
  });
}

int opir_client_decode_response(const opir_client *c, uint64_t entry_index, const uint8_t *bytes,
                                uint64_t nbytes, uint8_t *entry, int *noise_budget) {
  if (!c || !bytes || !entry) return fail(OPIR_ERR_ARG, "null argument");
  if (nbytes < c->impl.response_bytes())
    return fail(OPIR_ERR_ARG, "unexpected end of response stream");
  return guard([&] {
    const auto plain = c->impl.decrypt_mod_q(c->impl.unpack_response(bytes), noise_budget);
    copy_out(c->impl.get_entry_from_plaintext(entry_index, plain), entry);
  });
}

void opir_chacha20_block(const uint32_t key[8], uint32_t counter, const uint32_t nonce[3],
                         uint32_t out[16]) {
  onionpir::ChaChaStream::block(key, counter, nonce, out);
}

}  // extern "C"
