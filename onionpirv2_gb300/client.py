"""PirClient: the client side of the protocol on the CPU (src/client.cpp,
src/includes/client.h:4-53), over the C ABI of ``include/onionpir_client.h``
(``_build/libopir_client.so``, no GPU needed).

Outputs are in the layouts the server takes, so

    client = PirClient(params, client_id=7)
    server.set_client_galois_key(7, client.create_galois_keys())
    server.set_client_gsw_key(7, client.generate_gsw_from_key())
    resp = server.make_query(7, client.fast_generate_query(i))
    entry, budget = client.decode_response(i, resp.packed)

Randomised methods take ``seed=None`` (ChaCha20 keyed from OS entropy) or an
integer seed (a reproducible SplitMix64 stream: tests and benchmarks only,
not secure).  Calls release the GIL, so threads generate keys in parallel.
"""
from __future__ import annotations

import ctypes
import io
import os
from typing import Optional, Tuple

import numpy as np

from ._capi import OpirDbShape, OpirError, OpirParams
from .build import CLIENT_LIB
from .params import POLY_DEGREE, PirParams

N = POLY_DEGREE
_u64p = ctypes.POINTER(ctypes.c_uint64)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_vp = ctypes.c_void_p

# every symbol include/onionpir_client.h declares
CLIENT_EXPORTS = (
    "opir_client_create", "opir_client_destroy", "opir_client_last_error", "opir_client_id",
    "opir_client_expansion_height", "opir_client_response_bytes", "opir_client_secret_key",
    "opir_client_galois_keys", "opir_client_gsw_key", "opir_client_query",
    "opir_client_query_indices", "opir_client_unpack_response", "opir_client_decrypt",
    "opir_client_entry_from_plaintext", "opir_client_decode_response", "opir_chacha20_block",
)

_lib = None


def load(path: str = CLIENT_LIB):
    """Load the client library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} not found: build it first "
                          "(python -c 'from onionpirv2_gb300 import build; build.build_client()')")
    L = ctypes.CDLL(path)
    sp = ctypes.POINTER(ctypes.c_uint64)
    L.opir_client_create.argtypes = [ctypes.POINTER(OpirParams), ctypes.POINTER(OpirDbShape),
                                     ctypes.c_uint64, sp, ctypes.POINTER(_vp)]
    L.opir_client_destroy.argtypes = [_vp]
    L.opir_client_destroy.restype = None
    L.opir_client_last_error.argtypes = []
    L.opir_client_last_error.restype = ctypes.c_char_p
    L.opir_client_id.argtypes = [_vp]
    L.opir_client_id.restype = ctypes.c_uint64
    L.opir_client_expansion_height.argtypes = [_vp]
    L.opir_client_expansion_height.restype = ctypes.c_uint32
    L.opir_client_response_bytes.argtypes = [_vp]
    L.opir_client_response_bytes.restype = ctypes.c_uint64
    L.opir_client_secret_key.argtypes = [_vp, ctypes.POINTER(ctypes.c_int8)]
    L.opir_client_galois_keys.argtypes = [_vp, sp, _u64p]
    L.opir_client_gsw_key.argtypes = [_vp, sp, _u64p]
    L.opir_client_query.argtypes = [_vp, ctypes.c_uint64, sp, _u64p]
    L.opir_client_query_indices.argtypes = [_vp, ctypes.c_uint64, _u64p,
                                            ctypes.POINTER(ctypes.c_uint32)]
    L.opir_client_unpack_response.argtypes = [_vp, _u8p, ctypes.c_uint64, _u64p]
    L.opir_client_decrypt.argtypes = [_vp, _u64p, ctypes.c_int, _u64p, ctypes.POINTER(ctypes.c_int)]
    L.opir_client_entry_from_plaintext.argtypes = [_vp, ctypes.c_uint64, _u64p, _u8p]
    L.opir_client_decode_response.argtypes = [_vp, ctypes.c_uint64, _u8p, ctypes.c_uint64, _u8p,
                                              ctypes.POINTER(ctypes.c_int)]
    L.opir_chacha20_block.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint32,
                                      ctypes.POINTER(ctypes.c_uint32),
                                      ctypes.POINTER(ctypes.c_uint32)]
    L.opir_chacha20_block.restype = None
    _lib = L
    return L


def _check(rc: int):
    if rc != 0:
        msg = load().opir_client_last_error().decode()
        if rc == -1:
            raise ValueError(msg)
        raise OpirError(rc, msg)


def _seed(seed: Optional[int]):
    return ctypes.byref(ctypes.c_uint64(seed)) if seed is not None else None


def _u64(a: np.ndarray):
    return a.ctypes.data_as(_u64p)


def chacha20_block(key: bytes, counter: int, nonce: bytes) -> bytes:
    """The ChaCha20 block function (RFC 8439 section 2.3) of the client's
    random stream: 32-byte key, 12-byte nonce, 64 serialised bytes."""
    k = np.frombuffer(key, "<u4").astype(np.uint32)
    n = np.frombuffer(nonce, "<u4").astype(np.uint32)
    out = np.zeros(16, np.uint32)
    p32 = ctypes.POINTER(ctypes.c_uint32)
    load().opir_chacha20_block(k.ctypes.data_as(p32), counter, n.ctypes.data_as(p32),
                               out.ctypes.data_as(p32))
    return out.astype("<u4").tobytes()


class PirClient:
    """PirClient (client.cpp:11-16): a ternary secret key and the calls that
    use it.  ``secret_seed=None`` draws the key from OS entropy."""

    def __init__(self, pir_params: PirParams, client_id: int = 0,
                 secret_seed: Optional[int] = None):
        self.pir_params = P = pir_params
        self._L = load()
        prm = OpirParams(
            poly_degree=P.poly_degree, coeff_modulus=P.coeff_modulus[0],
            special_modulus=P.coeff_modulus[-1], plain_modulus=P.plain_mod,
            small_modulus=P.small_q, gsw_l=P.gsw_l, gsw_base_log2=P.base_log2,
            gsw_l_key=P.gsw_l_key, gsw_base_log2_key=P.base_log2_key)
        shape = OpirDbShape(
            fst_dim_sz=P.get_fst_dim_sz(), other_dim_sz=P.get_other_dim_sz(),
            entry_size=P.get_entry_size(), entries_per_pt=P.get_num_entries_per_plaintext(),
            bits_per_coeff=P.get_num_bits_per_coeff())
        h = _vp()
        _check(self._L.opir_client_create(ctypes.byref(prm), ctypes.byref(shape), client_id,
                                          _seed(secret_seed), ctypes.byref(h)))
        self._h = h
        self.height = int(self._L.opir_client_expansion_height(h))
        self.resp_bytes = int(self._L.opir_client_response_bytes(h))

    def close(self):
        if getattr(self, "_h", None):
            self._L.opir_client_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_client_id(self) -> int:
        return int(self._L.opir_client_id(self._h))

    def secret_key(self) -> np.ndarray:
        sk = np.zeros(N, np.int8)
        _check(self._L.opir_client_secret_key(self._h, sk.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))))
        return sk

    def get_query_indices(self, plaintext_index: int):
        out = np.zeros(64, np.uint64)
        nd = ctypes.c_uint32()
        _check(self._L.opir_client_query_indices(self._h, plaintext_index, _u64(out),
                                                 ctypes.byref(nd)))
        return [int(x) for x in out[: nd.value]]

    def create_galois_keys(self, seed: Optional[int] = None) -> np.ndarray:
        """[h][2][2][N] NTT form (client.cpp:227-241)."""
        out = np.zeros((self.height, 2, 2, N), np.uint64)
        _check(self._L.opir_client_galois_keys(self._h, _seed(seed), _u64(out)))
        return out

    def generate_gsw_from_key(self, seed: Optional[int] = None) -> np.ndarray:
        """[2 l_key][2][N] coefficient form (client.cpp:17-31)."""
        out = np.zeros((2 * self.pir_params.get_l_key(), 2, N), np.uint64)
        _check(self._L.opir_client_gsw_key(self._h, _seed(seed), _u64(out)))
        return out

    def fast_generate_query(self, entry_index: int, seed: Optional[int] = None) -> np.ndarray:
        """[2][N] packed query for one entry (client.cpp:130-209)."""
        out = np.zeros((2, N), np.uint64)
        _check(self._L.opir_client_query(self._h, entry_index, _seed(seed), _u64(out)))
        return out

    def load_resp_from_stream(self, stream) -> np.ndarray:
        """Unpack a 27-bit packed response (client.cpp:364-412)."""
        data = stream.read(self.resp_bytes) if isinstance(stream, io.IOBase) else bytes(stream)
        buf = np.frombuffer(data, np.uint8)
        out = np.zeros((2, N), np.uint64)
        _check(self._L.opir_client_unpack_response(self._h, buf.ctypes.data_as(_u8p), buf.size,
                                                   _u64(out)))
        return out

    def decrypt_mod_q(self, ct) -> Tuple[np.ndarray, int]:
        """(plaintext mod t, noise budget) of a response mod small_q
        (client.cpp:415-479)."""
        return self._decrypt(ct, 0)

    def decrypt_ct(self, ct) -> Tuple[np.ndarray, int]:
        """The same at the ciphertext modulus q."""
        return self._decrypt(ct, 1)

    def _decrypt(self, ct, at_q: int):
        c = np.ascontiguousarray(ct, np.uint64).reshape(-1)
        if c.size != 2 * N:
            raise ValueError("ciphertext must be [2][N]")
        plain = np.zeros(N, np.uint64)
        budget = ctypes.c_int()
        _check(self._L.opir_client_decrypt(self._h, _u64(c), at_q, _u64(plain), ctypes.byref(budget)))
        return plain, budget.value

    def get_entry_from_plaintext(self, entry_index: int, plain) -> np.ndarray:
        p = np.ascontiguousarray(plain, np.uint64)
        out = np.zeros(self.pir_params.get_entry_size(), np.uint8)
        _check(self._L.opir_client_entry_from_plaintext(self._h, entry_index, _u64(p),
                                                        out.ctypes.data_as(_u8p)))
        return out

    def decode_response(self, entry_index: int, packed) -> Tuple[np.ndarray, int]:
        """Packed response bytes -> (entry bytes, noise budget)."""
        buf = np.frombuffer(bytes(packed), np.uint8)
        out = np.zeros(self.pir_params.get_entry_size(), np.uint8)
        budget = ctypes.c_int()
        _check(self._L.opir_client_decode_response(self._h, entry_index, buf.ctypes.data_as(_u8p),
                                                   buf.size, out.ctypes.data_as(_u8p),
                                                   ctypes.byref(budget)))
        return out, budget.value
