"""ctypes wrapper around the C oracle (``oracle/opir_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, by the smoke check and by
the CPU-baseline leg of ``bench.py`` -- never by the product package.  The
oracle restates the reference server path (src/server.cpp, src/gsw_eval.cpp,
src/matrix.cpp, src/pir.cpp, src/client.cpp); see ``opir_oracle.h`` for its
parity status (partially pinned).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libopir_oracle.so")
N = 2048

_u64p = ctypes.POINTER(ctypes.c_uint64)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_i8p = ctypes.POINTER(ctypes.c_int8)


SOURCES = ("opir_oracle.c", "opir_oracle_rns.c")


def build(force: bool = False) -> str:
    """Compile the oracle (single- and multi-modulus restatements) into
    ``oracle/_build`` (gcc, -O3, OpenMP)."""
    srcs = [os.path.join(HERE, f) for f in SOURCES]
    deps = srcs + [s[:-2] + ".h" for s in srcs]
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(d) for d in deps)):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-Wall", "-o", tmp] + srcs + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class OrcParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "poly_degree", "q", "p", "t", "small_q", "small_q_width", "l", "base_log2",
        "l_key", "base_log2_key", "num_entries", "num_pt", "entry_size",
        "entries_per_pt", "bits_per_coeff", "n1", "n_rest", "ndim", "u", "h",
        "ms_mant")] + [("ms_exp", ctypes.c_int64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        L.orc_create.restype = vp
        L.orc_create.argtypes = [ctypes.c_uint64] * 9
        L.orc_destroy.argtypes = [vp]
        L.orc_get_params.argtypes = [vp, ctypes.POINTER(OrcParams)]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_set_threads.restype = ctypes.c_int
        L.orc_is_prime.argtypes = [ctypes.c_uint64]
        L.orc_generate_prime.argtypes = [ctypes.c_uint64]
        L.orc_generate_prime.restype = ctypes.c_uint64
        L.orc_coeff_modulus_create.argtypes = [ctypes.c_uint64, _u64p, ctypes.c_size_t, _u64p]
        L.orc_minimal_root.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.orc_minimal_root.restype = ctypes.c_uint64
        L.orc_barrett_reduce_128.argtypes = [ctypes.c_uint64] * 3
        L.orc_barrett_reduce_128.restype = ctypes.c_uint64
        for f in ("orc_ntt_fwd", "orc_ntt_inv"):
            getattr(L, f).argtypes = [vp, ctypes.c_int, _u64p, ctypes.c_size_t]
        L.orc_ntt_tables.argtypes = [vp, ctypes.c_int, _u64p, _u64p, _u64p, _u64p]
        L.orc_gen_entries.argtypes = [vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, _u8p]
        L.orc_pack_plaintexts.argtypes = [vp, _u8p, ctypes.c_uint64, _u64p]
        L.orc_plain_to_ntt.argtypes = [vp, _u64p, ctypes.c_uint64]
        L.orc_realign.argtypes = [vp, _u64p, _u64p]
        L.orc_build_db.argtypes = [vp, ctypes.c_uint64, _u64p]
        L.orc_keygen.argtypes = [vp, ctypes.c_uint64, _i8p]
        L.orc_make_galois_keys.argtypes = [vp, _i8p, ctypes.c_uint64, _u64p]
        L.orc_make_gsw_key.argtypes = [vp, _i8p, ctypes.c_uint64, _u64p]
        L.orc_query_indices.argtypes = [vp, ctypes.c_uint64, _u64p]
        L.orc_make_query.argtypes = [vp, _i8p, ctypes.c_uint64, ctypes.c_uint64, _u64p]
        L.orc_decrypt.argtypes = [vp, _i8p, _u64p, ctypes.c_int, _u64p,
                                  ctypes.POINTER(ctypes.c_int)]
        L.orc_entry_from_plain.argtypes = [vp, ctypes.c_uint64, _u64p, _u8p]
        L.orc_unpack_response.argtypes = [vp, _u8p, _u64p]
        L.orc_negacyclic_shift.argtypes = [vp, _u64p, ctypes.c_int64, _u64p]
        L.orc_apply_galois.argtypes = [vp, _u64p, ctypes.c_uint64, _u64p, _u64p]
        L.orc_expand.argtypes = [vp, _u64p, _u64p, _u64p]
        L.orc_gsw_key_to_ntt.argtypes = [vp, _u64p, ctypes.c_uint64, _u64p]
        L.orc_ext_product.argtypes = [vp, _u64p, ctypes.c_uint64, ctypes.c_uint64, _u64p, _u64p]
        L.orc_query_to_gsw.argtypes = [vp, _u64p, _u64p, _u64p]
        L.orc_first_dim.argtypes = [vp, _u64p, _u64p, _u64p]
        L.orc_first_dim.restype = ctypes.c_int
        L.orc_first_dim_wrapping.argtypes = [vp, _u64p, _u64p, _u64p]
        L.orc_other_dim_mux.argtypes = [vp, _u64p, ctypes.c_uint64, _u64p]
        L.orc_mod_switch.argtypes = [vp, _u64p]
        L.orc_mod_switch_coeff.argtypes = [vp, ctypes.c_uint64]
        L.orc_mod_switch_coeff.restype = ctypes.c_uint64
        L.orc_x87_mod_switch.argtypes = [vp, ctypes.c_uint64, _u64p]
        L.orc_x87_mod_switch.restype = ctypes.c_int
        L.orc_pack_response.argtypes = [vp, _u64p, _u8p]
        L.orc_pack_response.restype = ctypes.c_uint64
        L.orc_response_bytes.argtypes = [vp]
        L.orc_response_bytes.restype = ctypes.c_uint64
        L.orc_make_query_server.argtypes = [vp, _u64p, _u64p, _u64p, _u64p, _u64p, _u8p,
                                            ctypes.POINTER(ctypes.c_double)]
        L.orc_make_query_server.restype = ctypes.c_int
        _bind_rns(L)
        _lib = L
    return _lib


def _p64(a: np.ndarray):
    assert a.dtype == np.uint64 and a.flags.c_contiguous
    return a.ctypes.data_as(_u64p)


def _p8(a: np.ndarray):
    assert a.dtype == np.uint8 and a.flags.c_contiguous
    return a.ctypes.data_as(_u8p)


def _pi8(a: np.ndarray):
    assert a.dtype == np.int8 and a.flags.c_contiguous
    return a.ctypes.data_as(_i8p)


@dataclass
class Params:
    poly_degree: int
    q: int
    p: int
    t: int
    small_q: int
    small_q_width: int
    l: int
    base_log2: int
    l_key: int
    base_log2_key: int
    num_entries: int
    num_pt: int
    entry_size: int
    entries_per_pt: int
    bits_per_coeff: int
    n1: int
    n_rest: int
    ndim: int
    u: int
    h: int
    ms_mant: int
    ms_exp: int


class Oracle:
    """One oracle context: parameters derived as in pir.cpp:29-95."""

    def __init__(self, num_entries: int, max_fst_dim: int, entry_size: int = 0, l: int = 5,
                 l_key: int = 10, plain_bits: int = 16, small_q_width: int = 27,
                 coeff_bits=(60, 60)):
        self.L = lib()
        self.h_ctx = self.L.orc_create(num_entries, max_fst_dim, entry_size, l, l_key,
                                       plain_bits, small_q_width, coeff_bits[0], coeff_bits[1])
        if not self.h_ctx:
            raise ValueError("invalid PIR parameters")
        op = OrcParams()
        self.L.orc_get_params(self.h_ctx, ctypes.byref(op))
        self.P = Params(**{f: int(getattr(op, f)) for f, _ in OrcParams._fields_})

    def __del__(self):
        if getattr(self, "h_ctx", None):
            self.L.orc_destroy(self.h_ctx)
            self.h_ctx = None

    # ---- primitives
    def ntt_fwd(self, a: np.ndarray, mod: int = 0) -> np.ndarray:
        a = np.ascontiguousarray(a, dtype=np.uint64).copy()
        self.L.orc_ntt_fwd(self.h_ctx, mod, _p64(a), a.size // N)
        return a

    def ntt_inv(self, a: np.ndarray, mod: int = 0) -> np.ndarray:
        a = np.ascontiguousarray(a, dtype=np.uint64).copy()
        self.L.orc_ntt_inv(self.h_ctx, mod, _p64(a), a.size // N)
        return a

    def ntt_tables(self, mod: int = 0):
        fwd = np.zeros(N, np.uint64)
        inv = np.zeros(N, np.uint64)
        psi = ctypes.c_uint64()
        ninv = ctypes.c_uint64()
        self.L.orc_ntt_tables(self.h_ctx, mod, _p64(fwd), _p64(inv), ctypes.byref(psi),
                              ctypes.byref(ninv))
        return fwd, inv, int(psi.value), int(ninv.value)

    # ---- database
    def gen_entries(self, seed: int, first: int, count: int) -> np.ndarray:
        out = np.zeros(count * self.P.entry_size, np.uint8)
        self.L.orc_gen_entries(self.h_ctx, seed, first, count, _p8(out))
        return out.reshape(count, self.P.entry_size)

    def pack_plaintexts(self, entries: np.ndarray, num_pt: int) -> np.ndarray:
        e = np.ascontiguousarray(entries, dtype=np.uint8)
        out = np.zeros(num_pt * N, np.uint64)
        self.L.orc_pack_plaintexts(self.h_ctx, _p8(e.reshape(-1)), num_pt, _p64(out))
        return out.reshape(num_pt, N)

    def plain_to_ntt(self, coeffs: np.ndarray) -> np.ndarray:
        c = np.ascontiguousarray(coeffs, dtype=np.uint64).copy()
        self.L.orc_plain_to_ntt(self.h_ctx, _p64(c.reshape(-1)), c.size // N)
        return c

    def build_db(self, seed: int) -> np.ndarray:
        out = np.empty(self.P.num_pt * N, np.uint64)
        self.L.orc_build_db(self.h_ctx, seed, _p64(out))
        return out.reshape(N, self.P.num_pt)

    # ---- client
    def keygen(self, seed: int) -> np.ndarray:
        sk = np.zeros(N, np.int8)
        self.L.orc_keygen(self.h_ctx, seed, _pi8(sk))
        return sk

    def galois_keys(self, sk: np.ndarray, seed: int) -> np.ndarray:
        out = np.zeros(self.P.h * 4 * N, np.uint64)
        self.L.orc_make_galois_keys(self.h_ctx, _pi8(sk), seed, _p64(out))
        return out.reshape(self.P.h, 2, 2, N)

    def gsw_key(self, sk: np.ndarray, seed: int) -> np.ndarray:
        out = np.zeros(2 * self.P.l_key * 2 * N, np.uint64)
        self.L.orc_make_gsw_key(self.h_ctx, _pi8(sk), seed, _p64(out))
        return out.reshape(2 * self.P.l_key, 2, N)

    def query_indices(self, pt_index: int):
        out = np.zeros(64, np.uint64)
        self.L.orc_query_indices(self.h_ctx, pt_index, _p64(out))
        return [int(x) for x in out[: self.P.ndim]]

    def make_query(self, sk: np.ndarray, seed: int, entry_index: int) -> np.ndarray:
        out = np.zeros(2 * N, np.uint64)
        self.L.orc_make_query(self.h_ctx, _pi8(sk), seed, entry_index, _p64(out))
        return out.reshape(2, N)

    def decrypt(self, sk: np.ndarray, ct: np.ndarray, mod: int = 2):
        c = np.ascontiguousarray(ct, dtype=np.uint64).reshape(-1)
        plain = np.zeros(N, np.uint64)
        nb = ctypes.c_int()
        self.L.orc_decrypt(self.h_ctx, _pi8(sk), _p64(c), mod, _p64(plain), ctypes.byref(nb))
        return plain, int(nb.value)

    def entry_from_plain(self, entry_index: int, plain: np.ndarray) -> np.ndarray:
        out = np.zeros(self.P.entry_size, np.uint8)
        self.L.orc_entry_from_plain(self.h_ctx, entry_index,
                                    _p64(np.ascontiguousarray(plain, dtype=np.uint64)), _p8(out))
        return out

    def unpack_response(self, data: np.ndarray) -> np.ndarray:
        out = np.zeros(2 * N, np.uint64)
        self.L.orc_unpack_response(self.h_ctx, _p8(np.ascontiguousarray(data, np.uint8)),
                                   _p64(out))
        return out.reshape(2, N)

    # ---- server path
    def negacyclic_shift(self, ct: np.ndarray, k: int) -> np.ndarray:
        out = np.zeros(2 * N, np.uint64)
        self.L.orc_negacyclic_shift(self.h_ctx, _p64(np.ascontiguousarray(ct, np.uint64).reshape(-1)),
                                    k, _p64(out))
        return out.reshape(2, N)

    def apply_galois(self, ct: np.ndarray, g: int, key: np.ndarray) -> np.ndarray:
        out = np.zeros(2 * N, np.uint64)
        self.L.orc_apply_galois(self.h_ctx, _p64(np.ascontiguousarray(ct, np.uint64).reshape(-1)),
                                g, _p64(np.ascontiguousarray(key, np.uint64).reshape(-1)),
                                _p64(out))
        return out.reshape(2, N)

    def expand(self, query: np.ndarray, gk: np.ndarray) -> np.ndarray:
        out = np.zeros(self.P.u * 2 * N, np.uint64)
        self.L.orc_expand(self.h_ctx, _p64(np.ascontiguousarray(query, np.uint64).reshape(-1)),
                          _p64(np.ascontiguousarray(gk, np.uint64).reshape(-1)), _p64(out))
        return out.reshape(self.P.u, 2, N)

    def gsw_key_to_ntt(self, rows: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(rows, np.uint64)
        out = np.zeros_like(r)
        self.L.orc_gsw_key_to_ntt(self.h_ctx, _p64(r.reshape(-1)), r.shape[0],
                                  _p64(out.reshape(-1)))
        return out

    def ext_product(self, gsw_ntt: np.ndarray, l: int, base_log2: int,
                    ct: np.ndarray) -> np.ndarray:
        out = np.zeros(2 * N, np.uint64)
        self.L.orc_ext_product(self.h_ctx, _p64(np.ascontiguousarray(gsw_ntt, np.uint64).reshape(-1)),
                               l, base_log2,
                               _p64(np.ascontiguousarray(ct, np.uint64).reshape(-1)), _p64(out))
        return out.reshape(2, N)

    def query_to_gsw(self, cts: np.ndarray, key_ntt: np.ndarray) -> np.ndarray:
        out = np.zeros(2 * self.P.l * 2 * N, np.uint64)
        self.L.orc_query_to_gsw(self.h_ctx, _p64(np.ascontiguousarray(cts, np.uint64).reshape(-1)),
                                _p64(np.ascontiguousarray(key_ntt, np.uint64).reshape(-1)),
                                _p64(out))
        return out.reshape(2 * self.P.l, 2, N)

    def first_dim(self, db_aligned: np.ndarray, fst: np.ndarray, wrapping: bool = False):
        out = np.zeros(self.P.n_rest * 2 * N, np.uint64)
        dbp = _p64(np.ascontiguousarray(db_aligned, np.uint64).reshape(-1))
        fp = _p64(np.ascontiguousarray(fst, np.uint64).reshape(-1))
        if wrapping:
            self.L.orc_first_dim_wrapping(self.h_ctx, dbp, fp, _p64(out))
            return out.reshape(self.P.n_rest, 2, N)
        wraps = self.L.orc_first_dim(self.h_ctx, dbp, fp, _p64(out))
        return out.reshape(self.P.n_rest, 2, N), wraps

    def other_dim_mux(self, result: np.ndarray, gsw_ntt: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(result, np.uint64).copy()
        self.L.orc_other_dim_mux(self.h_ctx, _p64(r.reshape(-1)), r.shape[0],
                                 _p64(np.ascontiguousarray(gsw_ntt, np.uint64).reshape(-1)))
        return r[: r.shape[0] // 2]

    def mod_switch(self, ct: np.ndarray) -> np.ndarray:
        c = np.ascontiguousarray(ct, np.uint64).copy()
        self.L.orc_mod_switch(self.h_ctx, _p64(c.reshape(-1)))
        return c

    def mod_switch_coeff(self, x: int) -> int:
        return int(self.L.orc_mod_switch_coeff(self.h_ctx, x))

    def x87_mod_switch(self, x: int):
        out = ctypes.c_uint64()
        ok = self.L.orc_x87_mod_switch(self.h_ctx, x, ctypes.byref(out))
        return int(out.value) if ok else None

    def response_bytes(self) -> int:
        return int(self.L.orc_response_bytes(self.h_ctx))

    def pack_response(self, ct: np.ndarray) -> np.ndarray:
        out = np.zeros(self.response_bytes(), np.uint8)
        self.L.orc_pack_response(self.h_ctx, _p64(np.ascontiguousarray(ct, np.uint64).reshape(-1)),
                                 _p8(out))
        return out

    def make_query_server(self, db_aligned, galois_keys, gsw_key_ntt, query):
        resp = np.zeros(2 * N, np.uint64)
        packed = np.zeros(self.response_bytes(), np.uint8)
        ms = (ctypes.c_double * 5)()
        wraps = self.L.orc_make_query_server(
            self.h_ctx, _p64(np.ascontiguousarray(db_aligned, np.uint64).reshape(-1)),
            _p64(np.ascontiguousarray(galois_keys, np.uint64).reshape(-1)),
            _p64(np.ascontiguousarray(gsw_key_ntt, np.uint64).reshape(-1)),
            _p64(np.ascontiguousarray(query, np.uint64).reshape(-1)),
            _p64(resp), _p8(packed), ms)
        return resp.reshape(2, N), packed, list(ms), wraps


def set_threads(n: int) -> int:
    return int(lib().orc_set_threads(n))


# ---------------------------------------------------------------------------
# multi-modulus oracle (opir_oracle_rns.c): R = 1 or 2 ciphertext primes, any
# power-of-two N up to 4096
# ---------------------------------------------------------------------------

ORR_MAX_RNS = 2


class OrrParams(ctypes.Structure):
    _fields_ = ([("n", ctypes.c_uint64), ("logn", ctypes.c_uint64), ("rns", ctypes.c_uint64),
                 ("q", ctypes.c_uint64 * ORR_MAX_RNS)]
                + [(f, ctypes.c_uint64) for f in (
                    "p", "t", "small_q", "small_q_width", "l", "base_log2", "l_key",
                    "base_log2_key", "num_entries", "num_pt", "entry_size", "entries_per_pt",
                    "bits_per_coeff", "n1", "n_rest", "ndim", "u", "h", "ms_mant")]
                + [("ms_exp", ctypes.c_int64)])


def _bind_rns(L):
    vp, u64 = ctypes.c_void_p, ctypes.c_uint64
    L.orr_create.restype = vp
    L.orr_create.argtypes = [u64] * 8 + [_u64p, u64]
    L.orr_destroy.argtypes = [vp]
    L.orr_get_params.argtypes = [vp, ctypes.POINTER(OrrParams)]
    for f in ("orr_ntt_fwd", "orr_ntt_inv"):
        getattr(L, f).argtypes = [vp, ctypes.c_int, _u64p, ctypes.c_size_t]
    L.orr_gen_entries.argtypes = [vp, u64, u64, u64, _u8p]
    L.orr_build_db.argtypes = [vp, u64, _u64p]
    L.orr_keygen.argtypes = [vp, u64, _i8p]
    L.orr_make_galois_keys.argtypes = [vp, _i8p, u64, _u64p]
    L.orr_make_gsw_key.argtypes = [vp, _i8p, u64, _u64p]
    L.orr_make_query.argtypes = [vp, _i8p, u64, u64, _u64p]
    L.orr_decrypt_small.argtypes = [vp, _i8p, _u64p, _u64p, ctypes.POINTER(ctypes.c_int)]
    L.orr_entry_from_plain.argtypes = [vp, u64, _u64p, _u8p]
    L.orr_apply_galois.argtypes = [vp, _u64p, u64, _u64p, _u64p]
    L.orr_expand.argtypes = [vp, _u64p, _u64p, _u64p]
    L.orr_gsw_to_ntt.argtypes = [vp, _u64p, u64, _u64p]
    L.orr_decompose.argtypes = [vp, _u64p, u64, u64, _u64p]
    L.orr_ext_product.argtypes = [vp, _u64p, u64, u64, _u64p, _u64p]
    L.orr_query_to_gsw.argtypes = [vp, _u64p, _u64p, _u64p]
    L.orr_first_dim.argtypes = [vp, _u64p, _u64p, _u64p]
    L.orr_first_dim.restype = ctypes.c_int
    L.orr_other_dim_mux.argtypes = [vp, _u64p, u64, _u64p]
    L.orr_mod_switch_next.argtypes = [vp, _u64p, _u64p]
    L.orr_mod_switch_coeff.argtypes = [vp, u64]
    L.orr_mod_switch_coeff.restype = u64
    L.orr_response_bytes.argtypes = [vp]
    L.orr_response_bytes.restype = u64
    L.orr_pack_response.argtypes = [vp, _u64p, _u8p]
    L.orr_pack_response.restype = u64
    L.orr_make_query_server.argtypes = [vp, _u64p, _u64p, _u64p, _u64p, _u64p, _u8p]
    L.orr_make_query_server.restype = ctypes.c_int


@dataclass
class RnsParams:
    n: int
    logn: int
    rns: int
    q: tuple
    p: int
    t: int
    small_q: int
    small_q_width: int
    l: int
    base_log2: int
    l_key: int
    base_log2_key: int
    num_entries: int
    num_pt: int
    entry_size: int
    entries_per_pt: int
    bits_per_coeff: int
    n1: int
    n_rest: int
    ndim: int
    u: int
    h: int
    ms_mant: int
    ms_exp: int


def _u64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint64)


class RnsOracle:
    """Multi-modulus oracle context (pir.cpp:29-95 for any N and CoeffMods).
    Ciphertexts are [2][R][N], RGSW rows [rows][2][R][N], Galois keys
    [h][R][2][R+1][N], the aligned database [R N][num_pt]."""

    def __init__(self, n: int, num_entries: int, max_fst_dim: int, entry_size: int = 0,
                 l: int = 4, l_key: int = 8, plain_bits: int = 46, small_q_width: int = 57,
                 coeff_bits=(60, 60, 60)):
        self.L = lib()
        bits = _u64(list(coeff_bits))
        self.h_ctx = self.L.orr_create(n, num_entries, max_fst_dim, entry_size, l, l_key,
                                       plain_bits, small_q_width, _p64(bits), bits.size)
        if not self.h_ctx:
            raise ValueError("invalid PIR parameters")
        op = OrrParams()
        self.L.orr_get_params(self.h_ctx, ctypes.byref(op))
        d = {f: int(getattr(op, f)) for f, _ in OrrParams._fields_ if f != "q"}
        d["q"] = tuple(int(op.q[i]) for i in range(int(op.rns)))
        self.P = RnsParams(**d)
        self.n, self.R = self.P.n, self.P.rns

    def __del__(self):
        if getattr(self, "h_ctx", None):
            self.L.orr_destroy(self.h_ctx)
            self.h_ctx = None

    @property
    def ct_shape(self):
        return (2, self.R, self.n)

    def ntt_fwd(self, a, mod=0):
        a = _u64(a).copy()
        self.L.orr_ntt_fwd(self.h_ctx, mod, _p64(a), a.size // self.n)
        return a

    def ntt_inv(self, a, mod=0):
        a = _u64(a).copy()
        self.L.orr_ntt_inv(self.h_ctx, mod, _p64(a), a.size // self.n)
        return a

    def gen_entries(self, seed, first, count):
        out = np.zeros(count * self.P.entry_size, np.uint8)
        self.L.orr_gen_entries(self.h_ctx, seed, first, count, _p8(out))
        return out.reshape(count, self.P.entry_size)

    def build_db(self, seed):
        db = np.zeros(self.R * self.n * self.P.num_pt, np.uint64)
        self.L.orr_build_db(self.h_ctx, seed, _p64(db))
        return db

    def keygen(self, seed):
        sk = np.zeros(self.n, np.int8)
        self.L.orr_keygen(self.h_ctx, seed, _pi8(sk))
        return sk

    def galois_keys(self, sk, seed):
        k = np.zeros(self.P.h * self.R * 2 * (self.R + 1) * self.n, np.uint64)
        self.L.orr_make_galois_keys(self.h_ctx, _pi8(sk), seed, _p64(k))
        return k.reshape(self.P.h, self.R, 2, self.R + 1, self.n)

    def gsw_key(self, sk, seed):
        rows = np.zeros(2 * self.P.l_key * 2 * self.R * self.n, np.uint64)
        self.L.orr_make_gsw_key(self.h_ctx, _pi8(sk), seed, _p64(rows))
        return rows.reshape(2 * self.P.l_key, 2, self.R, self.n)

    def make_query(self, sk, seed, entry_index):
        ct = np.zeros(2 * self.R * self.n, np.uint64)
        self.L.orr_make_query(self.h_ctx, _pi8(sk), seed, entry_index, _p64(ct))
        return ct.reshape(self.ct_shape)

    def decrypt_small(self, sk, ct):
        plain = np.zeros(self.n, np.uint64)
        b = ctypes.c_int()
        self.L.orr_decrypt_small(self.h_ctx, _pi8(sk), _p64(_u64(ct).reshape(-1)), _p64(plain),
                                 ctypes.byref(b))
        return plain, b.value

    def entry_from_plain(self, entry_index, plain):
        e = np.zeros(self.P.entry_size, np.uint8)
        self.L.orr_entry_from_plain(self.h_ctx, entry_index, _p64(_u64(plain)), _p8(e))
        return e

    def apply_galois(self, ct, g, key_level):
        out = np.zeros(2 * self.R * self.n, np.uint64)
        self.L.orr_apply_galois(self.h_ctx, _p64(_u64(ct).reshape(-1)), g,
                                _p64(_u64(key_level).reshape(-1)), _p64(out))
        return out.reshape(self.ct_shape)

    def expand(self, query, gk):
        out = np.zeros(self.P.u * 2 * self.R * self.n, np.uint64)
        self.L.orr_expand(self.h_ctx, _p64(_u64(query).reshape(-1)), _p64(_u64(gk).reshape(-1)),
                          _p64(out))
        return out.reshape((self.P.u,) + self.ct_shape)

    def gsw_to_ntt(self, rows):
        r = _u64(rows).reshape(-1)
        nrows = r.size // (2 * self.R * self.n)
        out = np.zeros_like(r)
        self.L.orr_gsw_to_ntt(self.h_ctx, _p64(r), nrows, _p64(out))
        return out.reshape((nrows,) + self.ct_shape)

    def decompose(self, ct, l, base_log2):
        out = np.zeros(2 * l * self.R * self.n, np.uint64)
        self.L.orr_decompose(self.h_ctx, _p64(_u64(ct).reshape(-1)), l, base_log2, _p64(out))
        return out.reshape(2 * l, self.R, self.n)

    def ext_product(self, gsw_ntt, l, base_log2, ct):
        out = np.zeros(2 * self.R * self.n, np.uint64)
        self.L.orr_ext_product(self.h_ctx, _p64(_u64(gsw_ntt).reshape(-1)), l, base_log2,
                               _p64(_u64(ct).reshape(-1)), _p64(out))
        return out.reshape(self.ct_shape)

    def query_to_gsw(self, cts, key_ntt):
        out = np.zeros(2 * self.P.l * 2 * self.R * self.n, np.uint64)
        self.L.orr_query_to_gsw(self.h_ctx, _p64(_u64(cts).reshape(-1)),
                                _p64(_u64(key_ntt).reshape(-1)), _p64(out))
        return out.reshape((2 * self.P.l,) + self.ct_shape)

    def first_dim(self, db, fst):
        out = np.zeros(self.P.n_rest * 2 * self.R * self.n, np.uint64)
        w = self.L.orr_first_dim(self.h_ctx, _p64(_u64(db)), _p64(_u64(fst).reshape(-1)), _p64(out))
        return out.reshape((self.P.n_rest,) + self.ct_shape), w

    def other_dim_mux(self, result, gsw_ntt):
        r = _u64(result).copy()
        self.L.orr_other_dim_mux(self.h_ctx, _p64(r.reshape(-1)), r.shape[0],
                                 _p64(_u64(gsw_ntt).reshape(-1)))
        return r[: r.shape[0] // 2]

    def mod_switch_next(self, ct):
        out = np.zeros(2 * (self.R - 1) * self.n, np.uint64)
        self.L.orr_mod_switch_next(self.h_ctx, _p64(_u64(ct).reshape(-1)), _p64(out))
        return out.reshape(2, self.R - 1, self.n)

    def mod_switch_coeff(self, x):
        return int(self.L.orr_mod_switch_coeff(self.h_ctx, x))

    def response_bytes(self):
        return int(self.L.orr_response_bytes(self.h_ctx))

    def pack_response(self, ct):
        out = np.zeros(self.response_bytes(), np.uint8)
        self.L.orr_pack_response(self.h_ctx, _p64(_u64(ct).reshape(-1)), _p8(out))
        return out

    def make_query_server(self, db, gk, gsw_key_ntt, query):
        resp = np.zeros(2 * self.n, np.uint64)
        packed = np.zeros(self.response_bytes(), np.uint8)
        w = self.L.orr_make_query_server(self.h_ctx, _p64(_u64(db)), _p64(_u64(gk).reshape(-1)),
                                         _p64(_u64(gsw_key_ntt).reshape(-1)),
                                         _p64(_u64(query).reshape(-1)), _p64(resp), _p8(packed))
        return resp.reshape(2, self.n), packed, w
