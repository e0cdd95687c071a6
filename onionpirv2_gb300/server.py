"""PirServer: the reference server interface (src/includes/server.h:13-51)
on the GB300 query path.

Method names, argument meaning and error behaviour follow the reference:
  gen_data()                        server.cpp:47-78   (seeded entries, ingested on the GPU)
  push_database_chunk(chunk, idx)   server.cpp:635-701 (+ preprocess_ntt, realign_db)
  set_client_galois_key(id, keys)   server.cpp:480-484
  set_client_gsw_key(id, rows)      server.cpp:486-500
  make_query(id, query)             server.cpp:520-579
  save_resp_to_stream(resp, stream) server.cpp:581-633
  direct_get_entry(idx)             server.cpp:503-517
Unknown client ids raise UnknownClientError (a KeyError, like the
reference's std::map::at); malformed arguments raise ValueError.

Ciphertexts are numpy uint64 arrays of shape (2, N) in SEAL's rns = 1
layout (c0 then c1, coefficient form).  Every computation runs in the CUDA
library through the C ABI; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import io
from typing import Optional, Sequence

import numpy as np

from . import _capi
from .params import POLY_DEGREE, PirParams

N = POLY_DEGREE


def _mix64(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def synthetic_entries(seed: int, first: int, count: int, entry_size: int) -> np.ndarray:
    """Entries of the seeded database (utils.cpp:160-172 with a seeded
    generator in place of /dev/urandom): 8-byte big-endian index, then bytes
    of mix64(seed * phi + entry * c + word)."""
    out = np.zeros((count, entry_size), np.uint8)
    idx = np.arange(first, first + count, dtype=np.uint64)
    for i in range(8):
        out[:, 7 - i] = ((idx >> np.uint64(8 * i)) & np.uint64(0xFF)).astype(np.uint8)
    nwords = (entry_size - 8 + 7) // 8
    with np.errstate(over="ignore"):
        base = np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15) + idx * np.uint64(0xD1B54A32D192ED03)
        words = _mix64(base[:, None] + np.arange(nwords, dtype=np.uint64)[None, :])
    raw = words.astype("<u8").view(np.uint8).reshape(count, nwords * 8)
    out[:, 8:] = raw[:, : entry_size - 8]
    return out


class ResponseCiphertext(np.ndarray):
    """Response ciphertext mod small_q (2, N) carrying its packed wire bytes."""

    packed: Optional[bytes] = None


class PirServer:
    """GPU-backed PirServer (one CUDA context, one database)."""

    def __init__(self, pir_params: PirParams, device: int = 0):
        self.pir_params = pir_params
        self._L = _capi.load()
        P = pir_params
        self.n, self.R = P.poly_degree, P.get_rns_mod_cnt()
        ctx = ctypes.c_void_p()
        if P.is_multi_modulus():
            qs = P.get_coeff_modulus()
            prm = _capi.OpirRnsParams(
                poly_degree=P.poly_degree, rns_count=self.R,
                coeff_moduli=(ctypes.c_uint64 * 2)(*(qs + [0] * (2 - len(qs)))),
                special_modulus=P.coeff_modulus[-1], plain_modulus=P.plain_mod,
                small_modulus=P.small_q, gsw_l=P.gsw_l, gsw_base_log2=P.base_log2,
                gsw_l_key=P.gsw_l_key, gsw_base_log2_key=P.base_log2_key)
            rc = self._L.opir_ctx_create_rns(ctypes.byref(prm), device, ctypes.byref(ctx))
        else:
            prm = _capi.OpirParams(
                poly_degree=P.poly_degree, coeff_modulus=P.coeff_modulus[0],
                special_modulus=P.coeff_modulus[-1], plain_modulus=P.plain_mod,
                small_modulus=P.small_q, gsw_l=P.gsw_l, gsw_base_log2=P.base_log2,
                gsw_l_key=P.gsw_l_key, gsw_base_log2_key=P.base_log2_key)
            rc = self._L.opir_ctx_create(ctypes.byref(prm), device, ctypes.byref(ctx))
        if rc != 0:
            raise _capi.OpirError(rc, "opir_ctx_create failed")
        self._ctx = ctx
        shape = _capi.OpirDbShape(
            fst_dim_sz=P.get_fst_dim_sz(), other_dim_sz=P.get_other_dim_sz(),
            entry_size=P.get_entry_size(), entries_per_pt=P.get_num_entries_per_plaintext(),
            bits_per_coeff=P.get_num_bits_per_coeff())
        db = ctypes.c_uint32()
        self._check(self._L.opir_db_create(self._ctx, ctypes.byref(shape), ctypes.byref(db)))
        self.db_id = db.value
        self._db_entry_size = {}  # databases added with add_database
        self.resp_bytes = int(self._L.opir_response_bytes(self._ctx))

    @property
    def ct_words(self) -> int:
        """uint64 words of one query ciphertext: 2 R N (SEAL's [2][R][N])."""
        return 2 * self.R * self.n

    # ---- plumbing
    def _check(self, rc: int):
        _capi.check(self._ctx, rc)

    def close(self):
        if getattr(self, "_ctx", None):
            self._L.opir_ctx_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ctx(self):
        return self._ctx

    def set_stream(self, stream_handle: int):
        """Run on a caller's cudaStream_t (e.g. torch.cuda.Stream().cuda_stream)."""
        self._check(self._L.opir_ctx_set_stream(self._ctx, ctypes.c_void_p(stream_handle)))

    # ---- database
    def gen_data(self, seed: int = 0x0B1A7):
        """Fill the whole database with seeded entries (server.cpp:47-78)."""
        self._check(self._L.opir_db_fill_synthetic(self._ctx, self.db_id, seed))

    def push_database_chunk(self, chunk_entry, chunk_idx: int):
        """Pack, NTT and realign one chunk of fst_dim_sz plaintexts
        (server.cpp:635-748).  Entries shorter than entry_size are zero-padded;
        longer ones raise ValueError."""
        P = self.pir_params
        es = P.get_entry_size()
        n = P.get_fst_dim_sz() * P.get_num_entries_per_plaintext()
        if isinstance(chunk_entry, np.ndarray) and chunk_entry.dtype == np.uint8 and chunk_entry.ndim == 2:
            if chunk_entry.shape[1] > es:
                raise ValueError("Entry size is too large")
            arr = np.zeros((chunk_entry.shape[0], es), np.uint8)
            arr[:, : chunk_entry.shape[1]] = chunk_entry
        else:
            rows = list(chunk_entry)
            arr = np.zeros((len(rows), es), np.uint8)
            for i, e in enumerate(rows):
                b = np.frombuffer(bytes(e), np.uint8)
                if b.size > es:
                    raise ValueError("Entry size is too large")
                arr[i, : b.size] = b
        if arr.shape[0] != n:
            raise ValueError(f"a chunk holds {n} entries, got {arr.shape[0]}")
        arr = np.ascontiguousarray(arr)
        self._check(self._L.opir_db_push_chunk(self._ctx, self.db_id, _capi.p8(arr.reshape(-1)),
                                               n, chunk_idx))

    def upload_ntt_db(self, db_aligned: np.ndarray):
        """Install an NTT-form database given in the reference layout
        db_aligned_[c * num_pt + row * n1 + col] (server.cpp:740)."""
        a = np.ascontiguousarray(db_aligned, np.uint64)
        if a.size != self.pir_params.get_num_pt() * self.n * self.R:
            raise ValueError("database has the wrong size")
        self._check(self._L.opir_db_upload_aligned(self._ctx, self.db_id, _capi.p64(a.reshape(-1))))

    def direct_get_entry(self, entry_idx: int, db_id: Optional[int] = None) -> np.ndarray:
        """Non-private lookup of an entry, for testing (server.cpp:503-517):
        decoded from the device database (its plaintext inverse-transformed
        and unpacked)."""
        out = np.zeros(self.pir_params.get_entry_size() if db_id is None else
                       self._db_entry_size.get(db_id, self.pir_params.get_entry_size()), np.uint8)
        self._check(self._L.opir_db_get_entry(self._ctx, self.db_id if db_id is None else db_id,
                                              entry_idx, _capi.p8(out)))
        return out

    # ---- keys
    def set_client_galois_key(self, client_id: int, galois_keys):
        keys = _read_u64(galois_keys)
        per = self.R * 2 * (self.R + 1) * self.n  # [R][2][R+1][N] per level
        levels = keys.size // per
        if levels * per != keys.size or levels == 0:
            raise ValueError("Galois keys must be [levels][R][2][R+1][N] uint64")
        self._check(self._L.opir_set_galois_key(self._ctx, client_id, _capi.p64(keys), levels))

    def set_client_gsw_key(self, client_id: int, gsw_rows):
        rows = _read_u64(gsw_rows)
        if rows.size != 2 * self.pir_params.get_l_key() * self.ct_words:
            raise ValueError("RGSW key must be [2*l_key][2][R][N] uint64")
        self._check(self._L.opir_set_gsw_key(self._ctx, client_id, _capi.p64(rows)))

    def erase_client(self, client_id: int):
        self._check(self._L.opir_erase_client(self._ctx, client_id))

    # ---- queries
    def make_query(self, client_id: int, query, db_id: Optional[int] = None) -> ResponseCiphertext:
        """Answer one query (server.cpp:520-579); returns the response
        ciphertext mod small_q with its packed bytes attached.  `db_id`
        selects a database added with add_database (default: this server's)."""
        q = _read_u64(query)
        if q.size != self.ct_words:
            raise ValueError("query must be one ciphertext [2][R][N]")
        resp = np.zeros(2 * self.n, np.uint64)
        packed = np.zeros(self.resp_bytes, np.uint8)
        self._check(self._L.opir_make_query(self._ctx, self.db_id if db_id is None else db_id,
                                            client_id, _capi.p64(q), _capi.p64(resp),
                                            _capi.p8(packed)))
        out = resp.reshape(2, self.n).view(ResponseCiphertext)
        out.packed = packed.tobytes()
        return out

    def make_query_batch(self, client_ids: Sequence[int], queries: np.ndarray):
        """Answer len(client_ids) queries in one batched pass."""
        ids = np.ascontiguousarray(np.asarray(client_ids, dtype=np.uint64))
        q = np.ascontiguousarray(queries, np.uint64).reshape(-1)
        B = ids.size
        if q.size != B * self.ct_words:
            raise ValueError("queries must be [batch][2][R][N]")
        resp = np.zeros(B * 2 * self.n, np.uint64)
        packed = np.zeros(B * self.resp_bytes, np.uint8)
        self._check(self._L.opir_make_query_batch(self._ctx, self.db_id, B, _capi.p64(ids),
                                                  _capi.p64(q), _capi.p64(resp), _capi.p8(packed)))
        return resp.reshape(B, 2, self.n), packed.reshape(B, self.resp_bytes)

    def make_query_device(self, client_ids: Sequence[int], d_queries: int, d_resps: int,
                          d_packed: int):
        """Enqueue a batch on the context stream with device pointers
        (queries [B][2][N] u64, responses [B][2][N] u64, packed [B][bytes])."""
        ids = np.ascontiguousarray(np.asarray(client_ids, dtype=np.uint64))
        self._check(self._L.opir_make_query_device(
            self._ctx, self.db_id, ids.size, _capi.p64(ids), ctypes.c_void_p(d_queries),
            ctypes.c_void_p(d_resps), ctypes.c_void_p(d_packed)))

    def make_query_trace(self, client_id: int, query):
        """make_query returning every intermediate (parity tests); shapes
        [u][2][R][N], [ndim-1][2l][2][R][N], [n_rest][2][R][N] (R = 1: the
        prime axis is dropped)."""
        P = self.pir_params
        q = _read_u64(query)
        ndim = len(P.get_dims())
        u = P.get_fst_dim_sz() + P.get_l() * (ndim - 1)
        cw = self.ct_words
        leaves = np.zeros(u * cw, np.uint64)
        gsw = np.zeros(max(ndim - 1, 1) * 2 * P.get_l() * cw, np.uint64)
        fd = np.zeros(P.get_other_dim_sz() * cw, np.uint64)
        resp = np.zeros(2 * self.n, np.uint64)
        packed = np.zeros(self.resp_bytes, np.uint8)
        self._check(self._L.opir_make_query_trace(
            self._ctx, self.db_id, client_id, _capi.p64(q), _capi.p64(leaves), _capi.p64(gsw),
            _capi.p64(fd), _capi.p64(resp), _capi.p8(packed)))
        ct = (2, self.n) if self.R == 1 else (2, self.R, self.n)
        return dict(leaves=leaves.reshape((u,) + ct),
                    gsw=gsw.reshape((max(ndim - 1, 1), 2 * P.get_l()) + ct),
                    first_dim=fd.reshape((-1,) + ct), resp=resp.reshape(2, self.n),
                    packed=packed)

    def save_resp_to_stream(self, response, stream: io.IOBase) -> int:
        """Write the response's packed bytes (server.cpp:581-633); returns the
        number of bytes written.  Any response ciphertext mod small_q ((2, N)
        uint64) is accepted: one that carries the bytes the GPU packed with it
        (make_query, poll, wait) is written as is, any other (a row of a
        batch, a stored ciphertext) is packed on the GPU (opir_pack_response)."""
        packed = getattr(response, "packed", None)
        if packed is None:
            packed = self.pack_responses(np.asarray(response).reshape(1, 2, self.n))[0].tobytes()
        stream.write(packed)
        return len(packed)

    def pack_responses(self, responses) -> np.ndarray:
        """The reference's packed wire bytes of every response
        ([count][2][N] mod small_q) -> uint8 [count][resp_bytes]."""
        r = np.ascontiguousarray(responses, np.uint64)
        if r.size == 0 or r.size % (2 * self.n):
            raise ValueError("responses must be [count][2][N] uint64")
        count = r.size // (2 * self.n)
        out = np.zeros(count * self.resp_bytes, np.uint8)
        self._check(self._L.opir_pack_response(self._ctx, _capi.p64(r.reshape(-1)), count,
                                               _capi.p8(out)))
        return out.reshape(count, self.resp_bytes)

    def other_dim_mux(self, result, selection_cipher) -> np.ndarray:
        """One folding level (server.cpp:295-334): result [count][2][N]
        (coefficient form mod q, count even) and the RGSW selection
        ciphertext [2l][2][N] (NTT form) -> the count/2 ciphertexts
        result[i] + INTT(RGSW(b) x (result[i + count/2] - result[i]))."""
        r = np.ascontiguousarray(result, np.uint64).copy()
        sel = np.ascontiguousarray(selection_cipher, np.uint64)
        if r.size % (2 * N) or (r.size // (2 * N)) % 2:
            raise ValueError("result must hold an even number of ciphertexts [count][2][N]")
        if sel.size != 2 * self.pir_params.get_l() * 2 * N:
            raise ValueError("selection_cipher must be one RGSW ciphertext [2l][2][N]")
        count = r.size // (2 * N)
        self._check(self._L.opir_other_dim_mux(self._ctx, _capi.p64(r.reshape(-1)), count,
                                               _capi.p64(sel.reshape(-1))))
        return r.reshape(count, 2, N)[: count // 2].copy()

    # ---- further databases on this context (served side by side)
    def add_database(self, pir_params: PirParams, seed: Optional[int] = None) -> int:
        """Create another resident database with the same ciphertext
        parameters; filled with seeded entries when `seed` is given.  Returns
        its id (the constructor's database is ``self.db_id``)."""
        P, Q = pir_params, self.pir_params
        if (P.coeff_modulus, P.plain_mod, P.small_q, P.gsw_l, P.gsw_l_key) != (
                Q.coeff_modulus, Q.plain_mod, Q.small_q, Q.gsw_l, Q.gsw_l_key):
            raise ValueError("a database on this context must share its ciphertext parameters")
        shape = _capi.OpirDbShape(
            fst_dim_sz=P.get_fst_dim_sz(), other_dim_sz=P.get_other_dim_sz(),
            entry_size=P.get_entry_size(), entries_per_pt=P.get_num_entries_per_plaintext(),
            bits_per_coeff=P.get_num_bits_per_coeff())
        db = ctypes.c_uint32()
        self._check(self._L.opir_db_create(self._ctx, ctypes.byref(shape), ctypes.byref(db)))
        if seed is not None:
            self._check(self._L.opir_db_fill_synthetic(self._ctx, db.value, seed))
        self._db_entry_size[db.value] = P.get_entry_size()
        return db.value

    # ---- key budget (client keys in a bounded pool, least recently used out)
    def set_key_budget(self, nbytes: int):
        self._check(self._L.opir_set_key_budget(self._ctx, int(nbytes)))

    def key_bytes_per_client(self) -> int:
        return int(self._L.opir_key_bytes_per_client(self._ctx))

    def resident_clients(self):
        """(clients with keys in device memory, slots of the budget or 0)"""
        r, sl = ctypes.c_uint32(), ctypes.c_uint32()
        self._check(self._L.opir_resident_clients(self._ctx, ctypes.byref(r), ctypes.byref(sl)))
        return r.value, sl.value

    # ---- first-dimension engine of batches
    def set_batch_engine(self, engine: str = "auto", tensor_min_batch: int = 0):
        """'auto' (tensor cores when the shape allows, from tensor_min_batch
        queries on), 'scan' (one pass per query), 'imad' or 'tensor'."""
        self._check(self._L.opir_set_batch_engine(self._ctx, _capi.ENGINES[engine],
                                                  tensor_min_batch))

    # ---- serving: continuous batching
    def autotune(self, max_batch: int = 64, reps: int = 3, db_id: Optional[int] = None) -> dict:
        """Measure every scan tile configuration and every first-dimension
        engine at batch sizes 2 .. max_batch on this GPU for one database,
        and adopt the fastest (opir_autotune).  Returns the measurements."""
        r = _capi.OpirTuneReport()
        self._check(self._L.opir_autotune(self._ctx, self.db_id if db_id is None else db_id,
                                          max_batch, reps, ctypes.byref(r)))
        names = {1: "scan", 2: "imad", 3: "tensor"}
        keys = ("rows", "warps", "ksteps", "stages", "ctas_per_sm", "karatsuba")
        stages = ("expand", "query_to_gsw", "fold")
        forms = ("one_cta", "two_cta", "cluster", "wide_cluster")
        return {
            "scan_configs": [dict(zip(keys, list(r.scan_desc[i])), ms=float(r.scan_ms[i]))
                             for i in range(r.scan_configs)],
            "scan_choice": int(r.scan_choice),
            "batches": [{"batch": int(r.batch[i]),
                         "ms": {names[e + 1]: float(r.engine_ms[i][e]) for e in range(3)},
                         "engine": names.get(int(r.engine[i]), "scan")}
                        for i in range(r.batch_points)],
            "tc_rings": [{"k_per_stage": int(r.tc_ring_desc[i][0]),
                          "stages": int(r.tc_ring_desc[i][1]), "ms": float(r.tc_ring_ms[i])}
                         for i in range(2)],
            "tc_ring_choice": int(r.tc_ring_choice),
            "tc_limbs": [{"bits": 8 + i, "ms": float(r.tc_limbs_ms[i])} for i in range(2)],
            "tc_limbs_choice": (8 + int(r.tc_limbs_choice)) if r.tc_limbs_choice >= 0 else None,
            "tc_forms": [{"form": ("one_cta", "cta_pair")[i], "ms": float(r.tc_pair_ms[i])}
                         for i in range(2)],
            "tc_form_choice": (("one_cta", "cta_pair")[r.tc_pair_choice]
                               if r.tc_pair_choice >= 0 else None),
            "forms": [{"stage": stages[r.form_stage[i]], "count": int(r.form_count[i]),
                       "ms": {forms[f]: float(r.form_ms[i][f]) for f in range(4)},
                       "form": forms[r.form_choice[i]] if r.form_choice[i] >= 0 else None}
                      for i in range(r.form_points)],
        }

    def serve_start(self, max_batch: int = 32, lanes: int = 2, max_wait_us: int = 2000):
        cfg = _capi.OpirServeConfig(max_batch=max_batch, lanes=lanes, max_wait_us=max_wait_us)
        self._check(self._L.opir_serve_start(self._ctx, ctypes.byref(cfg)))

    def serve_stop(self):
        self._check(self._L.opir_serve_stop(self._ctx))

    def submit(self, client_id: int, query, db_id: Optional[int] = None) -> int:
        """Queue one query; returns its ticket."""
        q = _read_u64(query)
        if q.size != 2 * N:
            raise ValueError("query must be one ciphertext [2][N]")
        t = ctypes.c_uint64()
        self._check(self._L.opir_submit(self._ctx, self.db_id if db_id is None else db_id,
                                        client_id, _capi.p64(q), ctypes.byref(t)))
        return t.value

    def _response(self, resp, packed) -> ResponseCiphertext:
        out = resp.reshape(2, N).view(ResponseCiphertext)
        out.packed = packed.tobytes()
        return out

    def poll(self, ticket: int) -> Optional[ResponseCiphertext]:
        """The response of a ticket, or None while it is queued or running."""
        resp = np.zeros(2 * N, np.uint64)
        packed = np.zeros(self.resp_bytes, np.uint8)
        done = ctypes.c_int()
        self._check(self._L.opir_poll(self._ctx, ticket, _capi.p64(resp), _capi.p8(packed),
                                      ctypes.byref(done)))
        return self._response(resp, packed) if done.value else None

    def wait(self, ticket: int, timeout_ms: int = 60000) -> ResponseCiphertext:
        resp = np.zeros(2 * N, np.uint64)
        packed = np.zeros(self.resp_bytes, np.uint8)
        self._check(self._L.opir_wait(self._ctx, ticket, timeout_ms, _capi.p64(resp),
                                      _capi.p8(packed)))
        return self._response(resp, packed)

    def serve_stats(self) -> dict:
        st = _capi.OpirServeStats()
        self._check(self._L.opir_serve_stats_get(self._ctx, ctypes.byref(st)))
        return {name: getattr(st, name) for name, _ in st._fields_}

    # ---- timing / accounting
    def set_graphs(self, enable: bool = True):
        """Replay single queries from a captured CUDA graph (default on)."""
        self._check(self._L.opir_set_graphs(self._ctx, 1 if enable else 0))

    def set_timing(self, enable: bool = True):
        self._check(self._L.opir_set_timing(self._ctx, 1 if enable else 0))

    def stage_times(self):
        """Device ms of the last timed query: Expand, Convert, First dim,
        Other dim, Mod switch, and the scan kernel alone."""
        ms = (ctypes.c_float * 6)()
        self._check(self._L.opir_stage_times(self._ctx, ms))
        keys = ("expand", "convert", "first_dim", "other_dim", "mod_switch", "scan_kernel")
        return dict(zip(keys, [float(x) for x in ms]))

    def launch_count(self) -> int:
        return int(self._L.opir_launch_count(self._ctx))

    def ntt(self, polys: np.ndarray, mod: int = 0, inverse: bool = False) -> np.ndarray:
        a = np.ascontiguousarray(polys, np.uint64).copy()
        self._check(self._L.opir_ntt(self._ctx, mod, 1 if inverse else 0, _capi.p64(a.reshape(-1)),
                                     a.size // self.n))
        return a


def _read_u64(x) -> np.ndarray:
    if isinstance(x, (io.IOBase, io.BytesIO)):
        return np.frombuffer(x.read(), dtype="<u8").astype(np.uint64)
    if isinstance(x, (bytes, bytearray, memoryview)):
        return np.frombuffer(bytes(x), dtype="<u8").astype(np.uint64)
    return np.ascontiguousarray(x, np.uint64).reshape(-1)
