"""ctypes binding of the C ABI in ``include/onionpir_gpu.h``.

The library is the in-tree ``_build/libopir_gb300.so``.  There is no CPU
fallback: if the library is missing or no GPU is present, loading fails
loudly.
"""
from __future__ import annotations

import ctypes
import os

from .build import LIB

_u64p = ctypes.POINTER(ctypes.c_uint64)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_vp = ctypes.c_void_p

OPIR_OK = 0
STATUS = {
    0: "OPIR_OK",
    -1: "OPIR_ERR_ARG",
    -2: "OPIR_ERR_UNKNOWN_CLIENT",
    -3: "OPIR_ERR_UNKNOWN_DB",
    -4: "OPIR_ERR_OOM",
    -5: "OPIR_ERR_CUDA",
    -6: "OPIR_ERR_STATE",
    -7: "OPIR_ERR_NO_DEVICE",
    -8: "OPIR_ERR_TIMEOUT",
}

# every symbol include/onionpir_gpu.h declares
EXPORTS = (
    "opir_ctx_create", "opir_ctx_destroy", "opir_ctx_set_stream", "opir_last_error",
    "opir_response_bytes", "opir_db_create", "opir_db_destroy", "opir_db_push_chunk",
    "opir_db_fill_synthetic", "opir_db_upload_aligned", "opir_set_galois_key",
    "opir_set_gsw_key", "opir_erase_client", "opir_make_query", "opir_make_query_batch",
    "opir_make_query_device", "opir_make_query_trace", "opir_first_dim_noalloc",
    "opir_set_timing", "opir_stage_times",
    "opir_launch_count", "opir_sync", "opir_ntt", "opir_ntt_device",
    "opir_set_key_budget", "opir_key_bytes_per_client", "opir_resident_clients",
    "opir_serve_start", "opir_serve_stop", "opir_submit", "opir_poll", "opir_wait",
    "opir_serve_stats_get", "opir_set_batch_engine", "opir_autotune", "opir_set_graphs",
    "opir_db_get_entry", "opir_pack_response", "opir_other_dim_mux",
    "opir_debug_withhold_scan_stage", "opir_debug_first_dim", "opir_ctx_create_rns",
)

ENGINES = {"auto": 0, "scan": 1, "imad": 2, "tensor": 3}


class OpirParams(ctypes.Structure):
    _fields_ = [
        ("poly_degree", ctypes.c_uint32),
        ("coeff_modulus", ctypes.c_uint64),
        ("special_modulus", ctypes.c_uint64),
        ("plain_modulus", ctypes.c_uint64),
        ("small_modulus", ctypes.c_uint64),
        ("gsw_l", ctypes.c_uint32),
        ("gsw_base_log2", ctypes.c_uint32),
        ("gsw_l_key", ctypes.c_uint32),
        ("gsw_base_log2_key", ctypes.c_uint32),
    ]


class OpirRnsParams(ctypes.Structure):
    _fields_ = [
        ("poly_degree", ctypes.c_uint32),
        ("rns_count", ctypes.c_uint32),
        ("coeff_moduli", ctypes.c_uint64 * 2),
        ("special_modulus", ctypes.c_uint64),
        ("plain_modulus", ctypes.c_uint64),
        ("small_modulus", ctypes.c_uint64),
        ("gsw_l", ctypes.c_uint32),
        ("gsw_base_log2", ctypes.c_uint32),
        ("gsw_l_key", ctypes.c_uint32),
        ("gsw_base_log2_key", ctypes.c_uint32),
    ]


class OpirDbShape(ctypes.Structure):
    _fields_ = [
        ("fst_dim_sz", ctypes.c_uint32),
        ("other_dim_sz", ctypes.c_uint32),
        ("entry_size", ctypes.c_uint32),
        ("entries_per_pt", ctypes.c_uint32),
        ("bits_per_coeff", ctypes.c_uint32),
    ]


class OpirServeConfig(ctypes.Structure):
    _fields_ = [
        ("max_batch", ctypes.c_uint32),
        ("lanes", ctypes.c_uint32),
        ("max_wait_us", ctypes.c_uint32),
    ]


class OpirServeStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_uint64),
        ("completed", ctypes.c_uint64),
        ("failed", ctypes.c_uint64),
        ("batches", ctypes.c_uint64),
        ("queued", ctypes.c_uint64),
        ("mean_batch", ctypes.c_double),
        ("p50_ms", ctypes.c_double),
        ("p99_ms", ctypes.c_double),
        ("mean_ms", ctypes.c_double),
        ("max_ms", ctypes.c_double),
        ("queries_per_s", ctypes.c_double),
    ]


class OpirTuneReport(ctypes.Structure):
    _fields_ = [
        ("scan_configs", ctypes.c_uint32),
        ("scan_desc", (ctypes.c_uint32 * 6) * 16),
        ("scan_ms", ctypes.c_float * 16),
        ("scan_choice", ctypes.c_int32),
        ("batch_points", ctypes.c_uint32),
        ("batch", ctypes.c_uint32 * 8),
        ("engine_ms", (ctypes.c_float * 3) * 8),
        ("engine", ctypes.c_int32 * 8),
        ("tc_ring_desc", (ctypes.c_uint32 * 2) * 2),
        ("tc_ring_ms", ctypes.c_float * 2),
        ("tc_ring_choice", ctypes.c_int32),
        ("form_points", ctypes.c_uint32),
        ("form_stage", ctypes.c_uint32 * 128),
        ("form_count", ctypes.c_uint32 * 128),
        ("form_ms", (ctypes.c_float * 4) * 128),
        ("form_choice", ctypes.c_int32 * 128),
        ("tc_limbs_ms", ctypes.c_float * 2),
        ("tc_limbs_choice", ctypes.c_int32),
        ("tc_pair_ms", ctypes.c_float * 2),
        ("tc_pair_choice", ctypes.c_int32),
    ]


class OpirError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class UnknownClientError(OpirError, KeyError):
    """No keys registered for a client id (the reference's std::out_of_range)."""


_lib = None


def load(path: str = LIB):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"{path} not found: build the CUDA extension first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    L = ctypes.CDLL(path)
    L.opir_ctx_create.argtypes = [ctypes.POINTER(OpirParams), ctypes.c_int, ctypes.POINTER(_vp)]
    L.opir_ctx_create_rns.argtypes = [ctypes.POINTER(OpirRnsParams), ctypes.c_int,
                                      ctypes.POINTER(_vp)]
    L.opir_ctx_destroy.argtypes = [_vp]
    L.opir_ctx_destroy.restype = None
    L.opir_ctx_set_stream.argtypes = [_vp, _vp]
    L.opir_last_error.argtypes = [_vp]
    L.opir_last_error.restype = ctypes.c_char_p
    L.opir_response_bytes.argtypes = [_vp]
    L.opir_response_bytes.restype = ctypes.c_uint64
    L.opir_db_create.argtypes = [_vp, ctypes.POINTER(OpirDbShape), ctypes.POINTER(ctypes.c_uint32)]
    L.opir_db_destroy.argtypes = [_vp, ctypes.c_uint32]
    L.opir_db_push_chunk.argtypes = [_vp, ctypes.c_uint32, _u8p, ctypes.c_uint64, ctypes.c_uint64]
    L.opir_db_fill_synthetic.argtypes = [_vp, ctypes.c_uint32, ctypes.c_uint64]
    L.opir_db_upload_aligned.argtypes = [_vp, ctypes.c_uint32, _u64p]
    L.opir_set_galois_key.argtypes = [_vp, ctypes.c_uint64, _u64p, ctypes.c_uint32]
    L.opir_set_gsw_key.argtypes = [_vp, ctypes.c_uint64, _u64p]
    L.opir_erase_client.argtypes = [_vp, ctypes.c_uint64]
    L.opir_make_query.argtypes = [_vp, ctypes.c_uint32, ctypes.c_uint64, _u64p, _u64p, _u8p]
    L.opir_make_query_batch.argtypes = [_vp, ctypes.c_uint32, ctypes.c_uint32, _u64p, _u64p, _u64p,
                                        _u8p]
    L.opir_make_query_device.argtypes = [_vp, ctypes.c_uint32, ctypes.c_uint32, _u64p, _vp, _vp,
                                         _vp]
    L.opir_make_query_trace.argtypes = [_vp, ctypes.c_uint32, ctypes.c_uint64, _u64p, _u64p, _u64p,
                                        _u64p, _u64p, _u8p]
    L.opir_first_dim_noalloc.argtypes = [_vp, ctypes.c_uint32, _vp, _vp]
    L.opir_pack_response.argtypes = [_vp, _u64p, ctypes.c_uint32, _u8p]
    L.opir_other_dim_mux.argtypes = [_vp, _u64p, ctypes.c_uint64, _u64p]
    L.opir_debug_withhold_scan_stage.argtypes = [_vp, ctypes.c_uint32]
    L.opir_debug_first_dim.argtypes = [_vp, ctypes.c_uint32, ctypes.c_uint32, _u64p, _u64p]
    L.opir_set_timing.argtypes = [_vp, ctypes.c_int]
    L.opir_set_graphs.argtypes = [_vp, ctypes.c_int]
    L.opir_db_get_entry.argtypes = [_vp, ctypes.c_uint32, ctypes.c_uint64, _u8p]
    L.opir_stage_times.argtypes = [_vp, ctypes.POINTER(ctypes.c_float)]
    L.opir_launch_count.argtypes = [_vp]
    L.opir_launch_count.restype = ctypes.c_uint64
    L.opir_sync.argtypes = [_vp]
    L.opir_ntt_device.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _vp, ctypes.c_uint64]
    L.opir_ntt.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _u64p, ctypes.c_uint64]
    L.opir_set_key_budget.argtypes = [_vp, ctypes.c_uint64]
    L.opir_key_bytes_per_client.argtypes = [_vp]
    L.opir_key_bytes_per_client.restype = ctypes.c_uint64
    L.opir_resident_clients.argtypes = [_vp, ctypes.POINTER(ctypes.c_uint32),
                                        ctypes.POINTER(ctypes.c_uint32)]
    L.opir_serve_start.argtypes = [_vp, ctypes.POINTER(OpirServeConfig)]
    L.opir_serve_stop.argtypes = [_vp]
    L.opir_submit.argtypes = [_vp, ctypes.c_uint32, ctypes.c_uint64, _u64p,
                              ctypes.POINTER(ctypes.c_uint64)]
    L.opir_poll.argtypes = [_vp, ctypes.c_uint64, _u64p, _u8p, ctypes.POINTER(ctypes.c_int)]
    L.opir_wait.argtypes = [_vp, ctypes.c_uint64, ctypes.c_uint32, _u64p, _u8p]
    L.opir_serve_stats_get.argtypes = [_vp, ctypes.POINTER(OpirServeStats)]
    L.opir_set_batch_engine.argtypes = [_vp, ctypes.c_int, ctypes.c_uint32]
    L.opir_autotune.argtypes = [_vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                ctypes.POINTER(OpirTuneReport)]
    _lib = L
    return L


def check(ctx, rc: int):
    if rc != OPIR_OK:
        msg = load().opir_last_error(ctx).decode() if ctx else ""
        if rc == -2:
            raise UnknownClientError(rc, msg)
        raise OpirError(rc, msg)


def p64(a):
    return a.ctypes.data_as(_u64p) if a is not None else None


def p8(a):
    return a.ctypes.data_as(_u8p) if a is not None else None
