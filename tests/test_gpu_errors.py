"""Error behaviour of the C ABI (no reference counterpart beyond the
exceptions of server.cpp): invalid parameter sets and shapes are rejected
with OPIR_ERR_ARG, unknown databases and clients with their own codes, calls
in the wrong state with OPIR_ERR_STATE -- and the context stays usable after
each of them."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048


def _params(**over):
    from onionpirv2_gb300 import PirParams, _capi
    P = PirParams(num_entries=4096, max_fst_dim=256)
    d = dict(poly_degree=P.poly_degree, coeff_modulus=P.coeff_modulus[0],
             special_modulus=P.coeff_modulus[-1], plain_modulus=P.plain_mod,
             small_modulus=P.small_q, gsw_l=P.gsw_l, gsw_base_log2=P.base_log2,
             gsw_l_key=P.gsw_l_key, gsw_base_log2_key=P.base_log2_key)
    d.update(over)
    return _capi.OpirParams(**d)


def _create(L, prm):
    ctx = ctypes.c_void_p()
    rc = L.opir_ctx_create(ctypes.byref(prm), 0, ctypes.byref(ctx))
    return rc, ctx


def test_invalid_parameter_sets_are_rejected(gpu_lib):
    from onionpirv2_gb300 import _capi
    L = _capi.load()
    q = _params().coeff_modulus
    for bad in (dict(poly_degree=4096), dict(coeff_modulus=q + 2),      # not 2048 / not prime
                dict(coeff_modulus=(1 << 61) - 1), dict(gsw_l=0),          # q >= 2^60 / no digits
                dict(gsw_l=2, gsw_base_log2=12), dict(small_modulus=15)):  # gadget too short / not prime
        rc, ctx = _create(L, _params(**bad))
        assert rc == -1, bad
        assert not ctx.value
    rc, ctx = _create(L, _params())
    assert rc == 0
    L.opir_ctx_destroy(ctx)


def test_misuse_returns_codes_and_the_context_stays_usable(oracle_lib, gpu_lib):
    from onionpirv2_gb300 import PirParams, PirServer, _capi
    L = _capi.load()
    o = oracle_lib.Oracle(4096, 256)
    server = PirServer(PirParams(num_entries=4096, max_fst_dim=256))
    ctx = server.ctx
    bad_shape = _capi.OpirDbShape(fst_dim_sz=256, other_dim_sz=12, entry_size=3840,
                                  entries_per_pt=1, bits_per_coeff=15)  # n_rest not a power of two
    db = ctypes.c_uint32()
    assert L.opir_db_create(ctx, ctypes.byref(bad_shape), ctypes.byref(db)) == -1
    huge = _capi.OpirDbShape(fst_dim_sz=256, other_dim_sz=16, entry_size=8000,
                             entries_per_pt=1, bits_per_coeff=15)         # entry exceeds a plaintext
    assert L.opir_db_create(ctx, ctypes.byref(huge), ctypes.byref(db)) == -1
    query = np.zeros(2 * N, np.uint64)
    resp = np.zeros(2 * N, np.uint64)
    assert L.opir_make_query(ctx, 77, 0, _capi.p64(query), _capi.p64(resp), None) == -3
    server.gen_data(5)
    assert L.opir_make_query(ctx, server.db_id, 12345, _capi.p64(query), _capi.p64(resp),
                             None) == -2
    sk = o.keygen(1)
    gk, gswk = o.galois_keys(sk, 2), o.gsw_key(sk, 3)
    short = np.ascontiguousarray(gk[:5])  # 5 Galois levels; the database needs 9
    assert L.opir_set_galois_key(ctx, 1, _capi.p64(short.reshape(-1)), 5) == 0
    server.set_client_gsw_key(1, gswk)
    q1 = o.make_query(sk, 4, 100)
    assert L.opir_make_query(ctx, server.db_id, 1, _capi.p64(q1.reshape(-1)), _capi.p64(resp),
                             None) == -1
    assert "Galois levels" in L.opir_last_error(ctx).decode()
    assert L.opir_set_key_budget(ctx, 1 << 30) == -6   # clients are already registered
    assert L.opir_erase_client(ctx, 999) == -2
    done = ctypes.c_int()
    assert L.opir_poll(ctx, 1, None, None, ctypes.byref(done)) == -6  # never served
    # the context still answers correctly
    server.set_client_galois_key(1, gk)
    db_ref = o.build_db(5)
    ref, _, _, _ = o.make_query_server(db_ref, gk, o.gsw_key_to_ntt(gswk), q1)
    assert np.array_equal(server.make_query(1, q1), ref)
    server.close()


def test_scan_wait_timeout_is_reported_and_the_context_recovers(oracle_lib, gpu_lib):
    """The bounded-wait failure path of the pipelined scan (async.cuh): the
    producer of the scan's first CTA withholds one stage, its consumers give
    up after a few thousand polls, the query returns OPIR_ERR_TIMEOUT with
    the status bits, and the next query on the same context is bit-exact
    against the oracle again (directly launched and replayed from a CUDA
    graph alike)."""
    from onionpirv2_gb300 import PirParams, PirServer, _capi
    L = _capi.load()
    o = oracle_lib.Oracle(4096, 256)
    server = PirServer(PirParams(num_entries=4096, max_fst_dim=256))
    seed = 4321
    server.gen_data(seed)
    db = o.build_db(seed)
    sk = o.keygen(61)
    gk, gswk = o.galois_keys(sk, 62), o.gsw_key(sk, 63)
    server.set_client_galois_key(1, gk)
    server.set_client_gsw_key(1, gswk)
    gsw_ntt = o.gsw_key_to_ntt(gswk)
    queries = [o.make_query(sk, 70 + j, i) for j, i in enumerate((5, 3000, 4095))]
    want = [o.make_query_server(db, gk, gsw_ntt, q)[0] for q in queries]
    for graphs in (True, False):
        server.set_graphs(graphs)
        assert np.array_equal(server.make_query(1, queries[0]), want[0])
        _capi.check(server.ctx, L.opir_debug_withhold_scan_stage(server.ctx, 4096))
        with pytest.raises(_capi.OpirError) as e:
            server.make_query(1, queries[1])
        assert e.value.code == -8  # OPIR_ERR_TIMEOUT
        msg = L.opir_last_error(server.ctx).decode()
        assert "timed out" in msg and "0x" in msg
        st = int(msg.split("0x")[1].split(")")[0], 16)
        assert st & 1, "a consumer wait ran out (kErrWaitFull)"
        assert not st & 4, "the producer drained every copy it issued"
        _capi.check(server.ctx, L.opir_debug_withhold_scan_stage(server.ctx, 0))
        assert np.array_equal(server.make_query(1, queries[1]), want[1])
        assert np.array_equal(server.make_query(1, queries[2]), want[2])
        _capi.check(server.ctx, L.opir_sync(server.ctx))
    assert L.opir_debug_withhold_scan_stage(server.ctx, (1 << 20) + 1) == -1
    server.close()
