"""The multi-modulus GPU path (opir_ctx_create_rns) against the multi-modulus
oracle, bit for bit: N = 4096 with two ciphertext primes (the PolyDegree =
4096, CoeffMods = {60, 60, 60} presets, database_constants.h:13-172) at every
stage of make_query -- expansion with RNS key switching, RGSW reconstruction
with the CRT decomposition (gsw_eval.cpp:108-182), the first dimension, the
folds, the switch to q_0 (server.cpp:567-570) and to small_q, the 57-bit
packing -- and the same generic kernels at N = 2048 with one prime against
the single-modulus oracle.
"""
import ctypes
import io

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rns_oracle(oracle_lib, params):
    P = params
    return oracle_lib.RnsOracle(P.poly_degree, P.num_entries, P.max_fst_dim, l=P.gsw_l,
                                l_key=P.gsw_l_key, plain_bits=P.plain_mod_bits,
                                small_q_width=P.small_q_width, coeff_bits=tuple(P.coeff_mods))


@pytest.fixture(scope="module")
def rns1024(oracle_lib, gpu_lib):
    from onionpirv2_gb300 import PirParams, PirServer
    params = PirParams.preset("rns1024")
    o = _rns_oracle(oracle_lib, params)
    server = PirServer(params)
    seed = 555
    server.gen_data(seed)
    db = o.build_db(seed)
    yield o, params, server, db, seed
    server.close()


def test_parameters_match_the_oracle(rns1024):
    o, params, server, _, _ = rns1024
    P = o.P
    assert (P.n, P.rns, P.q, P.p, P.t, P.small_q) == (
        params.poly_degree, params.get_rns_mod_cnt(), tuple(params.get_coeff_modulus()),
        params.coeff_modulus[-1], params.plain_mod, params.small_q)
    assert (P.base_log2, P.base_log2_key, P.entry_size) == (
        params.base_log2, params.base_log2_key, params.get_entry_size())
    assert server.resp_bytes == o.response_bytes() == 2 * 4096 * 57 // 8


def test_ntt_matches_oracle_on_every_modulus(rns1024):
    o, _, server, _, _ = rns1024
    rng = np.random.default_rng(2)
    for mod in range(3):  # q_0, q_1, p
        q = np.uint64((list(o.P.q) + [o.P.p])[mod])
        a = rng.integers(0, 2**62, size=(5, 4096), dtype=np.uint64) % q
        f = server.ntt(a, mod=mod)
        assert np.array_equal(f, o.ntt_fwd(a, mod)), mod
        assert np.array_equal(server.ntt(f, mod=mod, inverse=True), a), mod


def test_every_stage_matches_oracle(rns1024):
    o, params, server, db, seed = rns1024
    sk = o.keygen(71)
    gk, gsw = o.galois_keys(sk, 72), o.gsw_key(sk, 73)
    gsn = o.gsw_to_ntt(gsw)
    server.set_client_galois_key(4, gk)
    server.set_client_gsw_key(4, gsw)
    P = o.P
    for idx in (0, 777, 1023):
        query = o.make_query(sk, 80 + idx, idx)
        tr = server.make_query_trace(4, query)
        leaves = o.expand(query, gk)
        assert np.array_equal(tr["leaves"], leaves), "expansion"
        for d in range(1, P.ndim):
            cts = leaves[P.n1 + (d - 1) * P.l: P.n1 + d * P.l]
            assert np.array_equal(tr["gsw"][d - 1], o.query_to_gsw(cts, gsn)), f"RGSW dim {d}"
        fd, wraps = o.first_dim(db, leaves[: P.n1])
        assert wraps == 0
        assert np.array_equal(tr["first_dim"], fd), "first dimension"
        resp, packed, _ = o.make_query_server(db, gk, gsn, query)
        assert np.array_equal(tr["resp"], resp) and np.array_equal(tr["packed"], packed)
        got = server.make_query(4, query)
        assert np.array_equal(got, resp) and got.packed == packed.tobytes()
        plain, budget = o.decrypt_small(sk, got)
        assert np.array_equal(o.entry_from_plain(idx, plain), o.gen_entries(seed, idx, 1)[0])
        assert budget > 0
        buf = io.BytesIO()
        assert server.save_resp_to_stream(np.array(got), buf) == len(packed)
        assert buf.getvalue() == packed.tobytes()


def test_uploaded_database_and_batches(rns1024, gpu_lib):
    from onionpirv2_gb300 import PirServer, _capi
    o, params, _, db, _ = rns1024
    server = PirServer(params)
    server.upload_ntt_db(db)
    sk = o.keygen(91)
    gk, gsw = o.galois_keys(sk, 92), o.gsw_key(sk, 93)
    server.set_client_galois_key(1, gk)
    server.set_client_gsw_key(1, gsw)
    gsn = o.gsw_to_ntt(gsw)
    queries = np.stack([o.make_query(sk, 100 + j, i) for j, i in enumerate((3, 512, 1000))])
    resps, packed = server.make_query_batch([1, 1, 1], queries)
    for j in range(3):
        r, p, _ = o.make_query_server(db, gk, gsn, queries[j])
        assert np.array_equal(resps[j], r) and np.array_equal(packed[j], p)
    # more queries than the path has lanes, two clients: every response the
    # single query's, the lanes reused in turn
    sk2 = o.keygen(191)
    server.set_client_galois_key(2, o.galois_keys(sk2, 192))
    server.set_client_gsw_key(2, o.gsw_key(sk2, 193))
    ids = [1 + (j % 2) for j in range(9)]
    qs = np.stack([o.make_query(sk if ids[j] == 1 else sk2, 300 + j, (j * 131) % 1024)
                   for j in range(9)])
    resps9, packed9 = server.make_query_batch(ids, qs)
    for j in range(9):
        single = server.make_query(ids[j], qs[j])
        assert np.array_equal(resps9[j], single), j
        assert packed9[j].tobytes() == single.packed, j
    # what a multi-modulus context does not offer fails loudly
    L = _capi.load()
    assert L.opir_autotune(server.ctx, server.db_id, 8, 1, None) == -6
    assert L.opir_set_batch_engine(server.ctx, 3, 0) == -6
    with pytest.raises(_capi.OpirError):
        server.serve_start()
    with pytest.raises(_capi.UnknownClientError):
        server.make_query(77, queries[0])
    server.close()


def test_larger_preset_shape(oracle_lib, gpu_lib):
    """The "2^14 * 24KB = 384MB" preset: 256 x 2^6 plaintexts, six folds."""
    from onionpirv2_gb300 import PirParams, PirServer
    params = PirParams.preset("rns16384")
    o = _rns_oracle(oracle_lib, params)
    assert (o.P.n1, o.P.n_rest, o.P.ndim) == (256, 64, 7)
    server = PirServer(params)
    server.gen_data(9)
    db = o.build_db(9)
    sk = o.keygen(3)
    gk, gsw = o.galois_keys(sk, 4), o.gsw_key(sk, 5)
    server.set_client_galois_key(2, gk)
    server.set_client_gsw_key(2, gsw)
    for idx in (0, 16383, 9999):
        query = o.make_query(sk, 6 + idx, idx)
        got = server.make_query(2, query)
        resp, packed, _ = o.make_query_server(db, gk, o.gsw_to_ntt(gsw), query)
        assert np.array_equal(got, resp) and got.packed == packed.tobytes(), idx
        plain, _ = o.decrypt_small(sk, got)
        assert np.array_equal(o.entry_from_plain(idx, plain), o.gen_entries(9, idx, 1)[0])
    server.close()


def test_generic_kernels_with_one_prime_match_the_single_modulus_oracle(oracle_lib, gpu_lib):
    """opir_ctx_create_rns with N = 2048 and one prime runs the same generic
    kernels; its responses must equal the single-modulus oracle's."""
    from onionpirv2_gb300 import PirParams, _capi
    L = _capi.load()
    P = PirParams(num_entries=4096, max_fst_dim=256)
    prm = _capi.OpirRnsParams(
        poly_degree=2048, rns_count=1, coeff_moduli=(ctypes.c_uint64 * 2)(P.coeff_modulus[0], 0),
        special_modulus=P.coeff_modulus[1], plain_modulus=P.plain_mod, small_modulus=P.small_q,
        gsw_l=P.gsw_l, gsw_base_log2=P.base_log2, gsw_l_key=P.gsw_l_key,
        gsw_base_log2_key=P.base_log2_key)
    ctx = ctypes.c_void_p()
    assert L.opir_ctx_create_rns(ctypes.byref(prm), 0, ctypes.byref(ctx)) == 0
    try:
        shape = _capi.OpirDbShape(fst_dim_sz=256, other_dim_sz=16, entry_size=P.get_entry_size(),
                                  entries_per_pt=1, bits_per_coeff=15)
        db_id = ctypes.c_uint32()
        _capi.check(ctx, L.opir_db_create(ctx, ctypes.byref(shape), ctypes.byref(db_id)))
        _capi.check(ctx, L.opir_db_fill_synthetic(ctx, db_id.value, 31))
        o = oracle_lib.Oracle(4096, 256)
        db = o.build_db(31)
        sk = o.keygen(41)
        gk, gsw = o.galois_keys(sk, 42), o.gsw_key(sk, 43)
        _capi.check(ctx, L.opir_set_galois_key(ctx, 8, _capi.p64(np.ascontiguousarray(gk).reshape(-1)),
                                               gk.shape[0]))
        _capi.check(ctx, L.opir_set_gsw_key(ctx, 8, _capi.p64(np.ascontiguousarray(gsw).reshape(-1))))
        for idx in (1, 2222):
            q = np.ascontiguousarray(o.make_query(sk, 50 + idx, idx), np.uint64).reshape(-1)
            resp = np.zeros(2 * 2048, np.uint64)
            packed = np.zeros(L.opir_response_bytes(ctx), np.uint8)
            _capi.check(ctx, L.opir_make_query(ctx, db_id.value, 8, _capi.p64(q), _capi.p64(resp),
                                               _capi.p8(packed)))
            want, wpacked, _, _ = o.make_query_server(db, gk, o.gsw_key_to_ntt(gsw), q)
            assert np.array_equal(resp, want.reshape(-1)) and np.array_equal(packed, wpacked)
    finally:
        L.opir_ctx_destroy(ctx)


def test_graph_replay_matches_direct_launches(oracle_lib, gpu_lib):
    """Synchronous queries are replayed as CUDA graphs keyed by client and
    workspace: two clients (two executables) alternating, each replayed,
    equal the oracle and the same queries launched directly."""
    from onionpirv2_gb300 import PirParams, PirServer
    params = PirParams.preset("rns1024")
    o = _rns_oracle(oracle_lib, params)
    server = PirServer(params)
    server.gen_data(31)
    db = o.build_db(31)
    keys = []
    for c in (1, 2):
        sk = o.keygen(40 + c)
        gk, gsw = o.galois_keys(sk, 50 + c), o.gsw_key(sk, 60 + c)
        server.set_client_galois_key(c, gk)
        server.set_client_gsw_key(c, gsw)
        keys.append((sk, gk, o.gsw_to_ntt(gsw)))
    asked = [(1 + j % 2, (97 * j + 5) % params.num_entries) for j in range(6)]
    queries = [o.make_query(keys[c - 1][0], 70 + j, i) for j, (c, i) in enumerate(asked)]
    replayed = [server.make_query(c, q) for (c, _), q in zip(asked, queries)]
    server.set_graphs(False)
    direct = [server.make_query(c, q) for (c, _), q in zip(asked, queries)]
    for j, ((c, i), q) in enumerate(zip(asked, queries)):
        _, gk, gsn = keys[c - 1]
        ref, packed, _ = o.make_query_server(db, gk, gsn, q)
        assert np.array_equal(replayed[j], ref) and replayed[j].packed == packed.tobytes(), j
        assert np.array_equal(direct[j], ref), j
    server.close()
