"""GPU path vs the CPU oracle: every stage of make_query, bit for bit.

The oracle restates the reference server (src/server.cpp) and client
(src/client.cpp); all comparisons are exact (integer arithmetic, tolerance 0).
"""
import io

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048


@pytest.fixture(scope="module")
def setup_db4096(oracle_lib, gpu_lib):
    from onionpirv2_gb300 import PirParams, PirServer
    o = oracle_lib.Oracle(4096, 256)
    params = PirParams(num_entries=4096, max_fst_dim=256)
    server = PirServer(params)
    seed = 12345
    server.gen_data(seed)
    db = o.build_db(seed)
    return o, params, server, db, seed


def make_client(o, seed):
    sk = o.keygen(seed)
    gk = o.galois_keys(sk, seed + 1)
    gswk = o.gsw_key(sk, seed + 2)
    return sk, gk, gswk


def test_ntt_matches_oracle(setup_db4096):
    o, params, server, _, _ = setup_db4096
    rng = np.random.default_rng(1)
    for mod, q in ((0, o.P.q), (1, o.P.p)):
        a = (rng.integers(0, 2**63, size=(7, N), dtype=np.uint64) % np.uint64(q))
        fwd = server.ntt(a, mod=mod)
        assert np.array_equal(fwd, o.ntt_fwd(a, mod))
        back = server.ntt(fwd, mod=mod, inverse=True)
        assert np.array_equal(back, a)


def test_query_stages_match_oracle(setup_db4096):
    o, params, server, db, seed = setup_db4096
    P = o.P
    sk, gk, gswk = make_client(o, 77)
    cid = 9001
    server.set_client_galois_key(cid, gk)
    server.set_client_gsw_key(cid, gswk)
    idx = 2741
    query = o.make_query(sk, 4242, idx)
    tr = server.make_query_trace(cid, query)
    # expansion (fast_expand_qry)
    leaves = o.expand(query, gk)
    assert np.array_equal(tr["leaves"], leaves)
    # RGSW reconstruction (query_to_gsw)
    gsw_ntt = o.gsw_key_to_ntt(gswk)
    for i in range(1, P.ndim):
        s = P.n1 + (i - 1) * P.l
        rg = o.query_to_gsw(leaves[s:s + P.l], gsw_ntt)
        assert np.array_equal(tr["gsw"][i - 1], rg), f"dim {i}"
    # first dimension
    fd, wraps = o.first_dim(db, leaves[:P.n1])
    assert wraps == 0
    assert np.array_equal(tr["first_dim"], fd)
    # whole response, packed bytes
    resp, packed, _, _ = o.make_query_server(db, gk, gsw_ntt, query)
    assert np.array_equal(tr["resp"], resp)
    assert np.array_equal(tr["packed"], packed)


@pytest.mark.parametrize("idx", [0, 1, 255, 256, 4095, 1777])
def test_end_to_end_decrypts_entry(setup_db4096, idx):
    """tests.cpp:110-134: the decrypted entry equals the database entry."""
    o, params, server, db, seed = setup_db4096
    sk, gk, gswk = make_client(o, 1000 + idx)
    cid = 50 + idx
    server.set_client_galois_key(cid, gk)
    server.set_client_gsw_key(cid, gswk)
    query = o.make_query(sk, 99 + idx, idx)
    resp = server.make_query(cid, query)
    buf = io.BytesIO()
    n = server.save_resp_to_stream(resp, buf)
    assert n == o.response_bytes() == 13824
    ct = o.unpack_response(np.frombuffer(buf.getvalue(), np.uint8))
    plain, budget = o.decrypt(sk, ct, 2)
    entry = o.entry_from_plain(idx, plain)
    assert np.array_equal(entry, server.direct_get_entry(idx))
    assert budget > 0
    gsw_ntt = o.gsw_key_to_ntt(gswk)
    ref, ref_packed, _, _ = o.make_query_server(db, gk, gsw_ntt, query)
    assert np.array_equal(resp, ref)
    assert resp.packed == ref_packed.tobytes()


def test_batch_equals_single(setup_db4096):
    o, params, server, db, seed = setup_db4096
    ids, queries, singles = [], [], []
    for j in range(5):
        sk, gk, gswk = make_client(o, 3000 + j)
        cid = 7000 + j
        server.set_client_galois_key(cid, gk)
        server.set_client_gsw_key(cid, gswk)
        q = o.make_query(sk, 555 + j, (j * 977) % 4096)
        ids.append(cid)
        queries.append(q)
        singles.append(server.make_query(cid, q))
    resp, packed = server.make_query_batch(ids, np.stack(queries))
    for j in range(5):
        assert np.array_equal(resp[j], singles[j])
        assert packed[j].tobytes() == singles[j].packed


def test_unknown_client_raises(setup_db4096):
    from onionpirv2_gb300 import UnknownClientError
    o, params, server, db, seed = setup_db4096
    with pytest.raises(UnknownClientError):
        server.make_query(123456789, np.zeros((2, N), np.uint64))


def test_push_chunk_matches_reference_layout(oracle_lib, gpu_lib):
    """push_database_chunk path (host entries) == oracle packing + NTT."""
    from onionpirv2_gb300 import PirParams, PirServer
    o = oracle_lib.Oracle(4096, 256)
    params = PirParams(num_entries=4096, max_fst_dim=256)
    server = PirServer(params)
    P = o.P
    rng = np.random.default_rng(5)
    entries = rng.integers(0, 256, size=(P.num_pt, P.entry_size), dtype=np.uint8)
    for row in range(P.n_rest):
        server.push_database_chunk(entries[row * P.n1:(row + 1) * P.n1], row)
    coeffs = o.pack_plaintexts(entries, P.num_pt)
    ntt = o.plain_to_ntt(coeffs)
    db = np.ascontiguousarray(ntt.T)  # db_aligned[c][pt]
    sk, gk, gswk = make_client(o, 31)
    server.set_client_galois_key(1, gk)
    server.set_client_gsw_key(1, gswk)
    for idx in (3, 2222):
        query = o.make_query(sk, idx, idx)
        resp = server.make_query(1, query)
        ref, _, _, _ = o.make_query_server(db, gk, o.gsw_key_to_ntt(gswk), query)
        assert np.array_equal(resp, ref)
        plain, _ = o.decrypt(sk, resp, 2)
        assert np.array_equal(o.entry_from_plain(idx, plain), entries[idx])
    # direct_get_entry decodes the pushed bytes back from the device database
    for idx in (0, 1, 2222, P.num_entries - 1):
        assert np.array_equal(server.direct_get_entry(idx), entries[idx])
    # the aligned-upload path gives the same database
    server.upload_ntt_db(db)
    query = o.make_query(sk, 8, 1234)
    resp = server.make_query(1, query)
    ref, _, _, _ = o.make_query_server(db, gk, o.gsw_key_to_ntt(gswk), query)
    assert np.array_equal(resp, ref)
    assert np.array_equal(server.direct_get_entry(1234), entries[1234])


@pytest.mark.parametrize("shape", [(4096, 256), (1 << 14, 1024), (100, 16)])
def test_direct_get_entry_decodes_device_database(gpu_lib, shape):
    """direct_get_entry (server.cpp:503-517) reads an entry back from the
    device database: equal to the seeded generator's entries, for entry
    sizes that fill a plaintext and for several entries per plaintext."""
    from onionpirv2_gb300 import OpirError, PirParams, PirServer, synthetic_entries
    for entry_size in (0, 100):
        params = PirParams(num_entries=shape[0], max_fst_dim=shape[1], entry_size_cfg=entry_size)
        server = PirServer(params)
        server.gen_data(4321)
        n = params.get_num_entries()
        rng = np.random.default_rng(n)
        for idx in [0, 1, n - 1] + [int(x) for x in rng.integers(0, n, size=5)]:
            want = synthetic_entries(4321, idx, 1, params.get_entry_size())[0]
            assert np.array_equal(server.direct_get_entry(idx), want), (entry_size, idx)
        with pytest.raises(OpirError):
            server.direct_get_entry(n)
        server.close()


SHAPES = [
    # (num_entries, max_fst_dim): n1 x n_rest
    (4096, 256),   # 256 x 16   (32 planes per scan tile)
    (8192, 8),     # 8 x 1024   (row tiles of 512 rows)
    (512, 256),    # 256 x 2    (query runs exceed shared memory: generic kernel)
    (1024, 1024),  # 1024 x 1   (single dimension, no folding)
]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("cfg", [0, 1, 2, 3, 4, 5, 6, 7, 8])
def test_scan_configs_and_shapes(oracle_lib, gpu_lib, monkeypatch, shape, cfg):
    """Every compiled scan pipeline configuration and every tile geometry
    gives the oracle's first-dimension result and response."""
    if cfg and shape != (4096, 256) and shape != (8192, 8):
        pytest.skip("configurations are swept on the two bulk-copy geometries")
    from onionpirv2_gb300 import PirParams, PirServer
    monkeypatch.setenv("OPIR_SCAN_CFG", str(cfg))
    o = oracle_lib.Oracle(*shape)
    P = o.P
    server = PirServer(PirParams(num_entries=shape[0], max_fst_dim=shape[1]))
    server.gen_data(31)
    db = o.build_db(31)
    sk, gk, gswk = make_client(o, 5)
    server.set_client_galois_key(1, gk)
    server.set_client_gsw_key(1, gswk)
    idx = (P.num_entries * 2) // 3
    query = o.make_query(sk, 17, idx)
    tr = server.make_query_trace(1, query)
    leaves = o.expand(query, gk)
    fd, _ = o.first_dim(db, leaves[:P.n1])
    assert np.array_equal(tr["first_dim"], fd)
    resp, packed, _, _ = o.make_query_server(db, gk, o.gsw_key_to_ntt(gswk), query)
    assert np.array_equal(tr["resp"], resp)
    plain, _ = o.decrypt(sk, tr["resp"], 2)
    assert np.array_equal(o.entry_from_plain(idx, plain), server.direct_get_entry(idx))
    server.close()


@pytest.mark.parametrize("threshold,pair,wide", [(0, 0, 0), (1 << 30, 0, 0), (0, 1 << 30, 0),
                                                 (0, 0, 1 << 30)])
def test_one_cta_and_cluster_tree_forms(oracle_lib, gpu_lib, monkeypatch, threshold, pair, wide):
    """Expansion, RGSW reconstruction and folding give the oracle's results
    in every kernel form (one CTA per ciphertext, a cluster of CTAs, for
    expansion and folding a pair of CTAs per node / ciphertext pair, and for
    folding the ten-CTA cluster)."""
    from onionpirv2_gb300 import PirParams, PirServer
    monkeypatch.setenv("OPIR_CLUSTER_THRESHOLD", str(threshold))
    monkeypatch.setenv("OPIR_PAIR_THRESHOLD", str(pair))
    monkeypatch.setenv("OPIR_EXPAND_PAIR_THRESHOLD", str(pair))
    monkeypatch.setenv("OPIR_WIDE_THRESHOLD", str(wide))
    o = oracle_lib.Oracle(4096, 256)
    P = o.P
    server = PirServer(PirParams(num_entries=4096, max_fst_dim=256))
    server.gen_data(8)
    db = o.build_db(8)
    ids, queries, refs = [], [], []
    for j in range(3):
        sk, gk, gswk = make_client(o, 40 + j)
        server.set_client_galois_key(j, gk)
        server.set_client_gsw_key(j, gswk)
        qry = o.make_query(sk, 60 + j, 1000 * j + 7)
        ids.append(j)
        queries.append(qry)
        refs.append(o.make_query_server(db, gk, o.gsw_key_to_ntt(gswk), qry)[0])
        tr = server.make_query_trace(j, qry)
        leaves = o.expand(qry, gk)
        assert np.array_equal(tr["leaves"], leaves)
        gsw_ntt = o.gsw_key_to_ntt(gswk)
        for i in range(1, P.ndim):
            s = P.n1 + (i - 1) * P.l
            assert np.array_equal(tr["gsw"][i - 1], o.query_to_gsw(leaves[s:s + P.l], gsw_ntt))
        assert np.array_equal(tr["resp"], refs[-1])
    resp, _ = server.make_query_batch(ids, np.stack(queries))
    for j in range(3):
        assert np.array_equal(resp[j], refs[j])
    server.close()


@pytest.mark.parametrize("pdl", ["63", "0"])
def test_programmatic_launches_match_oracle(oracle_lib, gpu_lib, monkeypatch, pdl):
    """With and without programmatic dependent launches (each kernel stages
    its constant tables while the previous one runs): single queries from a
    replayed graph and from direct launches, and a batch, equal the oracle."""
    from onionpirv2_gb300 import PirParams, PirServer
    monkeypatch.setenv("OPIR_PDL", pdl)
    monkeypatch.setenv("OPIR_PDL_GRAPH", pdl)
    o = oracle_lib.Oracle(4096, 256)
    server = PirServer(PirParams(num_entries=4096, max_fst_dim=256))
    server.gen_data(21)
    db = o.build_db(21)
    ids, queries, refs = [], [], []
    for j in range(4):
        sk, gk, gswk = make_client(o, 70 + 3 * j)
        server.set_client_galois_key(j, gk)
        server.set_client_gsw_key(j, gswk)
        qry = o.make_query(sk, 90 + j, 977 * j + 13)
        ids.append(j)
        queries.append(qry)
        refs.append(o.make_query_server(db, gk, o.gsw_key_to_ntt(gswk), qry))
    for graphs in (True, False):
        server.set_graphs(graphs)
        for rep in range(2):  # the second pass replays the captured graphs
            for j in range(4):
                r = server.make_query(j, queries[j])
                assert np.array_equal(np.asarray(r), refs[j][0]), (graphs, rep, j)
                assert bytes(r.packed) == bytes(refs[j][1]), (graphs, rep, j)
    resp, _ = server.make_query_batch(ids, np.stack(queries))
    for j in range(4):
        assert np.array_equal(resp[j], refs[j][0])
    server.close()


@pytest.mark.parametrize("engine", ["tensor", "imad"])
@pytest.mark.parametrize("batch", [3, 33])
def test_batched_scan_matches_single_and_oracle(oracle_lib, gpu_lib, monkeypatch, batch, engine):
    """Batched GEMM (one pass over the database for up to 32 queries) equals
    the per-query scan and the oracle, also for a partial second group, on
    both engines (bf16-limb tensor cores, integer multiply-adds)."""
    from onionpirv2_gb300 import PirParams, PirServer
    monkeypatch.setenv("OPIR_TC", "1" if engine == "tensor" else "0")
    o = oracle_lib.Oracle(1 << 13, 64)  # 64 x 128
    P = o.P
    assert (P.n1, P.n_rest) == (64, 128)
    server = PirServer(PirParams(num_entries=1 << 13, max_fst_dim=64))
    server.gen_data(77)
    db = o.build_db(77)
    ids, queries, keys, idxs = [], [], [], []
    for j in range(batch):
        sk, gk, gswk = make_client(o, 500 + 3 * j)
        cid = 100 + (j % 7)  # clients repeat inside the batch
        if j < 7:
            server.set_client_galois_key(cid, gk)
            server.set_client_gsw_key(cid, gswk)
            keys.append((sk, gk, gswk))
        sk, gk, gswk = keys[j % 7]
        idx = (j * 2311 + 5) % P.num_entries
        ids.append(cid)
        idxs.append(idx)
        queries.append(o.make_query(sk, 900 + j, idx))
    resp, packed = server.make_query_batch(ids, np.stack(queries))
    for j in (0, 1, batch - 1):
        sk, gk, gswk = keys[j % 7]
        ref, ref_packed, _, _ = o.make_query_server(db, gk, o.gsw_key_to_ntt(gswk), queries[j])
        assert np.array_equal(resp[j], ref), j
        assert packed[j].tobytes() == ref_packed.tobytes()
    for j in range(batch):
        plain, _ = o.decrypt(keys[j % 7][0], resp[j], 2)
        assert np.array_equal(o.entry_from_plain(idxs[j], plain), server.direct_get_entry(idxs[j]))
    # the same batch through the per-query scan
    monkeypatch.setenv("OPIR_BATCH_SCAN", "0")
    server2 = PirServer(PirParams(num_entries=1 << 13, max_fst_dim=64))
    server2.gen_data(77)
    for j in range(len(keys)):
        server2.set_client_galois_key(100 + j, keys[j][1])
        server2.set_client_gsw_key(100 + j, keys[j][2])
    resp2, _ = server2.make_query_batch(ids, np.stack(queries))
    assert np.array_equal(resp, resp2)
    server.close()
    server2.close()


@pytest.mark.parametrize("shape,batch", [
    ((4096, 256), 2),       # 256 x 16: one row tile per slot
    ((4096, 256), 20),      # 40 query polynomials: a 256 + 64 column split
    ((1 << 15, 512), 5),    # 512 x 64
    ((1 << 15, 512), 32),   # 64 query polynomials: two column blocks
    ((1 << 14, 1024), 6),   # 1024 x 16: two k segments of 512 summed in the epilogue
    ((1 << 14, 1024), 40),  # the same for 40 queries: one pass of three column blocks
    ((1536, 128), 4),       # 96 x 16: 32-k pipeline stages (96 is not a multiple of 64)
    ((8704, 1024), 3),      # 544 x 16: k segments of 512 and 32, 32-k pipeline stages
    ((1 << 15, 1024), 33),  # 1024 x 32: one row-tile pair, two k segments, 66 polynomials
    ((3072, 128), 5),       # 96 x 32: a pair with 32-k pipeline stages
    ((17408, 1024), 3),     # 544 x 32: a pair over k segments of 512 and 32
])
@pytest.mark.parametrize("limbs", ["8", "9"])
@pytest.mark.parametrize("form", ["one_cta", "cta_pair"])
def test_tensor_core_first_dim_matches_single_queries(oracle_lib, gpu_lib, monkeypatch, shape,
                                                      batch, limbs, form):
    """The tensor-core batched product gives every query the response of the
    per-query scan (which the oracle pins) for several shapes and batch
    sizes, with 8-bit and 9-bit query limbs, one CTA per tile or CTA pairs
    sharing M = 256 MMAs (where the rows form pairs of 16-row tiles), and
    the oracle's response for the first and last query."""
    from onionpirv2_gb300 import PirParams, PirServer
    monkeypatch.setenv("OPIR_TC", "1")
    monkeypatch.setenv("OPIR_TC_LIMBS", "0" if limbs == "8" else "1")
    monkeypatch.setenv("OPIR_TC_PAIR", "0" if form == "one_cta" else "1")
    o = oracle_lib.Oracle(*shape)
    P = o.P
    server = PirServer(PirParams(num_entries=shape[0], max_fst_dim=shape[1]))
    server.gen_data(123)
    keys = [make_client(o, 900 + j) for j in range(3)]
    for j, (sk, gk, gswk) in enumerate(keys):
        server.set_client_galois_key(j, gk)
        server.set_client_gsw_key(j, gswk)
    ids = [j % 3 for j in range(batch)]
    idxs = [(j * 7919 + 11) % P.num_entries for j in range(batch)]
    queries = [o.make_query(keys[ids[j]][0], 40 + j, idxs[j]) for j in range(batch)]
    resp, packed = server.make_query_batch(ids, np.stack(queries))
    for j in range(batch):
        single = server.make_query(ids[j], queries[j])
        assert np.array_equal(resp[j], single), j
        assert packed[j].tobytes() == single.packed
    db = o.build_db(123)
    for j in (0, batch - 1):
        sk, gk, gswk = keys[ids[j]]
        ref, _, _, _ = o.make_query_server(db, gk, o.gsw_key_to_ntt(gswk), queries[j])
        assert np.array_equal(resp[j], ref), j
        plain, _ = o.decrypt(sk, resp[j], 2)
        assert np.array_equal(o.entry_from_plain(idxs[j], plain), server.direct_get_entry(idxs[j]))
    server.close()


@pytest.mark.parametrize("per_pass", ["16", "32", "48", "64"])
def test_tensor_pass_sizes_give_the_same_responses(oracle_lib, gpu_lib, monkeypatch, per_pass):
    """A batch split into tensor-core launches of 16, 32, 48 or 64 queries
    (OPIR_TC_PASS) answers every query as the per-query scan does: 70
    queries make several passes and a ragged last one, over two k segments."""
    from onionpirv2_gb300 import PirParams, PirServer
    monkeypatch.setenv("OPIR_TC", "1")
    monkeypatch.setenv("OPIR_TC_PASS", per_pass)
    shape, batch = (1 << 14, 1024), 70
    o = oracle_lib.Oracle(*shape)
    P = o.P
    server = PirServer(PirParams(num_entries=shape[0], max_fst_dim=shape[1]))
    server.gen_data(77)
    keys = [make_client(o, 300 + j) for j in range(2)]
    for j, (sk, gk, gswk) in enumerate(keys):
        server.set_client_galois_key(j, gk)
        server.set_client_gsw_key(j, gswk)
    ids = [j % 2 for j in range(batch)]
    idxs = [(j * 104729 + 5) % P.num_entries for j in range(batch)]
    queries = [o.make_query(keys[ids[j]][0], 70 + j, idxs[j]) for j in range(batch)]
    resp, packed = server.make_query_batch(ids, np.stack(queries))
    for j in range(batch):
        single = server.make_query(ids[j], queries[j])
        assert np.array_equal(resp[j], single), (per_pass, j)
        assert packed[j].tobytes() == single.packed
    server.close()


@pytest.mark.parametrize("copies", ["0", "1"])
def test_host_staging_matches_oracle(oracle_lib, gpu_lib, monkeypatch, copies):
    """Host-buffer calls, with the kernels reading queries from and writing
    responses to mapped pinned memory (default) or through device buffers
    and copies: single queries (graph replay and direct launches), a batch
    and a trace equal the oracle."""
    from onionpirv2_gb300 import PirParams, PirServer
    monkeypatch.setenv("OPIR_HOST_COPIES", copies)
    o = oracle_lib.Oracle(4096, 256)
    server = PirServer(PirParams(num_entries=4096, max_fst_dim=256))
    server.gen_data(33)
    db = o.build_db(33)
    ids, queries, refs = [], [], []
    for j in range(3):
        sk, gk, gswk = make_client(o, 200 + 3 * j)
        server.set_client_galois_key(j, gk)
        server.set_client_gsw_key(j, gswk)
        qry = o.make_query(sk, 40 + j, 1311 * j + 5)
        ids.append(j)
        queries.append(qry)
        refs.append(o.make_query_server(db, gk, o.gsw_key_to_ntt(gswk), qry))
    for graphs in (True, False):
        server.set_graphs(graphs)
        for j in range(3):
            r = server.make_query(j, queries[j])
            assert np.array_equal(np.asarray(r), refs[j][0]), (graphs, j)
            assert r.packed == refs[j][1].tobytes(), (graphs, j)
    resp, packed = server.make_query_batch(ids, np.stack(queries))
    for j in range(3):
        assert np.array_equal(resp[j], refs[j][0])
        assert np.array_equal(packed[j], refs[j][1])
    tr = server.make_query_trace(0, queries[0])
    assert np.array_equal(tr["resp"], refs[0][0])
    assert np.array_equal(tr["packed"], refs[0][1])
    server.close()


@pytest.mark.parametrize("pdl", ["63", "0"])
def test_batch_over_key_chunk_matches_oracle(oracle_lib, gpu_lib, monkeypatch, pdl):
    """70 queries in one batch: the tree kernels take client keys in chunks
    of 64 queries, so the batch launches each level twice (programmatic
    launches on and off); every response equals the oracle's."""
    from onionpirv2_gb300 import PirParams, PirServer
    monkeypatch.setenv("OPIR_PDL", pdl)
    o = oracle_lib.Oracle(4096, 256)
    server = PirServer(PirParams(num_entries=4096, max_fst_dim=256))
    server.gen_data(5)
    db = o.build_db(5)
    clients = [make_client(o, 800 + 3 * j) for j in range(5)]
    for j, (sk, gk, gswk) in enumerate(clients):
        server.set_client_galois_key(j, gk)
        server.set_client_gsw_key(j, gswk)
    B = 70
    ids = [(7 * b) % 5 for b in range(B)]
    idxs = [(b * 601 + 11) % 4096 for b in range(B)]
    queries = np.stack([o.make_query(clients[ids[b]][0], 300 + b, idxs[b]) for b in range(B)])
    resp, packed = server.make_query_batch(ids, queries)
    gsw_ntt = [o.gsw_key_to_ntt(c[2]) for c in clients]
    for b in list(range(0, B, 9)) + [63, 64, 65, B - 1]:
        ref, ref_packed, _, _ = o.make_query_server(db, clients[ids[b]][1], gsw_ntt[ids[b]],
                                                    queries[b])
        assert np.array_equal(resp[b], ref), b
        assert np.array_equal(packed[b], ref_packed), b
    for b in range(B):
        plain, _ = o.decrypt(clients[ids[b]][0], resp[b], 2)
        assert np.array_equal(o.entry_from_plain(idxs[b], plain), server.direct_get_entry(idxs[b]))
    server.close()


def test_graph_replay_matches_direct_launches(oracle_lib, gpu_lib):
    """Single queries replayed from the captured CUDA graph (updated for
    every query: other clients, other queries) equal direct launches and the
    oracle, on two databases of different shapes."""
    from onionpirv2_gb300 import PirParams, PirServer
    for shape in ((4096, 256), (1 << 13, 64)):
        o = oracle_lib.Oracle(*shape)
        server = PirServer(PirParams(num_entries=shape[0], max_fst_dim=shape[1]))
        server.gen_data(21)
        db = o.build_db(21)
        clients = [make_client(o, 70 + j) for j in range(3)]
        for j, (sk, gk, gswk) in enumerate(clients):
            server.set_client_galois_key(j, gk)
            server.set_client_gsw_key(j, gswk)
        for it in range(6):
            j = it % 3
            sk, gk, gswk = clients[j]
            qry = o.make_query(sk, 90 + it, (it * 1237) % o.P.num_entries)
            server.set_graphs(True)
            g = server.make_query(j, qry)
            server.set_graphs(False)
            d = server.make_query(j, qry)
            assert np.array_equal(g, d) and g.packed == d.packed
            if it < 2:
                ref = o.make_query_server(db, gk, o.gsw_key_to_ntt(gswk), qry)[0]
                assert np.array_equal(g, ref)
        server.close()
