"""The product client and the GPU server together, as a user runs them: the
PirClient (CPU library) makes keys and queries from OS entropy, the GPU
PirServer answers singly, in batches on every first-dimension engine and
through the serving loop, and every response decodes to the database entry."""
import io

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(4096, 256), (1 << 13, 64)])
def test_client_server_round_trip(gpu_lib, shape):
    from onionpirv2_gb300 import PirClient, PirParams, PirServer
    params = PirParams(num_entries=shape[0], max_fst_dim=shape[1])
    server = PirServer(params)
    server.gen_data(31337)
    clients = [PirClient(params, cid) for cid in range(6)]
    for c in clients:
        server.set_client_galois_key(c.get_client_id(), c.create_galois_keys())
        server.set_client_gsw_key(c.get_client_id(), c.generate_gsw_from_key())
    rng = np.random.default_rng(shape[1])
    entries = [int(x) for x in rng.integers(0, params.get_num_entries(), size=len(clients))]
    entries[0], entries[-1] = 0, params.get_num_entries() - 1
    queries = np.stack([c.fast_generate_query(e) for c, e in zip(clients, entries)])
    for c, e, q in zip(clients, entries, queries):
        resp = server.make_query(c.get_client_id(), q)
        stream = io.BytesIO()
        server.save_resp_to_stream(resp, stream)
        stream.seek(0)
        ct = c.load_resp_from_stream(stream)
        assert np.array_equal(ct, resp)
        plain, budget = c.decrypt_mod_q(ct)
        assert np.array_equal(c.get_entry_from_plaintext(e, plain), server.direct_get_entry(e))
        assert budget > 0
    ids = [c.get_client_id() for c in clients]
    for engine in ("scan", "imad", "tensor"):
        server.set_batch_engine(engine)
        resps, packed = server.make_query_batch(ids, queries)
        for j, (c, e) in enumerate(zip(clients, entries)):
            entry, _ = c.decode_response(e, packed[j].tobytes())
            assert np.array_equal(entry, server.direct_get_entry(e)), (engine, j)
    server.set_batch_engine("auto")
    server.close()


def test_served_responses_decode_for_many_clients(gpu_lib):
    """64 clients under a key budget of 16 (LRU admission) through the serving
    loop: every response decodes to its entry."""
    from onionpirv2_gb300 import PirClient, PirParams, PirServer
    params = PirParams(num_entries=1 << 13, max_fst_dim=64)
    server = PirServer(params)
    server.gen_data(4242)
    server.set_key_budget(16 * server.key_bytes_per_client())
    clients = [PirClient(params, 500 + i, secret_seed=i) for i in range(64)]
    for c in clients:
        server.set_client_galois_key(c.get_client_id(), c.create_galois_keys(seed=1))
        server.set_client_gsw_key(c.get_client_id(), c.generate_gsw_from_key(seed=2))
    rng = np.random.default_rng(9)
    picks = rng.integers(0, len(clients), size=160)
    entries = rng.integers(0, params.get_num_entries(), size=160)
    server.serve_start(max_batch=16, lanes=2, max_wait_us=500)
    tickets = [server.submit(clients[k].get_client_id(),
                             clients[k].fast_generate_query(int(e), seed=j))
               for j, (k, e) in enumerate(zip(picks, entries))]
    resps = [server.wait(t, 120000) for t in tickets]
    stats = server.serve_stats()
    server.serve_stop()
    assert stats["failed"] == 0 and stats["completed"] == 160
    for k, e, r in zip(picks, entries, resps):
        entry, budget = clients[k].decode_response(int(e), r.packed)
        assert np.array_equal(entry, server.direct_get_entry(int(e)))
    server.close()
