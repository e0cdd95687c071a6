"""Serving layer: continuous batching over resident databases and a key
budget with least-recently-used eviction.

Every response a query gets in the mix (other queries, other clients and
another database queued and running around it) must equal the response it
gets alone through opir_make_query -- which the parity tests pin to the
oracle -- and must decrypt to the requested entry.
"""
import random
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _clients(o, n, seed):
    out = []
    for j in range(n):
        sk = o.keygen(seed + 3 * j)
        out.append((sk, o.galois_keys(sk, seed + 3 * j + 1), o.gsw_key(sk, seed + 3 * j + 2)))
    return out


def test_results_same_alone_and_in_the_mix(oracle_lib, gpu_lib):
    from onionpirv2_gb300 import PirParams, PirServer
    oa = oracle_lib.Oracle(4096, 256)        # 256 x 16
    ob = oracle_lib.Oracle(1 << 13, 64)      # 64 x 128
    server = PirServer(PirParams(num_entries=4096, max_fst_dim=256))
    server.gen_data(71)
    db_a = server.db_id
    db_b = server.add_database(PirParams(num_entries=1 << 13, max_fst_dim=64), seed=72)
    keys = _clients(oa, 4, 300)  # Galois keys of height 9 serve both databases
    for cid, (sk, gk, gswk) in enumerate(keys):
        server.set_client_galois_key(cid, gk)
        server.set_client_gsw_key(cid, gswk)
    rng = random.Random(5)
    work = []
    for j in range(40):
        cid = rng.randrange(4)
        if rng.random() < 0.5:
            db, o = db_a, oa
        else:
            db, o = db_b, ob
        idx = rng.randrange(o.P.num_entries)
        work.append((cid, db, idx, o.make_query(keys[cid][0], 1000 + j, idx)))

    server.serve_start(max_batch=8, lanes=2, max_wait_us=500)
    # synchronous calls while serving go through the lanes as tickets
    during = server.make_query(work[0][0], work[0][3], db_id=work[0][1])
    during_batch, _ = server.make_query_batch([work[1][0], work[2][0]],
                                              np.stack([work[1][3], work[2][3]]))
    tickets = [None] * len(work)

    def submitter(part):
        r = random.Random(part)
        for j in range(part, len(work), 2):
            cid, db, _, q = work[j]
            tickets[j] = server.submit(cid, q, db_id=db)
            time.sleep(r.random() * 0.002)    # arrivals spread over the run

    threads = [threading.Thread(target=submitter, args=(p,)) for p in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    mixed = [server.wait(t, 60000) for t in tickets]
    stats = server.serve_stats()
    server.serve_stop()
    # the work and the three synchronous queries
    assert stats["completed"] == len(work) + 3 and stats["failed"] == 0
    assert stats["batches"] >= 2 and stats["mean_batch"] >= 1.0
    assert 0 < stats["p50_ms"] <= stats["p99_ms"] <= stats["max_ms"]
    assert stats["queries_per_s"] > 0

    # alone: one synchronous make_query per query on its own database
    from onionpirv2_gb300.server import synthetic_entries
    pb = PirParams(num_entries=1 << 13, max_fst_dim=64)
    for j, (cid, db, idx, q) in enumerate(work):
        alone = server.make_query(cid, q, db_id=db)
        assert np.array_equal(mixed[j], alone), j
        assert mixed[j].packed == alone.packed
        if j == 0:
            assert np.array_equal(during, alone) and during.packed == alone.packed
        o = oa if db == db_a else ob
        plain, _ = o.decrypt(keys[cid][0], mixed[j], 2)
        want = (server.direct_get_entry(idx) if db == db_a else
                synthetic_entries(72, idx, 1, pb.get_entry_size())[0])
        assert np.array_equal(o.entry_from_plain(idx, plain), want), j
    for i, j in enumerate((1, 2)):                # the batch ran on the default database
        assert np.array_equal(during_batch[i], server.make_query(work[j][0], work[j][3]))
    server.close()


def test_key_budget_evicts_least_recently_used(oracle_lib, gpu_lib):
    from onionpirv2_gb300 import PirParams, PirServer
    o = oracle_lib.Oracle(4096, 256)
    server = PirServer(PirParams(num_entries=4096, max_fst_dim=256))
    server.gen_data(9)
    per = server.key_bytes_per_client()
    assert per > 0
    server.set_key_budget(2 * per)              # two clients' keys in device memory
    keys = _clients(o, 5, 700)
    for cid, (sk, gk, gswk) in enumerate(keys):
        server.set_client_galois_key(cid, gk)
        server.set_client_gsw_key(cid, gswk)
    assert server.resident_clients() == (0, 2)
    db = o.build_db(9)
    # synchronous path: every query re-admits its client's keys
    for j, cid in enumerate([0, 1, 2, 0, 3, 4, 1]):
        idx = (j * 577 + 3) % 4096
        q = o.make_query(keys[cid][0], 50 + j, idx)
        resp = server.make_query(cid, q)
        sk, gk, gswk = keys[cid]
        ref, _, _, _ = o.make_query_server(db, gk, o.gsw_key_to_ntt(gswk), q)
        assert np.array_equal(resp, ref), (j, cid)
        assert server.resident_clients()[0] <= 2
    # serving: batches of at most two distinct clients (= slots), clients
    # rotating through the five, each batch re-admitting evicted keys
    server.serve_start(max_batch=2, lanes=1, max_wait_us=0)
    tickets, refs = [], []
    for j in range(10):
        cid = j % 5
        idx = (j * 911 + 1) % 4096
        q = o.make_query(keys[cid][0], 90 + j, idx)
        tickets.append(server.submit(cid, q))
        sk, gk, gswk = keys[cid]
        refs.append(o.make_query_server(db, gk, o.gsw_key_to_ntt(gswk), q)[0])
    for t, ref in zip(tickets, refs):
        assert np.array_equal(server.wait(t, 60000), ref)
    server.serve_stop()
    assert server.resident_clients()[0] <= 2
    server.close()


def test_serving_errors(oracle_lib, gpu_lib):
    from onionpirv2_gb300 import PirParams, PirServer, _capi
    o = oracle_lib.Oracle(4096, 256)
    server = PirServer(PirParams(num_entries=4096, max_fst_dim=256))
    server.gen_data(1)
    sk, gk, gswk = _clients(o, 1, 11)[0]
    server.set_client_galois_key(0, gk)
    server.set_client_gsw_key(0, gswk)
    q = o.make_query(sk, 3, 17)
    with pytest.raises(_capi.OpirError):        # not serving yet
        server.submit(0, q)
    server.serve_start(max_batch=4, lanes=2, max_wait_us=100)
    with pytest.raises(_capi.UnknownClientError):
        server.submit(42, q)
    with pytest.raises(_capi.OpirError):        # unknown database
        server.submit(0, q, db_id=999)
    with pytest.raises(_capi.OpirError):        # database changes wait for serving to stop
        server.gen_data(2)
    t = server.submit(0, q)
    resp = server.wait(t, 60000)
    with pytest.raises(_capi.OpirError):        # a ticket is released once its result is taken
        server.poll(t)
    server.serve_stop()
    server.serve_stop()                          # idempotent
    alone = server.make_query(0, q)
    assert np.array_equal(resp, alone)
    server.close()
