"""The CUDA path reproduces the committed golden fixtures (tests/golden/):
every intermediate of a single query, and the responses of the recorded
queries answered as one batch on each first-dimension engine."""
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).astype("<u8").tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["db4096", "db8192_n64", "db16384_n1024"])
def test_gpu_reproduces_golden(oracle_lib, gpu_lib, name):
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden as mg
    from onionpirv2_gb300 import PirParams, PirServer
    with open(os.path.join(GOLDEN, f"{name}.json")) as f:
        gold = json.load(f)
    arrays = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    o = oracle_lib.Oracle(gold["num_entries"], gold["max_fst_dim"])  # client side only
    sk, gk, gswk = mg.client(o, gold["key_seed"])
    server = PirServer(PirParams(num_entries=gold["num_entries"], max_fst_dim=gold["max_fst_dim"]))
    server.gen_data(gold["db_seed"])
    server.set_client_galois_key(1, gk)
    server.set_client_gsw_key(1, gswk)
    queries = []
    for j, q in enumerate(gold["queries"]):
        query = o.make_query(sk, q["query_seed"], q["entry"])
        assert sha(query) == q["sha256_query"]
        queries.append(query)
        tr = server.make_query_trace(1, query)
        assert sha(tr["leaves"]) == q["sha256_leaves"]
        if gold["ndim"] > 1:
            assert sha(tr["gsw"]) == q["sha256_gsw"]
        assert sha(tr["first_dim"]) == q["sha256_first_dim"]
        assert sha(tr["resp"]) == q["sha256_resp"]
        assert np.array_equal(tr["resp"], arrays[f"resp{j}"])
        assert np.array_equal(tr["packed"], arrays[f"packed{j}"])
    for engine in ("tensor", "imad", "scan"):
        server.set_batch_engine(engine)
        resp, packed = server.make_query_batch([1] * len(queries), np.stack(queries))
        for j in range(len(queries)):
            assert np.array_equal(resp[j], arrays[f"resp{j}"]), (engine, j)
            assert np.array_equal(packed[j], arrays[f"packed{j}"]), (engine, j)
    server.close()
