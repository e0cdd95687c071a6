"""The oracle reproduces the committed golden fixtures (tests/golden/, made
by tests/golden/make_golden.py from seeded inputs): every intermediate of the
query path hashes to the recorded value, the responses and packed bytes match
byte for byte, and each decrypted entry equals the database entry."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def load_cases():
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden
    return make_golden


@pytest.mark.parametrize("name", ["db4096", "db8192_n64", "db16384_n1024"])
def test_oracle_reproduces_golden(oracle_lib, name):
    mg = load_cases()
    with open(os.path.join(GOLDEN, f"{name}.json")) as f:
        gold = json.load(f)
    arrays = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    o = oracle_lib.Oracle(gold["num_entries"], gold["max_fst_dim"])
    assert (o.P.n1, o.P.n_rest, o.P.ndim) == (gold["n1"], gold["n_rest"], gold["ndim"])
    db = o.build_db(gold["db_seed"])
    assert mg.sha(db) == gold["sha256_db"]
    sk, gk, gswk = mg.client(o, gold["key_seed"])
    gsw_ntt = o.gsw_key_to_ntt(gswk)
    for j, q in enumerate(gold["queries"]):
        query = o.make_query(sk, q["query_seed"], q["entry"])
        assert mg.sha(query) == q["sha256_query"]
        leaves, gsw, fd, resp, packed = mg.stages(o, db, gk, gsw_ntt, query)
        assert mg.sha(leaves) == q["sha256_leaves"]
        assert mg.sha(gsw) == q["sha256_gsw"]
        assert mg.sha(fd) == q["sha256_first_dim"]
        assert mg.sha(resp) == q["sha256_resp"]
        assert np.array_equal(resp, arrays[f"resp{j}"])
        assert np.array_equal(packed, arrays[f"packed{j}"])
        plain, _ = o.decrypt(sk, resp, 2)
        assert np.array_equal(o.entry_from_plain(q["entry"], plain),
                              o.gen_entries(gold["db_seed"], q["entry"], 1)[0])
