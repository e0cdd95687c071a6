"""Generate the golden fixtures of the query path from the seeded oracle.

The reference ships no golden vectors and cannot be built here (it needs the
SEAL 4.1 fork), so these fixtures pin the oracle and the CUDA path to one
fixed, seeded run: for each shape, the SHA-256 of every intermediate of
PirServer::make_query (NTT-form database plane, expanded ciphertexts, RGSW
rows, first-dimension result mod q, response, packed bytes) plus the response
and packed bytes themselves, and the responses of a small batch of queries.
Each database entry decrypted from the response equals the generated entry
(the reference's own end-to-end criterion, tests.cpp:110-134).

    python tests/golden/make_golden.py      # rewrites tests/golden/*.json, *.npz
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# (name, num_entries, max_fst_dim, db seed, key seed, [(query seed, entry index)])
CASES = [
    ("db4096", 4096, 256, 2024, 1, [(4, 3001), (5, 0), (6, 4095)]),
    ("db8192_n64", 1 << 13, 64, 77, 500, [(900, 5), (901, 8191), (902, 4100)]),
    ("db16384_n1024", 1 << 14, 1024, 31, 5, [(17, 10922), (18, 1), (19, 16000)]),
]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).astype("<u8").tobytes()).hexdigest()


def client(o, key_seed):
    sk = o.keygen(key_seed)
    return sk, o.galois_keys(sk, key_seed + 1), o.gsw_key(sk, key_seed + 2)


def stages(o, db, gk, gsw_ntt, query):
    """Every intermediate of one query on the oracle."""
    P = o.P
    leaves = o.expand(query, gk)
    gsw = np.stack([o.query_to_gsw(leaves[P.n1 + (i - 1) * P.l:P.n1 + i * P.l], gsw_ntt)
                    for i in range(1, P.ndim)]) if P.ndim > 1 else np.zeros((0,), np.uint64)
    fd, _ = o.first_dim(db, leaves[:P.n1])
    resp, packed, _, _ = o.make_query_server(db, gk, gsw_ntt, query)
    return leaves, gsw, fd, resp, packed


def generate(oracle_mod):
    out = {}
    for name, ne, fd_max, db_seed, key_seed, queries in CASES:
        o = oracle_mod.Oracle(ne, fd_max)
        P = o.P
        db = o.build_db(db_seed)
        sk, gk, gswk = client(o, key_seed)
        gsw_ntt = o.gsw_key_to_ntt(gswk)
        case = {"num_entries": ne, "max_fst_dim": fd_max, "db_seed": db_seed,
                "key_seed": key_seed, "n1": P.n1, "n_rest": P.n_rest, "ndim": P.ndim,
                "sha256_db": sha(db), "queries": []}
        arrays = {}
        for j, (qseed, idx) in enumerate(queries):
            query = o.make_query(sk, qseed, idx)
            leaves, gsw, fd, resp, packed = stages(o, db, gk, gsw_ntt, query)
            plain, budget = o.decrypt(sk, resp, 2)
            entry = o.entry_from_plain(idx, plain)
            assert np.array_equal(entry, o.gen_entries(db_seed, idx, 1)[0]), (name, idx)
            case["queries"].append({
                "query_seed": qseed, "entry": idx, "sha256_query": sha(query),
                "sha256_leaves": sha(leaves), "sha256_gsw": sha(gsw),
                "sha256_first_dim": sha(fd), "sha256_resp": sha(resp),
                "sha256_packed": hashlib.sha256(packed.tobytes()).hexdigest(),
                "noise_budget": int(budget)})
            arrays[f"resp{j}"] = resp
            arrays[f"packed{j}"] = packed
        out[name] = (case, arrays)
    return out


def main():
    sys.path.insert(0, ROOT)
    from oracle import oracle as orc
    orc.build()
    for name, (case, arrays) in generate(orc).items():
        with open(os.path.join(HERE, f"{name}.json"), "w") as f:
            json.dump(case, f, indent=1)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
        print("wrote", name)


if __name__ == "__main__":
    main()
