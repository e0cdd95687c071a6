"""Replays a dump of the reference itself (oracle/reference_pin/): the
unmodified OnionPIRv2 server and client, built against SEAL 4.1, answering
one query, with its database, keys, query and every stage written out.

Where such a dump exists (oracle/_ref/dump, oracle/_ref/dump_n4096, or the
directory in $OPIR_REFERENCE_DUMP) the oracle must reproduce every stage and
the response bytes from the same inputs, and so must the GPU path: that pins
the SEAL conventions the oracle restates (prime order, plaintext lift,
key-switch rounding, NTT root and order).  SEAL is not in this image, so
without a dump these tests skip.
"""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _dumps():
    env = os.environ.get("OPIR_REFERENCE_DUMP")
    cands = [env] if env else [os.path.join(ROOT, "oracle", "_ref", d)
                               for d in ("dump", "dump_n4096")]
    return [d for d in cands if d and os.path.exists(os.path.join(d, "params.txt"))]


DUMPS = _dumps()
NO_DUMP = ("no dump of the reference: run oracle/reference_pin/build_and_dump.sh with "
           "SEAL_PREFIX set to a SEAL 4.1 install (SEAL is not in this image)")


class Dump:
    def __init__(self, d):
        self.dir = d
        self.p = {}
        with open(os.path.join(d, "params.txt")) as f:
            for line in f:
                k, v = line.split("=")
                self.p[k.strip()] = int(v)
        p = self.p
        self.n, self.R = p["poly_degree"], p["rns"]
        self.moduli = [p[f"modulus{i}"] for i in range(self.R + 1)]

    def u64(self, name, shape):
        a = np.fromfile(os.path.join(self.dir, name), dtype="<u8").astype(np.uint64)
        return a.reshape(shape)

    def raw(self, name):
        with open(os.path.join(self.dir, name), "rb") as f:
            return f.read()

    def params(self):
        from onionpirv2_gb300 import PirParams
        p = self.p
        kw = dict(num_entries=p["num_entries"], max_fst_dim=p["max_fst_dim"])
        if self.n != 2048 or self.R != 1:
            kw.update(poly_degree=self.n, gsw_l=p["l"], gsw_l_key=p["l_key"],
                      plain_mod_bits=p["plain_modulus"].bit_length(),
                      small_q_width=p["small_q"].bit_length(),
                      coeff_mods=tuple(m.bit_length() for m in self.moduli))
        return PirParams(**kw)


def _arrays(D):
    p, n, R = D.p, D.n, D.R
    ct = (2, n) if R == 1 else (2, R, n)
    u = p["n1"] + p["l"] * (p["ndim"] - 1)
    return dict(
        db=D.u64("db_aligned.u64", (-1,)),
        gk=D.u64("galois.u64", (p["expan_height"], R, 2, R + 1, n)),
        gsw=D.u64("gsw_ntt.u64", (2 * p["l_key"],) + ct),
        query=D.u64("query.u64", ct),
        leaves=D.u64("leaves.u64", (u,) + ct),
        gsw_rows=D.u64("gsw_rows.u64", (max(p["ndim"] - 1, 1), 2 * p["l"]) + ct),
        first_dim=D.u64("first_dim.u64", (p["n_rest"],) + ct),
        resp=D.u64("response.u64", (2, n)),
        packed=np.frombuffer(D.raw("response.bin"), np.uint8),
        entry=np.frombuffer(D.raw("entry.bin"), np.uint8))


def replay_oracle(oracle_lib, D):
    P = D.params()
    assert P.coeff_modulus == D.moduli, "prime order (CoeffModulus::Create)"
    assert (P.plain_mod, P.small_q, P.base_log2, P.base_log2_key, P.get_num_pt(),
            P.get_fst_dim_sz()) == (D.p["plain_modulus"], D.p["small_q"], D.p["base_log2"],
                                    D.p["base_log2_key"], D.p["num_pt"], D.p["n1"])
    A = _arrays(D)
    p = D.p
    if D.R == 1:
        o = oracle_lib.Oracle(p["num_entries"], p["max_fst_dim"])
        gk = A["gk"].reshape(p["expan_height"], 2, 2, D.n)
        assert np.array_equal(o.expand(A["query"], gk), A["leaves"]), "expansion"
        for i in range(1, p["ndim"]):
            s = p["n1"] + (i - 1) * p["l"]
            assert np.array_equal(o.query_to_gsw(A["leaves"][s:s + p["l"]], A["gsw"]),
                                  A["gsw_rows"][i - 1]), f"RGSW dimension {i}"
        fd, _ = o.first_dim(A["db"], A["leaves"][: p["n1"]])
        assert np.array_equal(fd, A["first_dim"]), "first dimension"
        resp, packed, _, _ = o.make_query_server(A["db"], gk, A["gsw"], A["query"])
    else:
        o = oracle_lib.RnsOracle(D.n, p["num_entries"], p["max_fst_dim"], l=p["l"],
                                 l_key=p["l_key"], plain_bits=p["plain_modulus"].bit_length(),
                                 small_q_width=p["small_q"].bit_length(),
                                 coeff_bits=tuple(m.bit_length() for m in D.moduli))
        assert np.array_equal(o.expand(A["query"], A["gk"]), A["leaves"]), "expansion"
        fd, _ = o.first_dim(A["db"], A["leaves"][: p["n1"]])
        assert np.array_equal(fd, A["first_dim"]), "first dimension"
        resp, packed, _ = o.make_query_server(A["db"], A["gk"], A["gsw"], A["query"])
    assert np.array_equal(resp, A["resp"]), "response"
    assert np.array_equal(packed, A["packed"]), "packed response"


def replay_gpu(D):
    from onionpirv2_gb300 import PirServer
    A = _arrays(D)
    server = PirServer(D.params())
    server.upload_ntt_db(A["db"])
    server.set_client_galois_key(1, A["gk"])
    # the server takes RGSW(sk) in coefficient form and transforms it itself
    rows = A["gsw"].reshape(-1, D.n)
    coeff = np.concatenate([server.ntt(rows[j::D.R], mod=j, inverse=True)[:, None]
                            for j in range(D.R)], axis=1).reshape(A["gsw"].shape)
    server.set_client_gsw_key(1, coeff)
    tr = server.make_query_trace(1, A["query"])
    assert np.array_equal(tr["leaves"], A["leaves"]), "expansion"
    assert np.array_equal(tr["first_dim"], A["first_dim"]), "first dimension"
    assert np.array_equal(tr["resp"], A["resp"]), "response"
    assert np.array_equal(tr["packed"], A["packed"]), "packed response"
    server.close()


@pytest.mark.skipif(not DUMPS, reason=NO_DUMP)
@pytest.mark.parametrize("d", DUMPS)
def test_oracle_reproduces_the_reference(oracle_lib, d):
    replay_oracle(oracle_lib, Dump(d))


@pytest.mark.gpu
@pytest.mark.skipif(not DUMPS, reason=NO_DUMP)
@pytest.mark.parametrize("d", DUMPS)
def test_gpu_path_reproduces_the_reference(gpu_lib, d):
    replay_gpu(Dump(d))


# ---- the harness itself, on dumps in the driver's format written by the oracle


def write_oracle_dump(oracle_lib, out, n):
    """What dump_reference writes, with the oracle standing in for the
    reference (n = 2048: one prime, 4096 entries; n = 4096: two primes, 1024)."""
    os.makedirs(out, exist_ok=True)
    if n == 2048:
        o = oracle_lib.Oracle(4096, 256)
        P, R, q = o.P, 1, [o.P.q, o.P.p]
        sk = o.keygen(5)
        gk, gsw = o.galois_keys(sk, 6), o.gsw_key(sk, 7)
        gsw_ntt = o.gsw_key_to_ntt(gsw)
        query = o.make_query(sk, 8, 1234)
        db = o.build_db(9)
        leaves = o.expand(query, gk)
        rows = [o.query_to_gsw(leaves[P.n1 + i * P.l: P.n1 + (i + 1) * P.l], gsw_ntt)
                for i in range(P.ndim - 1)]
        fd, _ = o.first_dim(db, leaves[: P.n1])
        resp, packed, _, _ = o.make_query_server(db, gk, gsw_ntt, query)
        entry = o.gen_entries(9, 1234, 1)[0]
        extra = dict(num_entries=4096, max_fst_dim=256, expan_height=P.h)
    else:
        o = oracle_lib.RnsOracle(4096, 1024, 256)
        P, R, q = o.P, 2, list(o.P.q) + [o.P.p]
        sk = o.keygen(5)
        gk, gsw = o.galois_keys(sk, 6), o.gsw_key(sk, 7)
        gsw_ntt = o.gsw_to_ntt(gsw)
        query = o.make_query(sk, 8, 1000)
        db = o.build_db(9)
        leaves = o.expand(query, gk)
        rows = [o.query_to_gsw(leaves[P.n1 + i * P.l: P.n1 + (i + 1) * P.l], gsw_ntt)
                for i in range(P.ndim - 1)]
        fd, _ = o.first_dim(db, leaves[: P.n1])
        resp, packed, _ = o.make_query_server(db, gk, gsw_ntt, query)
        entry = o.gen_entries(9, 1000, 1)[0]
        extra = dict(num_entries=1024, max_fst_dim=256, expan_height=P.h)
    lines = [f"poly_degree = {n}", f"rns = {R}"] + [f"modulus{i} = {m}" for i, m in enumerate(q)]
    lines += [f"plain_modulus = {P.t}", f"small_q = {P.small_q}", f"l = {P.l}",
              f"base_log2 = {P.base_log2}", f"l_key = {P.l_key}",
              f"base_log2_key = {P.base_log2_key}", f"num_pt = {P.num_pt}",
              f"entry_size = {P.entry_size}", f"n1 = {P.n1}", f"n_rest = {P.n_rest}",
              f"ndim = {P.ndim}", "query_index = 0"] + [f"{k} = {v}" for k, v in extra.items()]
    with open(os.path.join(out, "params.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    for name, a in (("db_aligned.u64", db), ("galois.u64", gk), ("gsw_ntt.u64", gsw_ntt),
                    ("query.u64", query), ("leaves.u64", leaves),
                    ("gsw_rows.u64", np.stack(rows)), ("first_dim.u64", fd),
                    ("response.u64", resp)):
        np.ascontiguousarray(a, dtype="<u8").tofile(os.path.join(out, name))
    with open(os.path.join(out, "response.bin"), "wb") as f:
        f.write(np.asarray(packed, np.uint8).tobytes())
    with open(os.path.join(out, "entry.bin"), "wb") as f:
        f.write(np.asarray(entry, np.uint8).tobytes())
    return Dump(out)


@pytest.mark.parametrize("n", [2048, 4096])
def test_replay_harness_on_an_oracle_written_dump(oracle_lib, tmp_path, n):
    replay_oracle(oracle_lib, write_oracle_dump(oracle_lib, str(tmp_path / "dump"), n))


@pytest.mark.gpu
@pytest.mark.parametrize("n", [2048, 4096])
def test_gpu_replay_harness_on_an_oracle_written_dump(oracle_lib, gpu_lib, tmp_path, n):
    replay_gpu(write_oracle_dump(oracle_lib, str(tmp_path / "dump"), n))
