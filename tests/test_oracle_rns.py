"""The multi-modulus oracle (oracle/opir_oracle_rns.c), on the CPU.

It must (1) reproduce the single-modulus oracle bit for bit at N = 2048 with
one ciphertext prime -- keys, queries, database and every server stage -- and
(2) at N = 4096 with two ciphertext primes (the PolyDegree = 4096,
CoeffMods = {60, 60, 60} presets of database_constants.h:13-172) answer
queries whose responses decrypt to the database entry (the reference's
criterion, tests.cpp:110-134), with the CRT decomposition and the modulus
switch to the next prime (server.cpp:567-570) checked against big-integer
arithmetic.
"""
import numpy as np
import pytest

# the "2^14 * 24KB" preset of database_constants.h at a CPU-sized entry count
N4096 = dict(l=4, l_key=8, plain_bits=46, small_q_width=57, coeff_bits=(60, 60, 60))


@pytest.fixture(scope="module")
def rns2(oracle_lib):
    r = oracle_lib.RnsOracle(4096, 1024, 256, **N4096)
    return r, r.build_db(7)


def test_single_prime_matches_the_single_modulus_oracle(oracle_lib):
    o = oracle_lib.Oracle(4096, 256)
    r = oracle_lib.RnsOracle(2048, 4096, 256, l=5, l_key=10, plain_bits=16, small_q_width=27,
                             coeff_bits=(60, 60))
    for f in ("t", "small_q", "small_q_width", "l", "base_log2", "l_key", "base_log2_key",
              "num_pt", "entry_size", "n1", "n_rest", "ndim", "u", "h", "ms_mant", "ms_exp"):
        assert getattr(o.P, f) == getattr(r.P, f), f
    assert (o.P.q, o.P.p) == (r.P.q[0], r.P.p)
    sk = o.keygen(11)
    assert np.array_equal(sk, r.keygen(11))
    gk, gs = o.galois_keys(sk, 12), o.gsw_key(sk, 13)
    assert np.array_equal(gk.reshape(-1), r.galois_keys(sk, 12).reshape(-1))
    assert np.array_equal(gs.reshape(-1), r.gsw_key(sk, 13).reshape(-1))
    db = o.build_db(5)
    assert np.array_equal(db.reshape(-1), r.build_db(5))
    gsn = o.gsw_key_to_ntt(gs)
    for idx in (0, 1234, 4095):
        q = o.make_query(sk, 99 + idx, idx)
        assert np.array_equal(q.reshape(-1), r.make_query(sk, 99 + idx, idx).reshape(-1))
        leaves = o.expand(q, gk)
        assert np.array_equal(leaves.reshape(-1), r.expand(q, gk).reshape(-1))
        resp, packed, _, _ = o.make_query_server(db, gk, gsn, q)
        resp2, packed2, _ = r.make_query_server(db, gk, gsn, q)
        assert np.array_equal(resp.reshape(-1), resp2.reshape(-1))
        assert np.array_equal(packed, packed2)


def test_two_primes_answer_decrypts_to_the_entry(rns2):
    r, db = rns2
    P = r.P
    assert (P.n, P.rns, P.base_log2, P.base_log2_key, P.small_q_width) == (4096, 2, 30, 15, 57)
    assert P.q[0] > P.q[1] > P.p  # CoeffModulus::Create order; the last is special
    sk = r.keygen(21)
    gk, gsn = r.galois_keys(sk, 22), r.gsw_to_ntt(r.gsw_key(sk, 23))
    for idx in (0, 5, 1023, 438):
        resp, packed, wraps = r.make_query_server(db, gk, gsn, r.make_query(sk, 30 + idx, idx))
        plain, budget = r.decrypt_small(sk, resp)
        assert np.array_equal(r.entry_from_plain(idx, plain), r.gen_entries(7, idx, 1)[0]), idx
        assert budget > 0 and wraps == 0
        assert len(packed) == r.response_bytes() == 2 * 4096 * 57 // 8


def test_crt_decomposition_and_modulus_switch_follow_big_integers(rns2):
    r, _ = rns2
    P = r.P
    q0, q1 = P.q
    rng = np.random.default_rng(4)
    ct = np.stack([rng.integers(0, q, size=(2, 4096), dtype=np.uint64) for q in (q0, q1)], axis=1)
    for l, b in ((P.l, P.base_log2), (P.l_key, P.base_log2_key)):
        d = r.decompose(ct, l, b)
        for poly in range(2):
            for c in (0, 1, 4095):
                x0, x1 = int(ct[poly, 0, c]), int(ct[poly, 1, c])
                X = x1 + q1 * (((x0 - x1) * pow(q1, -1, q0)) % q0)
                assert X % q0 == x0 and X % q1 == x1 and X < q0 * q1
                for j in range(l):
                    want = (X >> ((l - 1 - j) * b)) & ((1 << b) - 1)
                    assert int(d[poly * l + j, 0, c]) == want == int(d[poly * l + j, 1, c])
    nxt = r.mod_switch_next(ct)
    for poly in range(2):
        for c in (0, 7, 4095):
            x0, x1 = int(ct[poly, 0, c]), int(ct[poly, 1, c])
            X = x1 + q1 * (((x0 - x1) * pow(q1, -1, q0)) % q0)
            assert int(nxt[poly, 0, c]) == ((X + q1 // 2) // q1) % q0  # round(X / q1) mod q0


def test_product_parameters_match_the_oracle(oracle_lib):
    """onionpirv2_gb300.PirParams for the N = 4096 presets derives what the
    oracle derives (pir.cpp:9-95)."""
    from onionpirv2_gb300 import PirParams
    for name in ("n4096_384MB", "rns1024", "rns16384"):
        p = PirParams.preset(name)
        r = oracle_lib.RnsOracle(p.poly_degree, p.num_entries, p.max_fst_dim, l=p.gsw_l,
                                 l_key=p.gsw_l_key, plain_bits=p.plain_mod_bits,
                                 small_q_width=p.small_q_width, coeff_bits=tuple(p.coeff_mods))
        P = r.P
        assert p.is_multi_modulus() and p.get_rns_mod_cnt() == P.rns == 2
        assert tuple(p.get_coeff_modulus()) == P.q and p.coeff_modulus[-1] == P.p
        assert (p.plain_mod, p.small_q, p.base_log2, p.base_log2_key) == (
            P.t, P.small_q, P.base_log2, P.base_log2_key)
        assert (p.get_entry_size(), p.get_num_pt(), p.get_fst_dim_sz(), p.get_other_dim_sz(),
                len(p.get_dims()), p.get_expan_height()) == (
            P.entry_size, P.num_pt, P.n1, P.n_rest, P.ndim, P.h)
        assert p.response_bytes() == r.response_bytes()
