"""CPU oracle checks (no GPU): primitives against mathematics, the x87
rounding pin, and the reference's own end-to-end criterion
(tests.cpp:110-134: decrypted entry == database entry)."""
import platform

import numpy as np
import pytest

N = 2048


@pytest.fixture(scope="module")
def o(oracle_lib):
    return oracle_lib.Oracle(4096, 256)


def test_parameters_match_reference_derivation(o):
    P = o.P
    # pir.cpp:18 generate_prime(16); pir.cpp:22-23,40-41 CoeffModulus::Create
    assert P.t == 32771
    assert P.q == 1152921504606830593 and P.p == 1152921504606748673
    assert P.small_q == 134176769 and P.small_q_width == 27
    assert (P.l, P.base_log2, P.l_key, P.base_log2_key) == (5, 12, 10, 6)
    assert (P.entry_size, P.entries_per_pt, P.bits_per_coeff) == (3840, 1, 15)
    assert (P.n1, P.n_rest, P.ndim, P.u, P.h) == (256, 16, 5, 276, 9)
    for v in (P.q, P.p, P.small_q):
        assert v % (2 * N) == 1


def test_ntt_evaluates_at_odd_powers_of_psi(o):
    fwd, inv, psi, ninv = o.ntt_tables(0)
    q = o.P.q
    assert pow(psi, N, q) == q - 1
    rng = np.random.default_rng(3)
    a = rng.integers(0, q, size=N, dtype=np.uint64)
    A = o.ntt_fwd(a)

    def brv(x):
        return int(format(x, "011b")[::-1], 2)
    coeffs = [int(x) for x in a]
    for k in (0, 1, 2, 1000, 2047):
        x = pow(psi, 2 * brv(k) + 1, q)
        val = 0
        for c in reversed(coeffs):
            val = (val * x + c) % q
        assert val == int(A[k])
    assert np.array_equal(o.ntt_inv(A), a)


def test_ntt_product_is_negacyclic_convolution(o):
    q = o.P.p
    rng = np.random.default_rng(4)
    a = rng.integers(0, 1000, size=N, dtype=np.uint64)
    b = rng.integers(0, 1000, size=N, dtype=np.uint64)
    A, B = o.ntt_fwd(a, 1), o.ntt_fwd(b, 1)
    C = np.array([int(x) * int(y) % q for x, y in zip(A, B)], dtype=np.uint64)
    c = o.ntt_inv(C, 1)
    ai, bi = [int(x) for x in a], [int(x) for x in b]
    ref = [0] * N
    for i in range(N):
        if ai[i] == 0:
            continue
        for j in range(N):
            k = i + j
            if k < N:
                ref[k] += ai[i] * bi[j]
            else:
                ref[k - N] -= ai[i] * bi[j]
    assert [int(x) for x in c] == [r % q for r in ref]


def test_barrett_reduce_128(oracle_lib):
    rng = np.random.default_rng(5)
    L = oracle_lib.lib()
    for q in (1152921504606830593, 1152921504606748673, 134176769, 32771):
        for _ in range(200):
            lo, hi = (int(x) for x in rng.integers(0, 2**64, size=2, dtype=np.uint64))
            assert L.orc_barrett_reduce_128(lo, hi, q) == ((hi << 64) | lo) % q


@pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"),
                    reason="x87 long double exists only on x86")
def test_mod_switch_matches_x87_long_double(o):
    """server.cpp:795-799 on the reference's x86 machine: the integer
    emulation equals (uint64_t)round((long double)x * scale), near ties too."""
    rng = np.random.default_rng(6)
    xs = [0, 1, o.P.q - 1] + [int(x) for x in rng.integers(0, o.P.q, 20000, dtype=np.uint64)]
    M, E = o.P.ms_mant, o.P.ms_exp
    for k in range(1, 4000):
        x = ((2 * k + 1) << (-E - 1)) // M
        xs += [x - 1, x, x + 1]
    for x in xs:
        assert o.mod_switch_coeff(x) == o.x87_mod_switch(x), x


def test_negacyclic_shift_matches_reference_rule(o):
    q = o.P.q
    rng = np.random.default_rng(7)
    ct = rng.integers(0, q, size=(2, N), dtype=np.uint64)
    ct[0, :5] = 0
    k = 8
    out = o.negacyclic_shift(ct, -k)
    for poly in range(2):
        for i in range(N):
            v = int(ct[poly, i])
            if i >= k:
                assert out[poly, i - k] == v
            else:
                assert out[poly, N - k + i] == ((q - v) if v else 0)


def test_key_switch_preserves_plaintext(o):
    """apply_galois = automorphism + key switch: decryption commutes."""
    sk = o.keygen(11)
    gk = o.galois_keys(sk, 12)
    ct = o.make_query(sk, 13, 0)
    plain0, _ = o.decrypt(sk, ct, 0)
    g = N + 1  # level 0: x -> x^(N+1) = x * (-1)^i on coefficient i
    out = o.apply_galois(ct, g, gk[0])
    plain1, budget = o.decrypt(sk, out, 0)
    t = o.P.t
    expect = np.array([(int(v) if i % 2 == 0 else (t - int(v)) % t) for i, v in enumerate(plain0)],
                      dtype=np.uint64)
    assert np.array_equal(plain1, expect)
    assert budget > 20


@pytest.mark.parametrize("idx", [0, 17, 4095])
def test_end_to_end_round_trip(o, idx):
    """The reference's only correctness criterion, tests.cpp:110-134."""
    db = o.build_db(99)
    sk = o.keygen(idx + 1)
    gk = o.galois_keys(sk, idx + 2)
    gsw_ntt = o.gsw_key_to_ntt(o.gsw_key(sk, idx + 3))
    query = o.make_query(sk, idx + 4, idx)
    resp, packed, _, wraps = o.make_query_server(db, gk, gsw_ntt, query)
    assert wraps == 0
    assert packed.size == 13824
    ct = o.unpack_response(packed)
    assert np.array_equal(ct, resp & np.uint64((1 << 27) - 1))
    plain, budget = o.decrypt(sk, ct, 2)
    assert budget > 0
    assert np.array_equal(o.entry_from_plain(idx, plain), o.gen_entries(99, idx, 1)[0])


def test_first_dim_exact_vs_wrapping(o):
    """With n1 = 256 the reference's uint128 sums cannot wrap, so the exact
    oracle equals the reference loop (mat_mat_128) bit for bit."""
    rng = np.random.default_rng(8)
    P = o.P
    db = rng.integers(0, P.q, size=(N, P.num_pt), dtype=np.uint64)
    fst = rng.integers(0, P.q, size=(P.n1, 2, N), dtype=np.uint64)
    exact, wraps = o.first_dim(db, fst)
    assert wraps == 0
    assert np.array_equal(exact, o.first_dim(db, fst, wrapping=True))
