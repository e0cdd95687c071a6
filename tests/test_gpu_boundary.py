"""The reference's public PirServer methods beyond make_query, on the GPU.

save_resp_to_stream (server.cpp:581-633) packs any response ciphertext, not
only the one make_query just returned: rows of a batch and served tickets go
through it and must give the oracle's bytes.  other_dim_mux (server.h:39,
server.cpp:295-334) folds any even number of ciphertexts with one RGSW
selection ciphertext and must equal the oracle's fold bit for bit.
"""
import io

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048


@pytest.fixture(scope="module")
def served(oracle_lib, gpu_lib):
    from onionpirv2_gb300 import PirParams, PirServer
    o = oracle_lib.Oracle(4096, 256)
    server = PirServer(PirParams(num_entries=4096, max_fst_dim=256))
    seed = 777
    server.gen_data(seed)
    sk = o.keygen(31)
    gk, gswk = o.galois_keys(sk, 32), o.gsw_key(sk, 33)
    server.set_client_galois_key(5, gk)
    server.set_client_gsw_key(5, gswk)
    yield o, server, sk
    server.close()


def test_save_resp_to_stream_packs_batched_and_served_responses(served):
    o, server, sk = served
    idxs = [0, 17, 2048, 4095, 1234, 999]
    queries = np.stack([o.make_query(sk, 600 + j, i) for j, i in enumerate(idxs)])
    singles = [server.make_query(5, q) for q in queries]
    resps, packed = server.make_query_batch([5] * len(idxs), queries)
    for j in range(len(idxs)):
        want = o.pack_response(singles[j])
        assert singles[j].packed == want.tobytes()
        # a batch row is a plain array: packed on the GPU by save_resp_to_stream
        buf = io.BytesIO()
        n = server.save_resp_to_stream(np.array(resps[j]), buf)
        assert n == len(want) and buf.getvalue() == want.tobytes(), f"batch row {j}"
        assert np.array_equal(packed[j], want)
    server.serve_start(max_batch=4, lanes=2, max_wait_us=500)
    try:
        tickets = [server.submit(5, q) for q in queries]
        outs = [server.wait(t) for t in tickets]
    finally:
        server.serve_stop()
    for j, r in enumerate(outs):
        want = o.pack_response(singles[j]).tobytes()
        assert r.packed == want
        buf = io.BytesIO()
        server.save_resp_to_stream(np.array(r), buf)  # without the attached bytes
        assert buf.getvalue() == want, f"served response {j}"
    # several at once, and coefficients with bits above the packing width are
    # masked as the reference masks them (server.cpp:608)
    rng = np.random.default_rng(3)
    cts = rng.integers(0, 2**40, size=(3, 2, N), dtype=np.uint64)
    got = server.pack_responses(cts)
    for j in range(3):
        assert np.array_equal(got[j], o.pack_response(cts[j] & np.uint64((1 << 27) - 1)))


@pytest.mark.parametrize("count", [2, 96, 600])
def test_other_dim_mux_matches_oracle(served, count):
    """The one-CTA, two-CTA and cluster folding forms (chosen by the number
    of pairs) through the public other_dim_mux."""
    o, server, _ = served
    P = o.P
    rng = np.random.default_rng(count)
    q = np.uint64(P.q)
    result = rng.integers(0, 2**62, size=(count, 2, N), dtype=np.uint64) % q
    sel = rng.integers(0, 2**62, size=(2 * P.l, 2, N), dtype=np.uint64) % q
    got = server.other_dim_mux(result, sel)
    want = o.other_dim_mux(result, sel)
    assert got.shape == (count // 2, 2, N)
    assert np.array_equal(got, want)


def test_other_dim_mux_rejects_odd_counts(served):
    from onionpirv2_gb300 import _capi
    o, server, _ = served
    with pytest.raises(ValueError):
        server.other_dim_mux(np.zeros((3, 2, N), np.uint64), np.zeros((2 * o.P.l, 2, N), np.uint64))
    L = _capi.load()
    r = np.zeros(3 * 2 * N, np.uint64)
    sel = np.zeros(2 * o.P.l * 2 * N, np.uint64)
    assert L.opir_other_dim_mux(server.ctx, _capi.p64(r), 3, _capi.p64(sel)) == -1
