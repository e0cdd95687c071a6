"""The CPU PirClient (include/onionpir_client.hpp through libopir_client.so):
its seeded outputs equal the oracle client's bit for bit, it reproduces the
committed golden fixtures, it decodes the oracle server's responses back to
the database entries, and its ChaCha20 stream meets the RFC 8439 vectors."""
import io
import json
import os
import re
import threading

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def client_mod():
    from onionpirv2_gb300 import build
    build.build_client()
    from onionpirv2_gb300 import client
    return client


def _sha(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_client_library_exports_every_declared_symbol(client_mod):
    import ctypes
    with open(os.path.join(ROOT, "include", "onionpir_client.h")) as f:
        declared = set(re.findall(r"\b(opir_(?:client_\w+|chacha20_block))\s*\(", f.read()))
    assert declared == set(client_mod.CLIENT_EXPORTS)
    L = client_mod.load()
    for name in declared:
        assert isinstance(getattr(L, name), ctypes._CFuncPtr)


def test_chacha20_rfc8439_vectors(client_mod):
    # RFC 8439 section 2.3.2: key 00..1f, counter 1, nonce 00:00:00:09:00:00:00:4a:00:00:00:00
    out = client_mod.chacha20_block(bytes(range(32)), 1, bytes.fromhex("000000090000004a00000000"))
    assert out.hex() == (
        "10f1e7e4d13b5915500fdd1fa32071c4c7d1f4c733c068030422aa9ac3d46c4e"
        "d2826446079faa0914c2d705d98b02a2b5129cd1de164eb9cbd083e8a2503c4e")
    # RFC 8439 appendix A.1, test vector 1: all-zero key and nonce, counter 0
    out = client_mod.chacha20_block(bytes(32), 0, bytes(12))
    assert out.hex() == (
        "76b8e0ada0f13d90405d6ae55386bd28bdd219b8a08ded1aa836efcc8b770dc7"
        "da41597c5157488d7724e03fb8d84a376a43b8f41518a11cc387b669b2ee6586")


@pytest.mark.parametrize("shape", [(4096, 256), (1 << 13, 64), (1 << 14, 1024), (1024, 16)])
def test_seeded_client_equals_oracle_client(client_mod, oracle_lib, shape):
    from onionpirv2_gb300 import PirParams
    params = PirParams(num_entries=shape[0], max_fst_dim=shape[1])
    o = oracle_lib.Oracle(*shape)
    c = client_mod.PirClient(params, client_id=5, secret_seed=41)
    sk = o.keygen(41)
    assert np.array_equal(c.secret_key(), sk)
    assert c.height == o.P.h
    assert np.array_equal(c.create_galois_keys(seed=42), o.galois_keys(sk, 42))
    assert np.array_equal(c.generate_gsw_from_key(seed=43), o.gsw_key(sk, 43))
    rng = np.random.default_rng(shape[0])
    for idx in rng.integers(0, o.P.num_entries, size=4):
        idx = int(idx)
        assert np.array_equal(c.fast_generate_query(idx, seed=44 + idx), o.make_query(sk, 44 + idx, idx))
        pt = idx // params.get_num_entries_per_plaintext()
        assert c.get_query_indices(pt) == list(o.query_indices(pt))
    # decryption of arbitrary ciphertexts at both moduli, and the noise budget
    for mod, at_q in ((2, 0), (0, 1)):
        Q = o.P.small_q if mod == 2 else o.P.q
        ct = rng.integers(0, Q, size=(2, 2048), dtype=np.uint64)
        plain, budget = (c.decrypt_ct if at_q else c.decrypt_mod_q)(ct)
        ref_plain, ref_budget = o.decrypt(sk, ct, mod)
        assert np.array_equal(plain, ref_plain) and budget == ref_budget
    plain = rng.integers(0, o.P.t, size=2048, dtype=np.uint64)
    for idx in (0, 1, params.get_num_entries_per_plaintext() - 1):
        assert np.array_equal(c.get_entry_from_plaintext(idx, plain), o.entry_from_plain(idx, plain))
    packed = rng.integers(0, 256, size=c.resp_bytes, dtype=np.uint8)
    assert np.array_equal(c.load_resp_from_stream(io.BytesIO(packed.tobytes())),
                          o.unpack_response(packed))


@pytest.mark.parametrize("name", ["db4096", "db8192_n64", "db16384_n1024"])
def test_client_reproduces_golden_queries_and_decodes_golden_responses(client_mod, oracle_lib, name):
    from onionpirv2_gb300 import PirParams
    with open(os.path.join(GOLDEN, f"{name}.json")) as f:
        gold = json.load(f)
    arrays = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    params = PirParams(num_entries=gold["num_entries"], max_fst_dim=gold["max_fst_dim"])
    c = client_mod.PirClient(params, secret_seed=gold["key_seed"])
    o = oracle_lib.Oracle(gold["num_entries"], gold["max_fst_dim"])
    for j, q in enumerate(gold["queries"]):
        assert _sha(c.fast_generate_query(q["entry"], seed=q["query_seed"])) == q["sha256_query"]
        packed = arrays[f"packed{j}"]
        assert np.array_equal(c.load_resp_from_stream(io.BytesIO(packed.tobytes())), arrays[f"resp{j}"])
        entry, budget = c.decode_response(q["entry"], packed.tobytes())
        assert budget == q["noise_budget"]
        assert np.array_equal(entry, o.gen_entries(gold["db_seed"], q["entry"], 1)[0])


def test_os_entropy_client_round_trip_through_oracle_server(client_mod, oracle_lib):
    """Unseeded (ChaCha20) keys and queries: two clients differ, and the
    oracle server's responses decode to the database entries."""
    from onionpirv2_gb300 import PirParams
    params = PirParams(num_entries=4096, max_fst_dim=256)
    o = oracle_lib.Oracle(4096, 256)
    db = o.build_db(99)
    a, b = client_mod.PirClient(params, 1), client_mod.PirClient(params, 2)
    assert not np.array_equal(a.secret_key(), b.secret_key())
    assert set(np.unique(a.secret_key())) <= {-1, 0, 1}
    gk, gsw = a.create_galois_keys(), a.generate_gsw_from_key()
    assert not np.array_equal(gk, a.create_galois_keys())  # fresh randomness per call
    gsw_ntt = o.gsw_key_to_ntt(gsw)
    for idx in (0, 777, 4095):
        _, packed, _, _ = o.make_query_server(db, gk, gsw_ntt, a.fast_generate_query(idx))
        entry, budget = a.decode_response(idx, packed.tobytes())
        assert np.array_equal(entry, o.gen_entries(99, idx, 1)[0])
        assert budget > 0


def test_client_errors(client_mod):
    from onionpirv2_gb300 import PirParams
    params = PirParams(num_entries=4096, max_fst_dim=256)
    c = client_mod.PirClient(params, secret_seed=1)
    with pytest.raises(ValueError):
        c.fast_generate_query(params.get_num_entries(), seed=1)  # past the last entry
    with pytest.raises(ValueError):
        c.load_resp_from_stream(io.BytesIO(b"\0" * (c.resp_bytes - 1)))  # truncated stream
    with pytest.raises(ValueError):
        c.get_query_indices(params.get_num_pt())


def test_clients_generate_keys_concurrently(client_mod):
    """Threads share the NTT tables; each thread's seeded output is the same
    as when run alone."""
    from onionpirv2_gb300 import PirParams
    params = PirParams(num_entries=1 << 13, max_fst_dim=64)
    clients = [client_mod.PirClient(params, i, secret_seed=100 + i) for i in range(8)]
    alone = [c.create_galois_keys(seed=7) for c in clients]
    out = [None] * len(clients)

    def work(i):
        out[i] = clients[i].create_galois_keys(seed=7)

    ts = [threading.Thread(target=work, args=(i,)) for i in range(len(clients))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert all(np.array_equal(x, y) for x, y in zip(out, alone))


def test_cpp_client_header_against_oracle(oracle_lib):
    """tests/cpp/test_pir_client.cpp: PirParams::derive and the seeded C++
    PirClient equal the oracle's, and oracle-server responses decode."""
    import subprocess
    out_dir = os.path.join(ROOT, "tests", "cpp", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "test_pir_client")
    orc_dir = os.path.join(ROOT, "oracle", "_build")
    subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-Werror",
                    "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle"),
                    os.path.join(ROOT, "tests", "cpp", "test_pir_client.cpp"), "-o", exe,
                    f"-L{orc_dir}", "-lopir_oracle", f"-Wl,-rpath,{orc_dir}"], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Success rate: 6/6, same as the oracle client: 6/6" in r.stdout
