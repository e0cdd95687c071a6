"""The tensor engine's exactness bound, driven to its extremes.

The tensor-core first dimension splits database residues into balanced 8-bit
limbs ([-128, 127], top limb [0, 16]) and query residues into balanced 8-bit
or 9-bit limbs ([-256, 255], top limb [0, 64]); the fp32 sums of 512 limb
products must stay exact.  Random residues only reach about 2^17 there.
These tests give every database residue and every query-plane residue the
same value, chosen so that all of its lower limbs sit at one end of their
range: with 9-bit query limbs each product is then +-2^15 and a 512-k
segment sums to exactly +-2^24 (2^23 with 8-bit limbs).  A constant plane is
the transform of a constant polynomial, so the leaves are constant
polynomials and every first-dimension result is the constant polynomial
n1 * v_db * v_q mod q.
"""
import ctypes

import numpy as np
import pytest


def balanced(v, bits, count):
    """The kernel's balanced limbs of v (lower limbs in [-2^(bits-1), 2^(bits-1)))."""
    out, carry = [], 0
    for _ in range(count - 1):
        x = (v & ((1 << bits) - 1)) + carry
        v >>= bits
        carry = 1 if x >= 1 << (bits - 1) else 0
        out.append(x - (carry << bits))
    out.append(v + carry)
    return out


def from_limbs(limbs, bits):
    return sum(d << (bits * i) for i, d in enumerate(limbs))


def residue(bits, count, low, top):
    v = from_limbs([low] * (count - 1) + [top], bits)
    assert balanced(v, bits, count) == [low] * (count - 1) + [top]
    return v


# database residues (8-bit limbs) and query residues of each width, at the
# bottom and the top of the limb range
DB_LOW, DB_HIGH = residue(8, 8, -128, 16), residue(8, 8, 127, 14)
Q_LOW = {8: residue(8, 8, -128, 16), 9: residue(9, 7, -256, 64)}
Q_HIGH = {8: residue(8, 8, 127, 14), 9: residue(9, 7, 255, 62)}


def test_extreme_residues_are_below_q():
    from onionpirv2_gb300 import PirParams
    q = PirParams(num_entries=8192, max_fst_dim=512).coeff_modulus[0]
    for v in (DB_LOW, DB_HIGH, *Q_LOW.values(), *Q_HIGH.values()):
        assert 0 <= v < q


@pytest.mark.gpu
@pytest.mark.parametrize("limbs", [8, 9])
@pytest.mark.parametrize("shape", [(8192, 512), (16384, 1024), (16384, 512), (32768, 1024)])
@pytest.mark.parametrize("db_end,q_end", [("low", "low"), ("low", "high"), ("high", "high")])
def test_limb_sums_at_the_exactness_bound(gpu_lib, monkeypatch, limbs, shape, db_end, q_end):
    """Both query limb widths give n1 * v_db * v_q mod q in every slot when
    every limb product sits at the end of its range: one 512-k segment and
    two segments summed in the epilogue, one CTA per 16-row tile (n_rest =
    16) and CTA pairs (n_rest = 32)."""
    from onionpirv2_gb300 import PirParams, PirServer, _capi
    monkeypatch.setenv("OPIR_TC_LIMBS", "0" if limbs == 8 else "1")
    monkeypatch.setenv("OPIR_TC_PAIR", "1")  # pairs wherever the rows pair up
    monkeypatch.setenv("OPIR_GRAPHS", "0")
    P = PirParams(num_entries=shape[0], max_fst_dim=shape[1])
    n, n1, nr, q = 2048, P.get_fst_dim_sz(), P.get_other_dim_sz(), P.coeff_modulus[0]
    v_db = DB_LOW if db_end == "low" else DB_HIGH
    v_q = (Q_LOW if q_end == "low" else Q_HIGH)[limbs]
    server = PirServer(P)
    server.upload_ntt_db(np.full(P.get_num_pt() * n, v_db, np.uint64))
    server.set_batch_engine("tensor")
    batch = 4
    leaves = np.zeros((batch, n1, 2, n), np.uint64)
    leaves[:, :, :, 0] = v_q
    out = np.zeros((batch, nr, 2, n), np.uint64)
    L = server._L
    _capi.check(server.ctx, L.opir_debug_first_dim(
        server.ctx, server.db_id, batch, leaves.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
        out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
    want = np.zeros_like(out)
    want[:, :, :, 0] = n1 * v_db * v_q % q
    assert np.array_equal(out, want)
    server.close()


@pytest.mark.gpu
@pytest.mark.parametrize("limbs", [8, 9])
def test_hook_matches_the_oracle_on_random_operands(oracle_lib, gpu_lib, monkeypatch, limbs):
    """The first-dimension hook on the tensor engine equals the oracle's
    first dimension for random leaves (and so does the per-query scan)."""
    from onionpirv2_gb300 import PirParams, PirServer, _capi
    monkeypatch.setenv("OPIR_TC_LIMBS", "0" if limbs == 8 else "1")
    shape = (1 << 14, 1024)
    o = oracle_lib.Oracle(*shape)
    P = o.P
    server = PirServer(PirParams(num_entries=shape[0], max_fst_dim=shape[1]))
    server.gen_data(5)
    db = o.build_db(5)
    rng = np.random.default_rng(limbs)
    batch = 3
    leaves = rng.integers(0, P.q, size=(batch, P.n1, 2, 2048), dtype=np.uint64)
    for engine in ("tensor", "scan"):
        server.set_batch_engine(engine)
        out = np.zeros((batch, P.n_rest, 2, 2048), np.uint64)
        _capi.check(server.ctx, server._L.opir_debug_first_dim(
            server.ctx, server.db_id, batch,
            leaves.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
            out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
        for b in range(batch):
            ref, _ = o.first_dim(db, leaves[b])
            assert np.array_equal(out[b], ref), (engine, b)
    server.close()
