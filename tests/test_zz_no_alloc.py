"""The allocation-free first-dimension entry point.

opir_first_dim_noalloc serves callers that cannot call cudaMalloc during a
request (a request thread with a latency budget, since allocation
synchronises the device, or a process whose device memory another allocator
reserved up front): it keeps the scan's query operand in a static device
array instead of context workspace.  Its output must equal the
first-dimension result that the regular entry point (opir_make_query_trace)
reports, call after call, since every call reuses the same static array, and
after the first call (which may load the library's device code) the device's
free memory must not move.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048


def _client(o, seed):
    sk = o.keygen(seed)
    return sk, o.galois_keys(sk, seed + 1), o.gsw_key(sk, seed + 2)


def test_first_dim_noalloc_matches_regular_entry_point(oracle_lib, gpu_lib):
    import torch
    from onionpirv2_gb300 import PirParams, PirServer, _capi
    L = _capi.load()
    o = oracle_lib.Oracle(4096, 256)
    P = o.P
    server = PirServer(PirParams(num_entries=4096, max_fst_dim=256))
    server.gen_data(404)
    sk, gk, gswk = _client(o, 9)
    server.set_client_galois_key(3, gk)
    server.set_client_gsw_key(3, gswk)
    out = torch.empty((P.n_rest, 2, N), dtype=torch.int64, device="cuda")
    traces = [server.make_query_trace(3, o.make_query(sk, 50 + call, idx))
              for call, idx in enumerate((123, 3999))]  # two calls in a row, different queries
    fsts = [torch.from_numpy(np.ascontiguousarray(tr["leaves"][:P.n1]).view(np.int64)).cuda()
            for tr in traces]
    for call, (tr, fst) in enumerate(zip(traces, fsts)):
        out.fill_(-1)  # stale contents must not survive
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        rc = L.opir_first_dim_noalloc(server.ctx, server.db_id, ctypes.c_void_p(fst.data_ptr()),
                                      ctypes.c_void_p(out.data_ptr()))
        _capi.check(server.ctx, rc)
        _capi.check(server.ctx, L.opir_sync(server.ctx))
        if call > 0:
            assert torch.cuda.mem_get_info()[0] == free0, "the call allocated device memory"
        got = out.cpu().numpy().view(np.uint64)
        assert np.array_equal(got, tr["first_dim"]), f"call {call}"
    server.close()


def test_first_dim_noalloc_rejects_oversized_first_dimension(gpu_lib):
    import torch
    from onionpirv2_gb300 import PirParams, PirServer, _capi
    L = _capi.load()
    server = PirServer(PirParams(num_entries=1024, max_fst_dim=1024))  # n1 = 1024 > 512
    assert server.pir_params.get_fst_dim_sz() == 1024
    fst = torch.zeros((1024, 2, N), dtype=torch.int64, device="cuda")
    out = torch.zeros((1, 2, N), dtype=torch.int64, device="cuda")
    rc = L.opir_first_dim_noalloc(server.ctx, server.db_id, ctypes.c_void_p(fst.data_ptr()),
                                  ctypes.c_void_p(out.data_ptr()))
    assert rc == -1
    assert "static scratch" in L.opir_last_error(server.ctx).decode()
    server.close()
