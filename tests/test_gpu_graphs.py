"""The device-pointer query call inside a caller's own CUDA graph: the
library launches directly while the caller captures, and replaying the
caller's graph gives the same responses as calling the library."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_query_in_a_callers_cuda_graph(gpu_lib):
    torch = pytest.importorskip("torch")
    from onionpirv2_gb300 import PirClient, PirParams, PirServer
    params = PirParams(num_entries=4096, max_fst_dim=256)
    server = PirServer(params)
    server.gen_data(606)
    clients = [PirClient(params, i, secret_seed=10 + i) for i in range(2)]
    for c in clients:
        server.set_client_galois_key(c.get_client_id(), c.create_galois_keys(seed=1))
        server.set_client_gsw_key(c.get_client_id(), c.generate_gsw_from_key(seed=2))
    n = 2048
    queries = np.stack([clients[j].fast_generate_query(100 + 17 * j, seed=5) for j in range(2)])
    dq = torch.from_numpy(queries.view(np.int64)).cuda()
    dresp = torch.zeros((2, 2, n), dtype=torch.int64, device="cuda")
    dpack = torch.zeros((2, server.resp_bytes), dtype=torch.uint8, device="cuda")
    qbytes, rb = 2 * n * 8, server.resp_bytes
    s = torch.cuda.Stream()
    server.set_stream(s.cuda_stream)

    def calls():
        for j in range(2):
            server.make_query_device([j], dq.data_ptr() + j * qbytes, dresp.data_ptr() + j * qbytes,
                                     dpack.data_ptr() + j * rb)

    with torch.cuda.stream(s):
        calls()  # warm-up: workspace sized, library graphs captured
        s.synchronize()
    ref = dresp.clone()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        calls()
    dresp.zero_()
    with torch.cuda.stream(s):
        g.replay()
        s.synchronize()
    assert torch.equal(dresp, ref)
    for j in range(2):
        entry, _ = clients[j].decode_response(100 + 17 * j, dpack[j].cpu().numpy().tobytes())
        assert np.array_equal(entry, server.direct_get_entry(100 + 17 * j))
    server.close()
