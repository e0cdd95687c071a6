#!/usr/bin/env python3
"""Benchmark of the OnionPIRv2 server query path on GB300.

Workload (default): the 262,144-plaintext database (n1 x n_rest = 512 x 512,
N = 2048, one 60-bit q, ~1 GB of raw entries, 4.29 GB in NTT form), one
query per step through the whole pipeline of PirServer::make_query
(expansion, RGSW reconstruction, first-dimension scan, 9 folds, modulus
switch, packing).

  value  queries/s with queries resident in HBM, CUDA events on the
         library's stream around K steps (each step one query).
  e2e    the same through the public host API (opir_make_query): host query
         -> pinned staging -> device -> response and packed bytes -> host.
  roofline  the dominant kernel (first-dimension scan): NTT-form DB bytes per
         launch / mean launch time (CUDA events around the launch), against
         the measured HBM copy bandwidth.
  cpu_baseline  the CPU restatement of the reference server (oracle/), all
         host threads, full queries on the same database and inputs; its
         responses are also compared bit for bit with the GPU's.
  batched  32 queries per step sharing one pass over the database on the
         tensor-core engine (and the integer engine beside it).
  large  the 2,097,152-plaintext database (1024 x 2048, 34.4 GB in NTT form):
         64 queries per batch on the tensor-core engine against the same
         queries one at a time, the tensor kernel's roofline, every response
         decoded.
  rns    the multi-modulus path: N = 4096 with two ciphertext primes on the
         "2^14 * 24KB = 384MB" preset (1.07 GB in NTT form), one query per
         call through the host API, with the multi-modulus CPU restatement
         timed beside it.

Inputs: the database is seeded entries ingested on the GPU; four seeded
PirClients (the CPU client library) make the Galois keys, RGSW keys and the
queries for seeded entries, and after the timed regions every response is
decoded by its client and compared with the database entry
(`entries_decoded`).  The NTT-form database (4.29 GB) is larger than L2
(129 MB), so no L2 flush is needed between steps.

--impl reference times the reference algorithm on the host cores (the
oracle port: the reference itself needs the absent SEAL fork) on the same
workload and prints its own JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "server queries/s and DB GB/s scanned, batched limb-TC vs plain GPU, bit-exact"
N = 2048
DB_SEED = 0xDB5EED
NUM_CLIENTS = 4


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="db262144")
    ap.add_argument("--cpu-queries", type=int, default=10,
                    help="timed queries of the CPU baseline (after 3 untimed ones, as tests.cpp:16)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the library's default choices (profiling runs: timings taken "
                         "under a profiler would make the autotuner's choices meaningless)")
    ap.add_argument("--batch", type=int, default=32,
                    help="batch size of the batched measurement (0 = skip)")
    ap.add_argument("--batch-steps", type=int, default=10)
    ap.add_argument("--micro", choices=["ntt", "tc"], default=None,
                    help="kernel micro-benchmark instead of the query benchmark (tc: the "
                         "tensor-core first dimension of --batch random leaf sets on "
                         "--workload's database, --steps calls; a profiling target)")
    ap.add_argument("--count", type=int, default=152 * 64, help="polynomials for --micro ntt")
    ap.add_argument("--serve-rate", type=float, default=1500.0,
                    help="offered queries/s of the serving measurement (0 = skip)")
    ap.add_argument("--serve-seconds", type=float, default=1.5)
    ap.add_argument("--serve", action="store_true",
                    help="serving benchmark alone: three resident databases (4096, 262,144 and "
                         "2,097,152 plaintexts), 512 clients under a key budget, Poisson arrivals")
    ap.add_argument("--serve-clients", type=int, default=512)
    ap.add_argument("--serve-light-rate", type=float, default=700.0,
                    help="--serve: a second leg at this offered rate, for latency below capacity")
    ap.add_argument("--large-workload", default="db2097152",
                    help="database of the large batched leg (2,097,152 plaintexts, 1024 x 2048)")
    ap.add_argument("--large-batch", type=int, default=64,
                    help="queries per batch of the large leg (0 = skip the leg)")
    ap.add_argument("--large-steps", type=int, default=4, help="timed batches of the large leg")
    ap.add_argument("--only-large", action="store_true",
                    help="run the large batched leg alone and print its object")
    ap.add_argument("--rns-workload", default="rns16384",
                    help="database of the multi-modulus leg (N = 4096, two ciphertext primes)")
    ap.add_argument("--rns-steps", type=int, default=20,
                    help="timed queries of the multi-modulus leg (0 = skip the leg)")
    ap.add_argument("--only-rns", action="store_true",
                    help="run the multi-modulus leg alone and print its object")
    ap.add_argument("--batch-sweep", default=None,
                    help="comma-separated batch sizes: queries/s of every first-dimension "
                         "engine at each size (one JSON line per size)")
    return ap.parse_args()


def aggregate_replicas(ms, steps, world, dist=None, device="cpu"):
    """Whole-job throughput of `world` replicas (one per GPU, no data-path
    collective): every rank's timed region is reduced to the slowest rank's,
    and the queries of all ranks count.  Returns (max ms, queries/s)."""
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, steps * world / (ms / 1e3)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_clients(params, count, seed=1, first=0):
    """Seeded PirClients `first` .. `first + count - 1` of one database shape
    (client c's secret seed is seed * 7919 + c, so the same client id has the
    same secret key on every database)."""
    from onionpirv2_gb300 import PirClient
    return [PirClient(params, c, secret_seed=seed * 7919 + c) for c in range(first, first + count)]


def client_keys(clients, seed=1, threads=1):
    """Every client's (Galois keys, RGSW key) on `threads` host threads."""
    from concurrent.futures import ThreadPoolExecutor

    def one(c):
        cid = c.get_client_id()
        return (c.create_galois_keys(seed=seed * 104729 + cid),
                c.generate_gsw_from_key(seed=seed * 130363 + cid))
    if threads <= 1:
        return [one(c) for c in clients]
    with ThreadPoolExecutor(threads) as ex:
        return list(ex.map(one, clients))


def make_queries(clients, owners, entries, seed=1):
    """Query j asks for entries[j] on behalf of clients[owners[j]]."""
    return np.stack([clients[int(o)].fast_generate_query(int(e), seed=seed * 1000003 + j)
                     for j, (o, e) in enumerate(zip(owners, entries))])


class Inputs:
    """NUM_CLIENTS seeded clients of one database, their keys, and `count`
    queries for seeded entries; query i belongs to client i % NUM_CLIENTS."""

    def __init__(self, params, count, seed=1):
        self.params = params
        self.clients = make_clients(params, NUM_CLIENTS, seed)
        t = time.perf_counter()
        self.keys = client_keys(self.clients, seed)
        self.keygen_s = (time.perf_counter() - t) / NUM_CLIENTS
        rng = np.random.default_rng(seed)
        self.entries = rng.integers(0, params.get_num_entries(), size=count)
        self.owners = np.arange(count) % NUM_CLIENTS
        t = time.perf_counter()
        self.queries = make_queries(self.clients, self.owners, self.entries, seed)
        self.query_s = (time.perf_counter() - t) / count


def decode_check(clients, owners, entries, packed, db_seed, entry_size, threads=1):
    """Decode every packed response with its client: (entries equal to the
    database's, lowest noise budget, seconds per decode)."""
    from concurrent.futures import ThreadPoolExecutor

    from onionpirv2_gb300 import synthetic_entries

    def one(j):
        e, budget = clients[int(owners[j])].decode_response(int(entries[j]), packed[j])
        ref = synthetic_entries(db_seed, int(entries[j]), 1, entry_size)[0]
        return bool(np.array_equal(e, ref)), budget
    t = time.perf_counter()
    if threads <= 1:
        res = [one(j) for j in range(len(packed))]
    else:
        with ThreadPoolExecutor(threads) as ex:
            res = list(ex.map(one, range(len(packed))))
    el = time.perf_counter() - t
    return (sum(ok for ok, _ in res), min((b for _, b in res), default=0),
            el / max(1, len(packed)))


class QuerySet:
    """Queries of one resident database: the clients that own them (same
    ids and secret keys as the registered ones), their entries and seed."""

    def __init__(self, params, db_id, db_seed, clients, owners, entries, seed, queries=None):
        self.params, self.db_id, self.db_seed = params, db_id, db_seed
        self.clients, self.owners, self.entries = clients, owners, entries
        self.queries = (make_queries(clients, owners, entries, seed) if queries is None
                        else queries)


def serve_leg(server, qsets, rate, seconds, seed=7, max_batch=32, lanes=2, max_wait_us=2000,
              check=8, threads=1):
    """Continuous batching under seeded Poisson arrivals: `rate` queries/s for
    `seconds`, uniform choice of database and of query within it.  Returns the
    server's counters and latency percentiles, the arrival count, whether the
    first `check` responses equal the synchronous path's bit for bit, and how
    many responses the clients decoded to the database entry."""
    rng = np.random.default_rng(seed)
    n = max(1, int(rate * seconds))
    gaps = rng.exponential(1.0 / rate, size=n)
    pick_db = rng.integers(0, len(qsets), size=n)
    pick_q = np.array([rng.integers(0, qsets[d].queries.shape[0]) for d in pick_db])
    server.serve_start(max_batch=max_batch, lanes=lanes, max_wait_us=max_wait_us)
    tickets = []
    t = time.perf_counter()
    for j in range(n):
        t += gaps[j]
        while True:
            d = t - time.perf_counter()
            if d <= 0:
                break
            if d > 6e-4:
                time.sleep(d - 4e-4)
        qs, k = qsets[pick_db[j]], pick_q[j]
        tickets.append(server.submit(int(qs.owners[k]), qs.queries[k], db_id=qs.db_id))
    resps = [server.wait(tk, 600000) for tk in tickets]
    stats = server.serve_stats()
    server.serve_stop()
    same = all(np.array_equal(resps[j], server.make_query(
        int(qsets[pick_db[j]].owners[pick_q[j]]), qsets[pick_db[j]].queries[pick_q[j]],
        db_id=qsets[pick_db[j]].db_id)) for j in range(min(check, n)))
    ok = 0
    for d, qs in enumerate(qsets):
        sel = [j for j in range(n) if pick_db[j] == d]
        if sel:
            ok += decode_check(qs.clients, qs.owners[pick_q[sel]], qs.entries[pick_q[sel]],
                               [resps[j].packed for j in sel], qs.db_seed,
                               qs.params.get_entry_size(), threads)[0]
    return stats, n, same, ok


def tensor_engine(limb_bits):
    return ("tensor (tcgen05, 8-bit database limbs x %d-bit query limbs in bf16, exact)"
            % limb_bits)


def tensor_roofline(params, B, ms, workload, limb_bits=9):
    """Roofline of tc_scan_kernel: algorithmic bf16 flops of the limb GEMM
    (8 database limbs x 7 query limbs of 9 bits = 56 limb products, or 64
    with 8-bit query limbs, of 2 flops per 60x60-bit MAC; N * n_rest * n1 *
    2B MACs) over the kernel's time, against the measured burst bf16 peak
    (the kernel is timed per launch, not over a seconds-long loop)."""
    n1, nrest = params.get_fst_dim_sz(), params.get_other_dim_sz()
    products = 8 * (7 if limb_bits == 9 else 8)
    flops = 2.0 * products * nrest * 2 * B * n1 * N
    peak, kind = measured_peak("bf16_tflops")
    ach = flops / (ms / 1e3) / 1e12
    return {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
            "frac": ach / peak, "traffic": read_traffic(f"{workload}_b{B}", "tc_scan_kernel"),
            "kernel": "tc_scan_kernel (first dimension of the batch)",
            "limb_products_per_mac": products,
            "flops_per_step": flops, "kernel_ms": ms,
            "peak_source": f"{kind} bf16_tflops (burst)"}


def large_leg(args, local, clocks=None):
    """The 2,097,152-plaintext database (1024 x 2048: 34.4 GB in NTT form,
    68.7 GB of tensor-engine limbs), B queries per batch on the tensor engine,
    and the same queries one at a time.  Every response is decoded by its
    client; the batch must equal the single queries bit for bit."""
    import torch
    from onionpirv2_gb300 import PirParams, PirServer
    params = PirParams.preset(args.large_workload)
    B = args.large_batch
    dev = f"cuda:{local}"
    server = PirServer(params, device=local)
    stream = torch.cuda.Stream(device=local)
    server.set_stream(stream.cuda_stream)
    seed = DB_SEED + 2
    t = time.perf_counter()
    server.gen_data(seed)
    ingest_s = time.perf_counter() - t
    inp = Inputs(params, 2 * B, seed=3)
    for cid, (gk, gsw) in enumerate(inp.keys):
        server.set_client_galois_key(cid, gk)
        server.set_client_gsw_key(cid, gsw)
    nq = 2 * B
    qbytes, rb = 2 * N * 8, server.resp_bytes
    dq = torch.from_numpy(inp.queries.view(np.int64)).to(dev)
    dresp = torch.empty((nq, 2, N), dtype=torch.int64, device=dev)
    dpack = torch.empty((nq, rb), dtype=torch.uint8, device=dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def one(i):
        server.make_query_device([i % NUM_CLIENTS], dq.data_ptr() + i * qbytes,
                                 dresp.data_ptr() + i * qbytes, dpack.data_ptr() + i * rb)

    def batch(k):  # batch k holds queries [k B, (k + 1) B)
        ids = [(k * B + j) % NUM_CLIENTS for j in range(B)]
        server.make_query_device(ids, dq.data_ptr() + k * B * qbytes,
                                 dresp.data_ptr() + k * B * qbytes, dpack.data_ptr() + k * B * rb)

    with torch.cuda.stream(stream):
        # single queries: every query once (the first B are the batch's reference)
        for i in range(3):
            one(i)
        stream.synchronize()
        e0, e1 = ev(), ev()
        e0.record(stream)
        for i in range(nq):
            one(i)
        e1.record(stream)
        e1.synchronize()
        single_ms = e0.elapsed_time(e1) / nq
        single = dresp.cpu().numpy().view(np.uint64).reshape(nq, -1).copy()
        server.set_batch_engine("tensor")
        batch(0)  # builds the limb plane
        batch(1)
        stream.synchronize()
        t1 = time.time()
        e0.record(stream)
        for k in range(args.large_steps):
            batch(k % 2)
        e1.record(stream)
        e1.synchronize()
        t2 = time.time()
        bms = e0.elapsed_time(e1) / args.large_steps
        server.set_timing(True)
        st = []
        for k in range(2):
            batch(k)
            stream.synchronize()
            st.append(server.stage_times())
        server.set_timing(False)
        server.set_batch_engine("auto")
    got = dresp.cpu().numpy().view(np.uint64).reshape(nq, -1)
    same = bool(np.array_equal(got, single))
    decoded, budget, _ = decode_check(inp.clients, inp.owners[:nq], inp.entries[:nq],
                                      dpack.cpu().numpy(), seed, params.get_entry_size(),
                                      threads=os.cpu_count() or 1)
    stages = {k: statistics.mean(x[k] for x in st) for k in st[0]}
    db_bytes = params.get_num_pt() * N * 8
    out = {
        "workload": args.large_workload, "db_plaintexts": params.get_num_pt(),
        "n1": params.get_fst_dim_sz(), "n_rest": params.get_other_dim_sz(),
        "ndim": len(params.get_dims()), "ntt_db_bytes": db_bytes, "batch": B,
        "engine": tensor_engine(9),
        "value": B / (bms / 1e3), "unit": "queries/s", "ms_per_batch": bms,
        "steps": args.large_steps, "stages_ms": stages,
        "single_query": {"value": 1e3 / single_ms, "unit": "queries/s", "ms_per_query": single_ms,
                         "queries": nq},
        "speedup_vs_single": single_ms * B / bms,
        "roofline": tensor_roofline(params, B, stages["scan_kernel"], args.large_workload),
        "matches_single_query_responses": same,
        "entries_decoded": f"{decoded}/{nq}", "min_noise_budget": budget,
        "ingest_s": ingest_s,
        "l2": f"inputs larger than L2 (NTT-form database {db_bytes / 1e9:.1f} GB > 129 MB)",
    }
    if clocks is not None:
        out["clocks"] = clocks.summary(t1, t2)
    server.close()
    return out


def rns_inputs(params, count, seed=11):
    """Seeded synthetic client material of a multi-modulus database: Galois
    keys [h][R][2][R+1][N], RGSW rows [2 l_key][2][R][N] and `count` queries
    [2][R][N] of uniform residues (the server's work does not depend on the
    values; the parity tests check real keys and queries against the oracle)."""
    rng = np.random.default_rng(seed)
    n, R = params.poly_degree, params.get_rns_mod_cnt()
    qs = params.get_coeff_modulus()
    mods = np.array(qs + [params.coeff_modulus[-1]], dtype=np.uint64)
    h = params.get_expan_height()
    gk = rng.integers(0, 2**62, size=(h, R, 2, R + 1, n), dtype=np.uint64) % mods[None, None, None, :, None]
    data = np.array(qs, dtype=np.uint64)[None, None, :, None]
    gsw = rng.integers(0, 2**62, size=(2 * params.get_l_key(), 2, R, n), dtype=np.uint64) % data
    queries = rng.integers(0, 2**62, size=(count, 2, R, n), dtype=np.uint64) % data
    return gk, gsw, queries


def rns_leg(args, local, clocks=None, cpu=True):
    """The multi-modulus path (N = 4096, two ciphertext primes; the
    "2^14 * 24KB = 384MB" preset of database_constants.h) through the public
    host API: one query per step, host buffers, stage times, the scan
    kernel's HBM roofline, and the multi-modulus CPU restatement of the
    reference timed on the host cores beside it."""
    from onionpirv2_gb300 import PirParams, PirServer
    params = PirParams.preset(args.rns_workload)
    server = PirServer(params, device=local)
    t = time.perf_counter()
    server.gen_data(DB_SEED + 3)
    ingest_s = time.perf_counter() - t
    steps = args.rns_steps
    gk, gsw, queries = rns_inputs(params, steps + 3)
    server.set_client_galois_key(0, gk)
    server.set_client_gsw_key(0, gsw)
    for i in range(3):
        server.make_query(0, queries[i])
    t1 = time.time()
    t = time.perf_counter()
    for i in range(steps):
        server.make_query(0, queries[3 + i])
    el = time.perf_counter() - t
    t2 = time.time()
    server.set_timing(True)
    st = []
    for i in range(5):
        server.make_query(0, queries[i])
        st.append(server.stage_times())
    server.set_timing(False)
    stages = {k: statistics.mean(x[k] for x in st) for k in st[0]}
    # batches: the queries spread over the path's concurrent lanes
    B = 32
    bq = np.stack([queries[(3 + i) % len(queries)] for i in range(B)])
    server.make_query_batch([0] * B, bq)
    reps = max(1, steps // B)
    t = time.perf_counter()
    for _ in range(reps):
        bresp, _ = server.make_query_batch([0] * B, bq)
    bel = time.perf_counter() - t
    same = all(np.array_equal(bresp[j], server.make_query(0, bq[j])) for j in (0, B // 2, B - 1))
    server.close()
    R, n = params.get_rns_mod_cnt(), params.poly_degree
    db_bytes = params.get_num_pt() * n * R * 8
    peak, kind = measured_peak()
    ach = db_bytes / (stages["scan_kernel"] / 1e3) / 1e9
    out = {
        "workload": args.rns_workload, "poly_degree": n, "ciphertext_primes": R,
        "db_plaintexts": params.get_num_pt(), "n1": params.get_fst_dim_sz(),
        "n_rest": params.get_other_dim_sz(), "ndim": len(params.get_dims()),
        "entry_size": params.get_entry_size(), "raw_db_mb": params.get_DBSize_MB(),
        "ntt_db_bytes": db_bytes,
        "value": steps / el, "unit": "queries/s", "ms_per_query": el / steps * 1e3,
        "timing": "wall clock around blocking opir_make_query calls (host query in, "
                  "response and packed bytes out)",
        "stages_ms": stages,
        "batched": {"value": B * reps / bel, "unit": "queries/s", "batch": B, "batches": reps,
                    "what": "opir_make_query_batch, host buffers; queries on concurrent lanes",
                    "matches_single_query_responses": bool(same)},
        "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": ach / peak,
                     "traffic": read_traffic(args.rns_workload, "scan_bulk_kernel"),
                     "kernel": "scan_bulk_kernel (first dimension, both primes in one launch)",
                     "peak_source": f"{kind} hbm_gbs"},
        "inputs": "seeded uniform residues as keys and queries (value-independent work; "
                  "bit-exactness against the oracle is the -m gpu tests' job)",
        "ingest_s": ingest_s,
    }
    if clocks is not None:
        out["clocks"] = clocks.summary(t1, t2)
    if cpu:
        from oracle import oracle as orc
        orc.build()
        threads = os.cpu_count() or 1
        orc.set_threads(threads)
        P = params
        o = orc.RnsOracle(P.poly_degree, P.num_entries, P.max_fst_dim, l=P.gsw_l,
                          l_key=P.gsw_l_key, plain_bits=P.plain_mod_bits,
                          small_q_width=P.small_q_width, coeff_bits=tuple(P.coeff_mods))
        db = o.build_db(DB_SEED + 3)
        gsn = o.gsw_to_ntt(gsw)
        o.make_query_server(db, gk, gsn, queries[0])
        nq = 3
        t = time.perf_counter()
        for i in range(nq):
            o.make_query_server(db, gk, gsn, queries[1 + i])
        cpu_s = (time.perf_counter() - t) / nq
        out["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": "queries/s", "cores": threads,
                               "kind": "port",
                               "sample": f"{nq} full queries after 1 untimed on the same database "
                                         f"and inputs, {threads} threads (multi-modulus CPU "
                                         "restatement of the reference server)",
                               "cpu": host_cpu_model()}
        del db
    return out


def rns_main(args):
    """The multi-modulus leg alone (one JSON object)."""
    import torch
    _, _, local = dist_env()
    torch.cuda.set_device(local)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.5)
    out = rns_leg(args, local, clocks, cpu=not args.no_cpu_baseline)
    clocks.stop()
    print(json.dumps(out), flush=True)
    return 0


def large_main(args):
    """The large batched leg alone (one JSON object)."""
    import torch
    _, _, local = dist_env()
    torch.cuda.set_device(local)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.5)
    out = large_leg(args, local, clocks)
    clocks.stop()
    print(json.dumps(out), flush=True)
    return 0


def sweep_main(args):
    """Queries/s of the scan, integer-GEMM and tensor-core engines per batch size."""
    import torch
    from onionpirv2_gb300 import PirParams, PirServer
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    params = PirParams.preset(args.workload)
    server = PirServer(params, device=local)
    stream = torch.cuda.Stream(device=local)
    server.set_stream(stream.cuda_stream)
    server.gen_data(DB_SEED)
    sizes = [int(x) for x in args.batch_sweep.split(",")]
    inp = Inputs(params, max(sizes) * 4)
    clients, queries = inp.keys, inp.queries
    for cid, (gk, gsw) in enumerate(clients):
        server.set_client_galois_key(cid, gk)
        server.set_client_gsw_key(cid, gsw)
    dq = torch.from_numpy(queries.view(np.int64)).to(f"cuda:{local}")
    nq = queries.shape[0]
    dresp = torch.empty((nq, 2, N), dtype=torch.int64, device=f"cuda:{local}")
    dpack = torch.empty((nq, server.resp_bytes), dtype=torch.uint8, device=f"cuda:{local}")
    qbytes = 2 * N * 8
    for B in sizes:
        line = {"workload": args.workload, "batch": B, "unit": "queries/s"}
        for engine in ("scan", "imad", "tensor"):
            server.set_batch_engine(engine)

            def bstep(i):
                off = (i % 4) * B
                ids = [(off + j) % NUM_CLIENTS for j in range(B)]
                server.make_query_device(ids, dq.data_ptr() + off * qbytes,
                                         dresp.data_ptr() + off * qbytes,
                                         dpack.data_ptr() + off * server.resp_bytes)

            with torch.cuda.stream(stream):
                for i in range(3):
                    bstep(i)
                stream.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                steps = max(3, min(20, 256 // B))
                e0.record(stream)
                for i in range(steps):
                    bstep(i)
                e1.record(stream)
                e1.synchronize()
            line[engine] = B * steps / (e0.elapsed_time(e1) / 1e3)
        print(json.dumps(line), flush=True)
    server.close()
    return 0


def serve_main(args):
    """Serving benchmark: three resident databases, 512 clients, Poisson arrivals."""
    import torch
    from onionpirv2_gb300 import PirParams, PirServer
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    names = ["db4096", "db262144", "db2097152"]
    params = [PirParams.preset(w) for w in names]
    server = PirServer(params[1], device=local)
    t0 = time.perf_counter()
    server.gen_data(DB_SEED)
    dbs = [server.add_database(params[0], seed=DB_SEED + 1), server.db_id,
           server.add_database(params[2], seed=DB_SEED + 2)]
    ingest_s = time.perf_counter() - t0
    # per-database tuning: scan tiles and the engine per batch size
    t = time.perf_counter()
    tuned = {names[d]: server.autotune(max_batch=32, db_id=dbs[d]) for d in range(3)}
    tune_s = time.perf_counter() - t
    per = server.key_bytes_per_client()
    slots = max(2, args.serve_clients // 2)
    server.set_key_budget(slots * per)  # half the clients' keys fit: LRU admission
    # the clients: keys made on the host cores with the product PirClient
    # (Galois keys for the deepest database serve the shallower ones too)
    threads = os.cpu_count() or 1
    deepest = max(range(3), key=lambda d: params[d].get_expan_height())
    t = time.perf_counter()
    keyed = make_clients(params[deepest], args.serve_clients)
    keys = client_keys(keyed, threads=threads)
    keygen_s = time.perf_counter() - t
    for c, (gk, gsw) in zip(keyed, keys):
        server.set_client_galois_key(c.get_client_id(), gk)
        server.set_client_gsw_key(c.get_client_id(), gsw)
    rng = np.random.default_rng(3)
    qsets = []
    t = time.perf_counter()
    for d in range(3):
        cl = keyed if d == deepest else make_clients(params[d], args.serve_clients)
        owners = rng.integers(0, args.serve_clients, size=256)
        entries = rng.integers(0, params[d].get_num_entries(), size=256)
        qsets.append(QuerySet(params[d], dbs[d], DB_SEED + (1, 0, 2)[d], cl, owners, entries,
                              seed=20 + d))
    query_s = (time.perf_counter() - t) / (3 * 256)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.5)
    # warm-up: limb planes, workspaces and first-touch costs
    serve_leg(server, qsets, 200.0, 0.2, seed=1, check=0, threads=threads)
    t1 = time.time()
    stats, n, same, decoded = serve_leg(server, qsets, args.serve_rate, args.serve_seconds,
                                        seed=11, threads=threads)
    t2 = time.time()
    light = None
    if args.serve_light_rate > 0:
        lstats, ln, lsame, ldecoded = serve_leg(server, qsets, args.serve_light_rate,
                                                args.serve_seconds, seed=12, threads=threads)
        light = {"offered_qps": args.serve_light_rate, "arrivals": ln,
                 "queries_per_s": lstats["queries_per_s"], "p50_ms": lstats["p50_ms"],
                 "p99_ms": lstats["p99_ms"], "mean_batch": lstats["mean_batch"],
                 "failed": lstats["failed"], "bit_exact_sample": lsame,
                 "entries_decoded": f"{ldecoded}/{ln}"}
    clocks.stop()
    resident, nslots = server.resident_clients()
    line = {
        "metric": "server queries/s under Poisson arrivals (continuous batching, 3 resident DBs)",
        "value": stats["queries_per_s"], "unit": "queries/s", "n_gpus": 1,
        "steps": n, "warmup": 40, "ms_per_step": 1e3 / max(stats["queries_per_s"], 1e-9),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic",
        "config": {"workload": "serving: db4096 + db262144 + db2097152 resident",
                   "clients": args.serve_clients, "key_slots": nslots,
                   "offered_qps": args.serve_rate, "seconds": args.serve_seconds,
                   "arrivals": "seeded Poisson, uniform database and query (256 client "
                               "queries per database, owners uniform over the clients)",
                   "max_batch": 32, "lanes": 2, "max_wait_us": 2000},
        "p50_ms": stats["p50_ms"], "p99_ms": stats["p99_ms"], "mean_ms": stats["mean_ms"],
        "max_ms": stats["max_ms"], "completed": stats["completed"], "failed": stats["failed"],
        "batches": stats["batches"], "mean_batch": stats["mean_batch"],
        "resident_clients": resident, "bit_exact_sample": same, "ingest_s": ingest_s,
        "entries_decoded": f"{decoded}/{n}",
        "light_load": light,
        "autotune": {"seconds": tune_s,
                     **{w: {b["batch"]: b["engine"] for b in t["batches"]}
                        for w, t in tuned.items()}},
        "client": {"threads": threads, "clients": args.serve_clients,
                   "keygen_s": keygen_s,
                   "keys_per_s": args.serve_clients / keygen_s,
                   "key_bytes_per_client": int(sum(a.nbytes for a in keys[0])),
                   "query_ms": query_s * 1e3,
                   "what": "PirClient (CPU): Galois keys + RGSW(sk) per client, one "
                           "query per ms figure; every served response decoded"},
        "clocks": clocks.summary(t1, t2),
    }
    print(json.dumps(line), flush=True)
    server.close()
    return 0


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.samples.append((time.time(), parts))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0, t1):
        sel = [s for t, s in self.samples if t0 - 0.25 <= t <= t1 + 0.25] or \
              [s for _, s in self.samples]
        if not sel:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(s[0]) for s in sel if num(s[0]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in sel for i in range(4) if s[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": num(sel[0][1]), "reasons": reasons, "samples": len(sel)}


def read_traffic(workload, kernel="scan_kernel"):
    """DRAM bytes of `kernel` per launch -- or per batch, where a batch is
    several launches -- from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    try:
        with open(path) as f:
            for line in f:
                if line.strip().startswith(("traffic_bytes_per_launch:",
                                            "traffic_bytes_per_batch:")):
                    return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def measured_peak(key="hbm_gbs"):
    """Measured peak (HBM GB/s, or bf16 TFLOP/s) of this GPU pool."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    fallback = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}
    try:
        with open(path) as f:
            return float(json.load(f)[key]), "measured"
    except (OSError, KeyError, ValueError):
        return fallback[key], "fallback"


def cpu_baseline(params, workload, clients, queries, gpu_resps, nq):
    """Time the oracle (CPU restatement of the reference server) on full
    queries with all host threads; check its responses against the GPU's."""
    from oracle import oracle as orc
    orc.build()
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    o = orc.Oracle(params.num_entries, params.max_fst_dim)
    t = time.perf_counter()
    db = o.build_db(DB_SEED)
    build_s = time.perf_counter() - t
    times, match = [], True
    nq = max(1, min(nq, len(queries)))
    gsw_ntt = [o.gsw_key_to_ntt(c[1]) for c in clients]
    for i in range(3):  # warm-up (EXPERIMENT_ITERATIONS = 10 timed + 3)
        j = i % len(queries)
        o.make_query_server(db, clients[j % NUM_CLIENTS][0], gsw_ntt[j % NUM_CLIENTS], queries[j])
    for i in range(nq):
        gk = clients[i % NUM_CLIENTS][0]
        t = time.perf_counter()
        resp, packed, stages, wraps = o.make_query_server(db, gk, gsw_ntt[i % NUM_CLIENTS], queries[i])
        times.append(time.perf_counter() - t)
        if gpu_resps is not None and i < len(gpu_resps):
            match &= bool(np.array_equal(resp, gpu_resps[i]))
    # the reference itself is single-threaded: one more query on one thread
    orc.set_threads(1)
    gk = clients[0][0]
    t = time.perf_counter()
    resp1, _, _, _ = o.make_query_server(db, gk, gsw_ntt[0], queries[0])
    one_s = time.perf_counter() - t
    orc.set_threads(threads)
    if gpu_resps is not None and len(gpu_resps):
        match &= bool(np.array_equal(resp1, gpu_resps[0]))
    del db
    qps = nq / sum(times)
    return {
        "value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
        "sample": (f"{nq} full queries (all stages) after 3 untimed on the {workload} "
                   f"database ({params.get_num_pt()} plaintexts), {threads} threads; "
                   f"database build {build_s:.1f} s untimed; first dimension: the "
                   "mat_mat_128 loop nest with exact sums (orc_first_dim)"),
        "single_thread_value": 1.0 / one_s,
        "cpu": host_cpu_model(),
    }, match


def host_cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from onionpirv2_gb300.params import PirParams
    from oracle import oracle as orc
    orc.build()
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    params = PirParams.preset(args.workload)
    o = orc.Oracle(params.num_entries, params.max_fst_dim)
    db = o.build_db(DB_SEED)
    # a bounded sample: at most 200 timed queries (about 20 s on 16 cores) and
    # 3 warm-up queries, so the arm ends within minutes whatever K and W are
    steps, warm = min(args.steps, 200), min(args.warmup, 3)
    # the inputs of the GPU arm (same seeds), made by the oracle's own client
    sks = [o.keygen(7919 + c) for c in range(NUM_CLIENTS)]
    clients = [(o.galois_keys(sks[c], 104729 + c), o.gsw_key(sks[c], 130363 + c))
               for c in range(NUM_CLIENTS)]
    entries = np.random.default_rng(1).integers(0, params.get_num_entries(), size=warm + steps)
    queries = [o.make_query(sks[j % NUM_CLIENTS], 1000003 + j, int(e)) for j, e in enumerate(entries)]
    gsw_ntt = [o.gsw_key_to_ntt(c[1]) for c in clients]
    for i in range(warm):
        o.make_query_server(db, clients[i % NUM_CLIENTS][0], gsw_ntt[i % NUM_CLIENTS], queries[i])
    t = time.perf_counter()
    for i in range(warm, warm + steps):
        o.make_query_server(db, clients[i % NUM_CLIENTS][0], gsw_ntt[i % NUM_CLIENTS], queries[i])
    el = time.perf_counter() - t
    qps = steps / el
    db_bytes = params.get_num_pt() * N * 8
    line = {
        "impl": "reference", "metric": METRIC, "value": qps, "unit": "queries/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": args.workload, "db_plaintexts": params.get_num_pt(),
                   "n1": params.get_fst_dim_sz(), "n_rest": params.get_other_dim_sz(),
                   "batch": 1, "ntt_db_bytes": db_bytes},
        "db_gbs_scanned": db_bytes * qps / 1e9,
        "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": f"{steps} full queries after {warm} warm-up, "
                                   f"{threads} threads (CPU restatement of the reference "
                                   "server; the reference needs the absent SEAL fork)",
                         "cpu": host_cpu_model()},
        "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_micro_ntt(args):
    """Throughput of the batched 2048-point NTT kernel (device buffers)."""
    import ctypes

    import torch
    from onionpirv2_gb300 import PirParams, PirServer, _capi
    L = _capi.load()
    server = PirServer(PirParams.preset("db4096"))
    stream = torch.cuda.Stream()
    server.set_stream(stream.cuda_stream)
    q = server.pir_params.coeff_modulus[0]
    x = torch.randint(0, 2**62, (args.count, N), dtype=torch.int64, device="cuda") % q
    torch.cuda.synchronize()
    out = {"micro": "ntt", "count": args.count}
    for inv in (0, 1):
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                L.opir_ntt_device(server.ctx, 0, inv, ctypes.c_void_p(x.data_ptr()), args.count)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                L.opir_ntt_device(server.ctx, 0, inv, ctypes.c_void_p(x.data_ptr()), args.count)
            e1.record(stream)
            e1.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        out["inverse" if inv else "forward"] = {"us": ms * 1e3, "ntt_per_us": args.count / (ms * 1e3)}
    print(json.dumps(out), flush=True)
    return 0


def run_micro_tc(args):
    """The tensor-core first dimension alone (query transform, limb split,
    tc_scan_kernel) of args.batch random leaf sets on the workload's database,
    through the first-dimension hook: args.warmup + args.steps calls, host
    leaves in and results out on every call.  For kernel profiles."""
    import ctypes

    from onionpirv2_gb300 import PirParams, PirServer, _capi
    P = PirParams.preset(args.workload)
    n1, nr, B = P.get_fst_dim_sz(), P.get_other_dim_sz(), max(2, args.batch)
    server = PirServer(P)
    server.gen_data(DB_SEED)
    server.set_batch_engine("tensor")
    leaves = np.random.default_rng(1).integers(0, P.coeff_modulus[0], size=(B, n1, 2, N),
                                               dtype=np.uint64)
    out = np.zeros((B, nr, 2, N), np.uint64)
    p64 = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))

    def call():
        _capi.check(server.ctx, server._L.opir_debug_first_dim(server.ctx, server.db_id, B,
                                                                p64(leaves), p64(out)))
    for _ in range(args.warmup):
        call()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        call()
    wall = (time.perf_counter() - t0) / max(1, args.steps)
    server.close()
    print(json.dumps({"micro": "tc", "workload": args.workload, "batch": B, "n1": n1,
                      "n_rest": nr, "calls": args.steps,
                      "wall_ms_per_call": wall * 1e3,
                      "what": "host leaves in, first dimension out (coefficient form)"}),
          flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.micro == "ntt":
        return run_micro_ntt(args)
    if args.micro == "tc":
        return run_micro_tc(args)
    if args.serve:
        return serve_main(args)
    if args.batch_sweep:
        return sweep_main(args)
    if args.only_large:
        return large_main(args)
    if args.only_rns:
        return rns_main(args)
    rank, world, local = dist_env()
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist
    from onionpirv2_gb300 import PirParams, PirServer

    params = PirParams.preset(args.workload)
    server = PirServer(params, device=local)
    stream = torch.cuda.Stream(device=local)
    server.set_stream(stream.cuda_stream)
    t_ingest = time.perf_counter()
    server.gen_data(DB_SEED)
    ingest_s = time.perf_counter() - t_ingest
    total = args.warmup + args.steps
    nbatchq = args.batch * (args.batch_steps + 3) if args.batch > 1 else 0
    inp = Inputs(params, max(total, nbatchq))
    clients, queries = inp.keys, inp.queries
    for cid, (gk, gsw) in enumerate(clients):
        server.set_client_galois_key(cid, gk)
        server.set_client_gsw_key(cid, gsw)
    # the autotuner picks the scan tile configuration and the engine per batch
    # size for this database on this GPU (untimed; all choices are bit-exact)
    t_tune = time.perf_counter()
    tune = None if args.no_autotune else server.autotune(max_batch=max(2, args.batch))
    tune_s = time.perf_counter() - t_tune
    rb = server.resp_bytes
    nq = queries.shape[0]
    dq = torch.from_numpy(queries.view(np.int64)).to(f"cuda:{local}")
    dresp = torch.empty((nq, 2, N), dtype=torch.int64, device=f"cuda:{local}")
    dpack = torch.empty((nq, rb), dtype=torch.uint8, device=f"cuda:{local}")
    torch.cuda.synchronize()
    qbytes = 2 * N * 8

    def step(i):
        server.make_query_device([i % NUM_CLIENTS], dq.data_ptr() + i * qbytes,
                                 dresp.data_ptr() + i * qbytes, dpack.data_ptr() + i * rb)

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.5)
    # ---- value: device-resident inputs, CUDA events on the library stream
    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            step(i)
        stream.synchronize()
        if pg:
            pg.barrier()
        torch.cuda.synchronize()
        l0 = server.launch_count()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.time()
        ev0.record(stream)
        for i in range(args.warmup, total):
            step(i)
        ev1.record(stream)
        ev1.synchronize()
        t1 = time.time()
        torch.cuda.synchronize()
    launches = server.launch_count() - l0
    ms, qps = aggregate_replicas(ev0.elapsed_time(ev1), args.steps, world, pg, f"cuda:{local}")
    gpu_resps = dresp[: args.cpu_queries].cpu().numpy().view(np.uint64)

    # ---- roofline pass: per-stage CUDA events inside the library
    server.set_timing(True)
    kt = min(args.steps, 50)
    stages = []
    with torch.cuda.stream(stream):
        for i in range(kt):
            step(args.warmup + i)
            stream.synchronize()
            stages.append(server.stage_times())
    server.set_timing(False)
    mean = {k: statistics.mean(s[k] for s in stages) for k in stages[0]}

    # ---- e2e: public host API, host buffers, copies inside the region
    e2e_steps = min(args.steps, 100)
    with torch.cuda.stream(stream):
        for i in range(min(args.warmup, 5)):
            server.make_query(i % NUM_CLIENTS, queries[i])
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(e2e_steps):
            r = server.make_query(i % NUM_CLIENTS, queries[i % total])
        e1.record(stream)
        e1.synchronize()
    e2e_ms = e0.elapsed_time(e1)

    # ---- batched: B queries per step share one pass over the database,
    # on both first-dimension engines (bf16-limb tensor cores, integer IMAD)
    batched = None
    if args.batch > 1:
        B = args.batch

        def bstep(i):
            ids = [(i * B + j) % NUM_CLIENTS for j in range(B)]
            server.make_query_device(ids, dq.data_ptr() + i * B * qbytes,
                                     dresp.data_ptr() + i * B * qbytes, dpack.data_ptr() + i * B * rb)

        def run_batched(engine):
            server.set_batch_engine(engine)
            with torch.cuda.stream(stream):
                for i in range(3):
                    bstep(i)
                stream.synchronize()
                b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                b0.record(stream)
                for i in range(args.batch_steps):
                    bstep(i % (args.batch_steps + 3))
                b1.record(stream)
                b1.synchronize()
                bms = b0.elapsed_time(b1) / args.batch_steps
                server.set_timing(True)
                bst = []
                for i in range(min(args.batch_steps, 5)):
                    bstep(i)
                    stream.synchronize()
                    bst.append(server.stage_times())
                server.set_timing(False)
            # bit-exact against the single-query responses of the same queries
            same = bool(np.array_equal(dresp[:B].cpu().numpy().view(np.uint64).reshape(B, -1),
                                       single_resps[:B]))
            server.set_batch_engine("auto")
            return {"value": B * world / (bms / 1e3), "unit": "queries/s", "ms_per_batch": bms,
                    "stages_ms": {k: statistics.mean(x[k] for x in bst) for k in bst[0]},
                    "matches_single_query_responses": same}

        # responses of the first B queries through the single-query path
        with torch.cuda.stream(stream):
            for i in range(B):
                server.make_query_device([i % NUM_CLIENTS], dq.data_ptr() + i * qbytes,
                                         dresp.data_ptr() + i * qbytes, dpack.data_ptr() + i * rb)
            stream.synchronize()
        single_resps = dresp[:B].cpu().numpy().view(np.uint64).reshape(B, -1).copy()
        tensor = run_batched("tensor")
        imad = run_batched("imad")
        # tensor-core kernel roofline (limb-GEMM flops / kernel time, burst peak)
        bits = (tune or {}).get("tc_limbs_choice") or 9  # the tuned width (9 bits for full passes)
        batched = dict(tensor, batch=B, engine=tensor_engine(bits),
                       speedup_vs_single=tensor["value"] / qps,
                       roofline=tensor_roofline(params, B, tensor["stages_ms"]["scan_kernel"],
                                                args.workload, bits),
                       imad=dict(imad, engine="integer multiply-add GEMM"))
    # ---- client side: every response of the timed queries (rewritten by
    # the batched passes, which equal them) decodes to its database entry
    decoded, min_budget, decode_s = decode_check(
        inp.clients, inp.owners[:total], inp.entries[:total], dpack[:total].cpu().numpy(),
        DB_SEED, params.get_entry_size())
    # ---- serving: continuous batching under Poisson arrivals over this
    # database and a small second one (the full three-database run: --serve)
    serving = None
    if args.serve_rate > 0 and world == 1:
        from onionpirv2_gb300 import PirParams as _PP
        sp = _PP.preset("db4096")
        small = server.add_database(sp, seed=DB_SEED + 1)
        qsets = [QuerySet(params, server.db_id, DB_SEED, inp.clients, inp.owners, inp.entries,
                          0, queries=inp.queries),
                 QuerySet(sp, small, DB_SEED + 1, make_clients(sp, NUM_CLIENTS),
                          np.arange(256) % NUM_CLIENTS,
                          np.random.default_rng(5).integers(0, sp.get_num_entries(), size=256), 6)]
        sstats, sn, ssame, sok = serve_leg(server, qsets, args.serve_rate, args.serve_seconds,
                                           threads=os.cpu_count() or 1)
        serving = {"databases": [args.workload, "db4096"], "offered_qps": args.serve_rate,
                   "arrivals": sn, "queries_per_s": sstats["queries_per_s"],
                   "p50_ms": sstats["p50_ms"], "p99_ms": sstats["p99_ms"],
                   "mean_batch": sstats["mean_batch"], "batches": sstats["batches"],
                   "failed": sstats["failed"], "bit_exact_sample": ssame,
                   "entries_decoded": f"{sok}/{sn}",
                   "policy": "max_batch 32, 2 lanes, max_wait 2 ms"}
    e2e_qps = e2e_steps * world / (e2e_ms / 1e3)
    # ---- large: the 2,097,152-plaintext database, batches on the tensor
    # engine (this database's device memory released first)
    server.close()
    large = None
    if args.large_batch > 1 and world == 1:
        large = large_leg(args, local, clocks)
    # ---- rns: the multi-modulus path (N = 4096, two ciphertext primes)
    rns = None
    if args.rns_steps > 0 and world == 1:
        rns = rns_leg(args, local, clocks, cpu=rank == 0 and not args.no_cpu_baseline)
    clocks.stop()

    db_bytes = db_bytes_cfg = params.get_num_pt() * N * 8
    peak, peak_kind = measured_peak()
    achieved = db_bytes / (mean["scan_kernel"] / 1e3) / 1e9
    traffic = read_traffic(args.workload)
    line = {
        "metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic",
        "config": {"workload": args.workload, "db_plaintexts": params.get_num_pt(),
                   "n1": params.get_fst_dim_sz(), "n_rest": params.get_other_dim_sz(),
                   "ndim": len(params.get_dims()), "batch": 1, "ntt_db_bytes": db_bytes,
                   "raw_db_mb": params.get_DBSize_MB(), "parallelism": f"replicas{world}",
                   "l2": (f"inputs larger than L2 (NTT-form database {db_bytes_cfg / 1e9:.2f} GB "
                          "> 129 MB)")},
        "db_gbs_scanned": db_bytes * qps / 1e9,
        "raw_db_mbs": params.get_DBSize_MB() * qps,
        "stages_ms": mean,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": "scan_kernel (first-dimension DB x query product)",
                     "peak_source": f"{peak_kind} hbm_gbs"},
        "e2e": {"value": e2e_qps, "unit": "queries/s", "h2d_bytes_per_step": qbytes,
                "d2h_bytes_per_step": qbytes + rb},
        "gpu_launches": launches,
        "clocks": clocks.summary(t0, t1),
        "ingest_s": ingest_s,
        "autotune": None if tune is None else {"seconds": tune_s, "scan_choice": tune["scan_choice"],
                     "scan_ms": [round(c["ms"], 4) for c in tune["scan_configs"]],
                     "engine_by_batch": {str(b["batch"]): b["engine"] for b in tune["batches"]},
                     "first_dim_ms_by_batch": {str(b["batch"]): {k: round(v, 3) for k, v in
                                                                 b["ms"].items()}
                                               for b in tune["batches"]},
                     "tc_ring": {"choice": tune["tc_ring_choice"],
                                 "ms": {f'{r["k_per_stage"]}x{r["stages"]}': round(r["ms"], 4)
                                        for r in tune["tc_rings"]}},
                     "tc_limbs": {"choice_bits": tune["tc_limbs_choice"],
                                  "ms": {f'{r["bits"]}bit': round(r["ms"], 4)
                                         for r in tune["tc_limbs"]}},
                     "tc_form": {"choice": tune["tc_form_choice"],
                                 "ms": {r["form"]: round(r["ms"], 4) for r in tune["tc_forms"]}},
                     "tree_forms": [{"stage": f["stage"], "count": f["count"], "form": f["form"],
                                     "ms": {k: round(v, 4) for k, v in f["ms"].items()}}
                                    for f in tune["forms"]]},
        "entries_decoded": f"{decoded}/{total}",
        "min_noise_budget": min_budget,
        "client": {"threads": 1, "keygen_ms": inp.keygen_s * 1e3, "query_ms": inp.query_s * 1e3,
                   "decode_ms": decode_s * 1e3,
                   "what": "PirClient (CPU) per client: Galois keys + RGSW(sk); per query: "
                           "generation; per response: unpack, decrypt, entry"},
        "batched": batched,
        "large": large,
        "rns": rns,
        "serving": serving,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb, match = cpu_baseline(params, args.workload, clients, queries, gpu_resps,
                                 args.cpu_queries)
        line["cpu_baseline"] = cb
        line["full_size_parity"] = "bit-exact vs oracle" if match else "MISMATCH vs oracle"
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
