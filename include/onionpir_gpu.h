/*
 * onionpir_gpu.h -- C ABI of the GB300-native OnionPIRv2 server query path.
 *
 * This is the boundary a PirServer implementation calls instead of running
 * the reference's single-threaded CPU loops.  Every entry point names the
 * reference interface it replaces (paths are within chenyue42/OnionPIRv2).
 *
 * Conventions
 *   - N = 2048 (DatabaseConstants::PolyDegree), one ciphertext prime q plus
 *     SEAL's special key-switching prime p (CoeffMods = {60, 60}: rns = 1).
 *   - A ciphertext is uint64_t[2][N] (c0 then c1), fully reduced mod q,
 *     coefficient form -- SEAL's in-memory layout for rns = 1.
 *   - "NTT form" means the negacyclic transform A[k] = a(psi^(2 brv(k)+1)),
 *     psi the smallest primitive 2N-th root of unity mod the prime.
 *   - Host buffers are caller-owned; the context owns all device memory.
 *   - Every call returns an opir_status; opir_last_error() explains the
 *     most recent failure.  No C++ exception crosses this ABI.
 *   - Calls on one context are serialised by an internal mutex.
 */
#ifndef ONIONPIR_GPU_H
#define ONIONPIR_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  OPIR_OK = 0,
  OPIR_ERR_ARG = -1,            /* invalid argument / parameter set        */
  OPIR_ERR_UNKNOWN_CLIENT = -2, /* no keys for this client id (server.cpp:389 .at()) */
  OPIR_ERR_UNKNOWN_DB = -3,
  OPIR_ERR_OOM = -4,            /* device allocation failed                 */
  OPIR_ERR_CUDA = -5,           /* CUDA runtime error                       */
  OPIR_ERR_STATE = -6,          /* call not valid in the current state      */
  OPIR_ERR_NO_DEVICE = -7,
  OPIR_ERR_TIMEOUT = -8         /* a bounded device-side wait gave up       */
} opir_status;

/* Ciphertext-side parameters (PirParams, pir.cpp:9-54; database_constants.h). */
typedef struct opir_params {
  uint32_t poly_degree;     /* N; must be 2048                                  */
  uint64_t coeff_modulus;   /* q  (CoeffModulus::Create(N,{60,60})[0])          */
  uint64_t special_modulus; /* p  (the last, key-switching prime)               */
  uint64_t plain_modulus;   /* t  (utils::generate_prime(PlainMod))             */
  uint64_t small_modulus;   /* small_q (pir.cpp:40-41)                          */
  uint32_t gsw_l;           /* l      (GSW_L)                                   */
  uint32_t gsw_base_log2;   /* log2 B (pir.cpp:53)                              */
  uint32_t gsw_l_key;       /* l_key  (GSW_L_KEY)                               */
  uint32_t gsw_base_log2_key; /* (pir.cpp:54)                                   */
} opir_params;

/* Database shape (PirParams::get_dims / get_entry_size, pir.cpp:29-95). */
typedef struct opir_db_shape {
  uint32_t fst_dim_sz;      /* n1                                                */
  uint32_t other_dim_sz;    /* n_rest = 2^(ndim-1)                               */
  uint32_t entry_size;      /* bytes per entry                                   */
  uint32_t entries_per_pt;  /* entries packed per plaintext                      */
  uint32_t bits_per_coeff;  /* bits of entry data per plaintext coefficient      */
} opir_db_shape;

typedef struct opir_ctx opir_ctx;

/* PirServer::PirServer (server.cpp:25-39): parameters, NTT tables, device. */
int opir_ctx_create(const opir_params *params, int device, opir_ctx **out);
void opir_ctx_destroy(opir_ctx *ctx);
/* Run all work of this context on a caller-provided cudaStream_t (NULL =
 * the context's own stream). */
int opir_ctx_set_stream(opir_ctx *ctx, void *cuda_stream);
const char *opir_last_error(const opir_ctx *ctx);
uint64_t opir_response_bytes(const opir_ctx *ctx);

/* Multi-modulus parameter sets (rns_mod_cnt > 1: the PolyDegree = 4096,
 * CoeffMods = {60, 60, 60} presets of database_constants.h:13-172), and any
 * power-of-two N from 1024 to 4096 with one or two ciphertext primes.
 * Replaces PirServer::PirServer for those presets (server.cpp:25-39).
 * On such a context a ciphertext is uint64_t[2][R][N] (SEAL's layout: poly,
 * prime, coefficient); Galois keys are [level][R][2][R+1][N] (decomposition
 * prime j, key polynomial, modulus q_0 .. q_{R-1}, p; NTT form), the RGSW
 * key [2 l_key][2][R][N] (coefficient form), the reference-layout database
 * [R N][num_pt]; responses stay [2][N] mod small_q after the switch to q_0
 * (server.cpp:567-570) and to small_q.  Supported: the database calls but
 * push_chunk and get_entry, the key calls, opir_make_query, _batch (one
 * query after another) and _trace (leaves [u][2][R][N], gsw
 * [ndim-1][2l][2][R][N], first_dim [n_rest][2][R][N]), opir_pack_response,
 * opir_ntt (mod 0 .. R-1 = q_i, R = p), timing, opir_sync.  The others return
 * OPIR_ERR_STATE. */
typedef struct opir_rns_params {
  uint32_t poly_degree;        /* N                                           */
  uint32_t rns_count;          /* ciphertext primes R: 1 or 2                 */
  uint64_t coeff_moduli[2];    /* q_0 .. q_{R-1} (CoeffModulus::Create order) */
  uint64_t special_modulus;    /* p                                           */
  uint64_t plain_modulus;      /* t                                           */
  uint64_t small_modulus;      /* small_q                                     */
  uint32_t gsw_l;              /* l      (GSW_L)                              */
  uint32_t gsw_base_log2;      /* ceil(log2 Q / l)       (pir.cpp:53)         */
  uint32_t gsw_l_key;          /* l_key  (GSW_L_KEY)                          */
  uint32_t gsw_base_log2_key;  /* ceil(log2 Q / l_key)   (pir.cpp:54)         */
} opir_rns_params;
int opir_ctx_create_rns(const opir_rns_params *params, int device, opir_ctx **out);

/* ---- database (server.h:22-25; server.cpp:47-78, 635-748) ---- */
int opir_db_create(opir_ctx *ctx, const opir_db_shape *shape, uint32_t *db_id);
int opir_db_destroy(opir_ctx *ctx, uint32_t db_id);
/* PirServer::push_database_chunk (server.cpp:635-701) + preprocess_ntt
 * (703-719) + realign_db (722-748) for one chunk: chunk_idx selects
 * plaintexts [chunk_idx*n1, (chunk_idx+1)*n1); `entries` holds
 * n1*entries_per_pt entries of entry_size bytes each. */
int opir_db_push_chunk(opir_ctx *ctx, uint32_t db_id, const uint8_t *entries,
                       uint64_t num_entries, uint64_t chunk_idx);
/* PirServer::gen_data (server.cpp:47-78) with entries derived from `seed`
 * (8-byte big-endian index + seeded bytes, utils.cpp:160-172), generated and
 * ingested on the device. */
int opir_db_fill_synthetic(opir_ctx *ctx, uint32_t db_id, uint64_t seed);
/* Upload an already-NTT'd database in the reference layout
 * db_aligned_[c*num_pt + row*n1 + col] (server.cpp:740). */
int opir_db_upload_aligned(opir_ctx *ctx, uint32_t db_id, const uint64_t *db_aligned);

/* PirServer::direct_get_entry (server.cpp:503-517): the entry's
 * entry_size bytes, read back from the device database (its plaintext
 * inverse-transformed and unpacked), for checking decrypted responses. */
int opir_db_get_entry(opir_ctx *ctx, uint32_t db_id, uint64_t entry_index, uint8_t *entry);

/* ---- per-client keys (server.cpp:480-500) ---- */
/* set_client_galois_key: keys[level][k][mod][N], NTT form, level a is the
 * Galois element 1 + (N >> a) (client.cpp:235-237), mod 0 = q, 1 = p. */
int opir_set_galois_key(opir_ctx *ctx, uint64_t client_id, const uint64_t *keys,
                        uint32_t levels);
/* set_client_gsw_key: 2*l_key RGSW(sk) rows [row][2][N], coefficient form;
 * transformed to NTT form on the device (gsw_eval.cpp:15-31). */
int opir_set_gsw_key(opir_ctx *ctx, uint64_t client_id, const uint64_t *rows);
int opir_erase_client(opir_ctx *ctx, uint64_t client_id);

/* Key budget (no reference counterpart; the reference keeps every client's
 * keys in std::map members, server.h:58-59).  With bytes > 0 the context keeps
 * host copies of client keys and holds at most bytes / opir_key_bytes_per_client
 * clients' keys in device memory, evicting the least recently used client
 * not needed by a query in flight; evicted keys are copied back when that
 * client queries again.  0 (the default) keeps every client's keys resident.
 * Call before the first key is registered. */
int opir_set_key_budget(opir_ctx *ctx, uint64_t bytes);
uint64_t opir_key_bytes_per_client(const opir_ctx *ctx);
/* clients whose keys are in device memory, and the slots of the budget (0: no budget) */
int opir_resident_clients(opir_ctx *ctx, uint32_t *resident, uint32_t *slots);

/* ---- queries (server.cpp:520-633) ---- */
/* PirServer::make_query + mod_switch_inplace + save_resp_to_stream:
 * query[2][N] (coefficient form, mod q) -> resp[2][N] (mod small_q, may be
 * NULL) and packed (opir_response_bytes() bytes, may be NULL).  Blocking. */
int opir_make_query(opir_ctx *ctx, uint32_t db_id, uint64_t client_id, const uint64_t *query,
                    uint64_t *resp, uint8_t *packed);
/* The same for `batch` independent queries against one database in one
 * pass: queries[batch][2][N], resps[batch][2][N], packed[batch][bytes]. */
int opir_make_query_batch(opir_ctx *ctx, uint32_t db_id, uint32_t batch,
                          const uint64_t *client_ids, const uint64_t *queries, uint64_t *resps,
                          uint8_t *packed);
/* Device-pointer variant, asynchronous on the context stream. */
int opir_make_query_device(opir_ctx *ctx, uint32_t db_id, uint32_t batch,
                           const uint64_t *client_ids, const uint64_t *d_queries,
                           uint64_t *d_resps, uint8_t *d_packed);
/* make_query with every intermediate copied out, for parity tests:
 * leaves[u][2][N] (after fast_expand_qry), gsw[(ndim-1)][2l][2][N] (NTT form),
 * first_dim[n_rest][2][N] (after evaluate_first_dim, coefficient form).
 * Any output pointer may be NULL. */
int opir_make_query_trace(opir_ctx *ctx, uint32_t db_id, uint64_t client_id,
                          const uint64_t *query, uint64_t *leaves, uint64_t *gsw,
                          uint64_t *first_dim, uint64_t *resp, uint8_t *packed);

/* PirServer::save_resp_to_stream (server.cpp:581-633) for any responses:
 * resps[count][2][N] (host; coefficients mod small_q, of which the low
 * ceil(log2 small_q) bits are kept, as the reference masks them) ->
 * packed[count][opir_response_bytes()] (host), each the reference's
 * LSB-first bit stream of c0 then c1.  opir_make_query* already return the
 * packed bytes of their own responses; this packs responses held elsewhere
 * (batches, served tickets, stored ciphertexts).  Blocking. */
int opir_pack_response(opir_ctx *ctx, const uint64_t *resps, uint32_t count, uint8_t *packed);

/* PirServer::other_dim_mux (server.h:39, server.cpp:295-334): one folding
 * level.  result[count][2][N] (host, coefficient form, fully reduced mod q;
 * count even) and the RGSW selection ciphertext sel[2l][2][N] (host, NTT
 * form: the layout query_to_gsw produces, gsw_eval.h:8).  For
 * i < count/2: result[i] = result[i] + INTT(sel (x) (result[i + count/2] -
 * result[i])); afterwards result[0 .. count/2) holds the folded ciphertexts
 * (the reference resizes its vector to that half).  Blocking. */
int opir_other_dim_mux(opir_ctx *ctx, uint64_t *result, uint64_t count, const uint64_t *sel);

/* First dimension only, without allocating device memory.  No counterpart
 * in the reference.  d_fst_cts: the n1 expanded selection ciphertexts
 * [n1][2][N] (device, coefficient form); d_out: the n_rest results
 * [n_rest][2][N] (device, coefficient form).  For callers that cannot call
 * cudaMalloc during a request (a request thread with a latency budget, since
 * allocation synchronises the device, or a process whose device memory is
 * reserved up front by another allocator): the scan's query operand lives in
 * a 16 MiB static device array, so n1 <= 512 (larger databases get
 * OPIR_ERR_ARG).  The first call on each context looks up that array's
 * address (cudaGetSymbolAddress) with the context's device current, so make
 * it before any stream capture.  Asynchronous on the context stream: a scan
 * that gives up on a bounded device wait records it in the context's status
 * word, which the next opir_sync reports as OPIR_ERR_TIMEOUT.  All calls (of
 * every context on a device) share the array, so calls that overlap on the
 * GPU race. */
int opir_first_dim_noalloc(opir_ctx *ctx, uint32_t db_id, const uint64_t *d_fst_cts,
                           uint64_t *d_out);

/* ---- first-dimension engine for batches (no reference counterpart) ----
 * A batch of queries on one database can share one pass over it: the
 * product becomes a per-slot (n_rest x n1) . (n1 x 2B) GEMM.  AUTO (default):
 * the tcgen05 tensor-core engine (residues split into 8-bit limbs, exact)
 * from tensor_min_batch queries on (default 4; 0 keeps the current value)
 * when the shape allows it (n1 a multiple of 32, n_rest of 16), else the
 * integer multiply-add GEMM from 32 queries on, else one streaming pass per
 * query -- the crossovers measured on GB300.  SCAN: one pass per query; IMAD /
 * TENSOR: that engine for every batch of 2 or more the shape allows.  All
 * give the same bits. */
enum {
  OPIR_ENGINE_AUTO = 0,
  OPIR_ENGINE_SCAN = 1,
  OPIR_ENGINE_IMAD = 2,
  OPIR_ENGINE_TENSOR = 3
};
int opir_set_batch_engine(opir_ctx *ctx, int engine, uint32_t tensor_min_batch);

/* ---- autotuner (no reference counterpart) ----
 * Times, on this GPU and for database db_id, every compiled tile
 * configuration of the single-query scan, the first-dimension product of
 * every engine (one scan per query, integer GEMM, tensor-core limb GEMM) at
 * the batch sizes 2, 4, ..., max_batch (at most 256), the tensor kernel's
 * two shared-memory ring shapes at the largest of them, and every launch
 * form (one CTA per ciphertext, two CTAs, a thread-block cluster) of every
 * expansion, RGSW-reconstruction and folding launch of this database's
 * pipeline at one query and at each batch size up to 64 -- each after a
 * warm-up, over `reps` repetitions (0: 3), on operands of valid residues.
 * The database then scans with the fastest configuration, runs the tensor
 * kernel with the faster ring, launches each tree stage in the form that was
 * fastest for its work count, and under OPIR_ENGINE_AUTO a batch of B
 * queries takes the engine that was fastest at the largest measured size
 * <= B.  Builds the database's limb plane if the tensor engine can run on
 * it.  Results are unchanged (every configuration, ring, form and engine
 * gives the same bits).  Not while serving (OPIR_ERR_STATE).
 * Times in ms of one launch or product; < 0: cannot run this shape. */
typedef struct opir_tune_report {
  uint32_t scan_configs;   /* compiled scan configurations (<= 16) */
  uint32_t scan_desc[16][6]; /* rows per thread, warps, k-steps, stages, CTAs per SM,
                                Karatsuba products (0/1) */
  float scan_ms[16];
  int32_t scan_choice;     /* chosen configuration, -1: the plain kernel */
  uint32_t batch_points;   /* number of batch sizes measured (<= 8) */
  uint32_t batch[8];
  float engine_ms[8][3];   /* [point][OPIR_ENGINE_SCAN - 1 .. OPIR_ENGINE_TENSOR - 1] */
  int32_t engine[8];       /* chosen OPIR_ENGINE_* per point */
  uint32_t tc_ring_desc[2][2]; /* tensor kernel rings: {k per stage, stages} */
  float tc_ring_ms[2];     /* at the largest batch size; < 0: not measured */
  int32_t tc_ring_choice;  /* -1: not tuned */
  uint32_t form_points;    /* distinct tree-stage launches measured (<= 128) */
  uint32_t form_stage[128]; /* 0 expansion, 1 RGSW reconstruction, 2 folding */
  uint32_t form_count[128]; /* work items: nodes / ciphertexts / pairs x queries */
  float form_ms[128][4];   /* one CTA, two CTAs, cluster, ten-CTA cluster (folding) per
                              ciphertext; the stage's whole launch sequence */
  int32_t form_choice[128];
  float tc_limbs_ms[2];    /* query limbs of 8 and 9 bits at the largest batch size (the
                              limb split plus the tensor kernel); < 0: not measured */
  int32_t tc_limbs_choice; /* 0: 8-bit, 1: 9-bit, -1: not tuned */
  float tc_pair_ms[2];     /* one CTA per tile, CTA pairs (M = 256, cta_group::2) at the
                              largest batch size; < 0: not measured or not applicable */
  int32_t tc_pair_choice;  /* 0: one CTA, 1: pairs, -1: not tuned */
} opir_tune_report;
int opir_autotune(opir_ctx *ctx, uint32_t db_id, uint32_t max_batch, uint32_t reps,
                  opir_tune_report *report);

/* ---- serving: continuous batching ----
 * No reference counterpart (PirServer::make_query, server.cpp:520-579,
 * answers one query per call).  opir_serve_start starts a worker thread that
 * takes submitted queries from per-database queues and runs them in batches
 * of up to max_batch queries against the resident database, with up to
 * `lanes` batches on the device at once.  A free lane takes a batch at once
 * when the device is otherwise idle; while another batch runs it waits for a
 * full batch or until the oldest request has waited max_wait_us.  Every
 * response is the one opir_make_query returns for the same query.  While
 * serving is active, opir_make_query and opir_make_query_batch submit their
 * queries as tickets and wait for them (same responses); the trace, device
 * and allocation-free calls and database changes return OPIR_ERR_STATE; keys
 * can be registered (a client's keys cannot change while its queries are in
 * flight). */
typedef struct opir_serve_config {
  uint32_t max_batch;    /* queries per batch (>= 1)                    */
  uint32_t lanes;        /* batches on the device at once (1 .. 4)      */
  uint32_t max_wait_us;  /* see above                                   */
} opir_serve_config;

typedef struct opir_serve_stats {
  uint64_t submitted, completed, failed, batches, queued;
  double mean_batch;                  /* queries per batch                      */
  double p50_ms, p99_ms, mean_ms, max_ms;  /* submission -> response ready       */
  double queries_per_s;               /* completed / (last completion - first submission) */
} opir_serve_stats;

int opir_serve_start(opir_ctx *ctx, const opir_serve_config *cfg);
/* finishes every queued query, then stops the worker; results stay pollable */
int opir_serve_stop(opir_ctx *ctx);
/* queue one query ([2][N] ciphertext, copied); *ticket identifies it */
int opir_submit(opir_ctx *ctx, uint32_t db_id, uint64_t client_id, const uint64_t *query,
                uint64_t *ticket);
/* *done = 0: still queued or running.  *done = 1: resp ([2][N]) and packed
 * (opir_response_bytes) are filled when not NULL, the ticket is released and
 * the return value is the query's status. */
int opir_poll(opir_ctx *ctx, uint64_t ticket, uint64_t *resp, uint8_t *packed, int *done);
/* as opir_poll, blocking up to timeout_ms (OPIR_ERR_TIMEOUT: still pending) */
int opir_wait(opir_ctx *ctx, uint64_t ticket, uint32_t timeout_ms, uint64_t *resp,
              uint8_t *packed);
/* counters and latency percentiles since opir_serve_start */
int opir_serve_stats_get(opir_ctx *ctx, opir_serve_stats *out);

/* ---- timing and accounting ---- */
/* Single queries on the synchronous calls (opir_make_query,
 * opir_make_query_device) are captured into a CUDA graph and replayed
 * (default on; OPIR_GRAPHS=0 in the environment turns it off at context
 * creation).  The graph is not used with stage timing, traces or a key
 * budget.  Results are the same either way. */
int opir_set_graphs(opir_ctx *ctx, int enable);
/* Enable per-stage CUDA-event timing of subsequent queries. */
int opir_set_timing(opir_ctx *ctx, int enable);
/* Device milliseconds of the last timed query for the reference's sections
 * (logging.h): [0] Expand, [1] Convert, [2] First dim, [3] Other dim,
 * [4] Mod switch; [5] = the first-dimension scan kernel alone. */
int opir_stage_times(opir_ctx *ctx, float *ms6);
/* Number of kernels this context has launched since creation. */
uint64_t opir_launch_count(const opir_ctx *ctx);
/* Wait for the context stream and report (then clear) any device-side
 * error recorded by asynchronous queries (OPIR_ERR_TIMEOUT). */
int opir_sync(opir_ctx *ctx);

/* Test hook of the bounded device waits (no reference counterpart).  With
 * polls > 0 the single-query scan of this context's synchronous calls
 * withholds the copies of one pipeline stage in its first CTA and gives up
 * waiting for that stage after `polls` polls (at most 2^20; the production
 * limit is 2^22): the call then returns OPIR_ERR_TIMEOUT with the status
 * bits in opir_last_error, and the next call on the context runs normally.
 * 0 turns it off.  Not for production use. */
int opir_debug_withhold_scan_stage(opir_ctx *ctx, uint32_t polls);
/* Test hook of the first dimension (the inside of evaluate_first_dim; no
 * public reference counterpart): `batch` queries' first-dimension leaves
 * given directly, leaves[batch][n1][2][N] in coefficient form, multiplied
 * with the database on the engine this batch size uses (opir_set_batch_engine,
 * the tuned table or the crossovers; OPIR_TC_LIMBS forces the tensor
 * engine's query limb width); out[batch][n_rest][2][N] in coefficient form.
 * Lets tests drive the products with operands no query expansion produces. */
int opir_debug_first_dim(opir_ctx *ctx, uint32_t db_id, uint32_t batch, const uint64_t *leaves,
                         uint64_t *out);

/* ---- primitives (tests) ---- */
/* Negacyclic NTT of `count` polynomials mod q (mod = 0) or p (mod = 1),
 * host buffers, in place. */
int opir_ntt(opir_ctx *ctx, int mod, int inverse, uint64_t *polys, uint64_t count);
/* The same on device memory, asynchronous on the context stream
 * (forward: natural order in, NTT slot order out; inverse: the reverse). */
int opir_ntt_device(opir_ctx *ctx, int mod, int inverse, uint64_t *d_polys, uint64_t count);

#ifdef __cplusplus
}
#endif
#endif
