/*
 * ceos_gb300.h - C ABI of the GB300 (sm_103a) CEOs / coCEOs / streamCEOs
 * maximum-inner-product-search index.
 *
 * Every entry point is a plain C function over plain pointers and sizes.
 * Host-buffer calls copy their inputs to device memory owned by the index and
 * copy results back; the *_device calls take device pointers and a
 * cudaStream_t (passed as void*, NULL = the index's own stream).
 *
 * Each declaration names the reference interface it replaces (NinhPham/CEOs,
 * paths relative to that project). The reference binds its classes to Python
 * through pybind11 in python/python_wrapper.cpp; the same methods map onto
 * these functions one to one.
 *
 * Status codes: every int-returning call returns CEOS_OK (0) or a negative
 * CEOS_ERR_* code; ceos_last_error() gives the message of the calling
 * thread's last failure. The reference prints to stderr and calls exit(1) on
 * the same conditions (src/CEOs.cpp:452-461, src/streamCEOs.cpp:179-189).
 *
 * Objects are not thread-safe: one host thread at a time per handle.
 */
#ifndef CEOS_GB300_H
#define CEOS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CEOS_ABI_VERSION 1

#define CEOS_OK 0
#define CEOS_ERR_ARG (-1)             /* invalid argument / shape */
#define CEOS_ERR_NOT_BUILT (-2)       /* search or update before build */
#define CEOS_ERR_PROBED_POINTS (-3)   /* n_probed_points > top_m (src/CEOs.cpp:452-456) */
#define CEOS_ERR_PROBED_VECTORS (-4)  /* n_probed_vectors > n_proj*n_repeats (src/CEOs.cpp:457-461);
                                         streamCEOs: > n_proj (src/streamCEOs.cpp:386-390) */
#define CEOS_ERR_UPDATE_DEL (-5)      /* n_delPoints > current size (src/streamCEOs.cpp:179-183) */
#define CEOS_ERR_UPDATE_TOPM (-6)     /* top_m > size after update (src/streamCEOs.cpp:185-189) */
#define CEOS_ERR_CUDA (-7)            /* CUDA runtime error */
#define CEOS_ERR_NO_DEVICE (-8)       /* no CUDA device visible */
#define CEOS_ERR_UNSUPPORTED (-9)     /* size outside what the kernels support */
#define CEOS_ERR_DEVICE_LIMIT (-10)   /* a bounded device-side loop gave up */
#define CEOS_ERR_TIMEOUT (-11)        /* ceos_server_wait: the request is still running */
#define CEOS_ERR_BUSY (-12)           /* the index is owned by a server (ceos_server_create*) */

/* Search algorithms for ceos_search_device. */
#define CEOS_ALGO_DENSE 0   /* CEOs-Est:   build / search */
#define CEOS_ALGO_COCEOS 1  /* coCEOs-Est: build_coCEOs_Est / search_coCEOs_Est */
#define CEOS_ALGO_HASH 2    /* CEOs-Hash:  build_CEOs_Hash / search_CEOs_Hash */

/* Numeric form of build and search. */
#define CEOS_PRECISION_FP32 0       /* bit-exact FP32 projections, FP32 rerank */
#define CEOS_PRECISION_SPLIT_BF16 1 /* BF16 rerank scan + FP32 rescore of the top 4k */

typedef struct ceos_index ceos_index;
typedef struct ceos_stream ceos_stream;

/* ---- library ---------------------------------------------------------- */
int ceos_abi_version(void);
const char* ceos_last_error(void);
/* Number of visible CUDA devices (0 when none); never fails. */
int ceos_device_count(void);
/* 0 = silent, 1 = the reference's build/search prints (src/CEOs.cpp:20-25,
 * :90-97, :278-294). Default from env CEOS_GB300_LOG, else 1. */
void ceos_set_log_level(int level);

/* Benchmark hygiene (no reference counterpart): overwrite `bytes` of a device
 * buffer owned by the library (allocated on first use) so that the next timed
 * call starts with a cold L2; synchronizes the device. */
int ceos_flush_l2(long bytes);

/* Test hook (no reference counterpart): with polls > 0, the tcgen05 projections that follow
 * (split precision, fhtDim 1024) issue no tensor-core products and give up every wait after
 * `polls` polls, so a test can check that a projection whose products never complete ends
 * its blocks, frees their tensor memory and is reported as CEOS_ERR_CUDA by the build, with
 * the device still usable. polls = 0 restores normal operation. Returns 0. */
int ceos_debug_stall_tensor_products(int polls);

/* ---- CEOs (src/CEOs.h:18-114) ----------------------------------------- */
/* CEOs(n_points, n_features): python/python_wrapper.cpp:14-21, src/CEOs.h:58-61 */
int ceos_create(int n_points, int n_features, ceos_index** out);
/* ~CEOs(): src/CEOs.h:113 */
void ceos_destroy(ceos_index* h);
/* setIndexParam(n_proj, n_repeats=1, top_m=10, n_threads=-1, random_seed=-1):
 * python/python_wrapper.cpp:23-30 -> CEOs::set_CEOsParam, src/CEOs.h:63-81.
 * Also resets n_probed_points = top_m as the reference does. */
int ceos_set_index_param(ceos_index* h, int n_proj, int n_repeats, int top_m, int n_threads,
                         int random_seed);
int ceos_get_index_param(const ceos_index* h, int* n_proj, int* n_repeats, int* top_m,
                         int* n_threads, int* random_seed, int* fht_dim);
/* set_threads(n_threads): python/python_wrapper.cpp:36 -> src/CEOs.h:96-102 (kept for API
 * compatibility; the GPU path does not use host threads). */
int ceos_set_threads(ceos_index* h, int n_threads);
/* clear(): python/python_wrapper.cpp:37 -> src/CEOs.h:83-89 (frees device memory). */
int ceos_clear(ceos_index* h);
/* n_probed_vectors / n_probed_points / n_cand attributes:
 * python/python_wrapper.cpp:32-34 (defaults 10/10/10, src/CEOs.h:52-54). */
int ceos_set_query_param(ceos_index* h, int n_probed_vectors, int n_probed_points, int n_cand);
int ceos_get_query_param(const ceos_index* h, int* n_probed_vectors, int* n_probed_points,
                         int* n_cand);
/* centering attribute: python/python_wrapper.cpp:35 (src/CEOs.h:55). Read by
 * ceos_build_ceos_hash only, as in the reference: 1 = center the rows by their column means
 * before the build. */
int ceos_set_centering(ceos_index* h, int centering);
int ceos_get_centering(const ceos_index* h, int* centering);
/* CEOS_PRECISION_* for the next search (no counterpart in the reference). The split form
 * scans the candidates' rows in bfloat16 (a copy made on the first split search) and
 * rescores the best 4 * n_neighbors of that scan exactly in FP32. Set before a build, it
 * also makes that build and the index's later updates project on the tensor cores (split
 * bfloat16 FWHT, fhtDim 256 and 1024); query projections use the FP32 transform either way. */
int ceos_set_precision(ceos_index* h, int precision);

/* build(dataset): python/python_wrapper.cpp:39 -> CEOs::build_CEOs, src/CEOs.cpp:18-98.
 * X: host, n_points x n_features float32 row-major. */
int ceos_build(ceos_index* h, const float* X);
/* search(queries, n_neighbors, verbose=False): python/python_wrapper.cpp:40-41 ->
 * CEOs::search_CEOs, src/CEOs.cpp:107-297. Q host n_queries x n_features; ids/dists host
 * n_queries x n_neighbors, best first, zero filled past the number of results. */
int ceos_search(ceos_index* h, const float* Q, int n_queries, int n_neighbors, int verbose,
                int32_t* ids, float* dists);
/* build_coCEOs_Est: python/python_wrapper.cpp:43 -> src/CEOs.cpp:311-441 */
int ceos_build_coceos_est(ceos_index* h, const float* X);
/* search_coCEOs_Est: python/python_wrapper.cpp:44-45 -> src/CEOs.cpp:450-694 */
int ceos_search_coceos_est(ceos_index* h, const float* Q, int n_queries, int n_neighbors,
                           int verbose, int32_t* ids, float* dists);
/* build_CEOs_Hash: python/python_wrapper.cpp:46 -> src/CEOs.cpp:708-840. With centering set,
 * the rows are centered by their column means (double sums in a fixed order) and the index,
 * its rerank and its scores use the centered rows. The reference's branch
 * (src/CEOs.cpp:721-728) subtracts an n-vector of row means from d-vectors, which is not a
 * column centering; this opt-in form is the corrected one. */
int ceos_build_ceos_hash(ceos_index* h, const float* X);
/* search_CEOs_Hash: python/python_wrapper.cpp:47-48 -> src/CEOs.cpp:850-1066 (n_cand unused,
 * as in the reference). */
int ceos_search_ceos_hash(ceos_index* h, const float* Q, int n_queries, int n_neighbors,
                          int verbose, int32_t* ids, float* dists);
/* Device-resident search (no reference counterpart: the queries and results already live in
 * HBM). algo = CEOS_ALGO_*, which must match the built index. */
int ceos_search_device(ceos_index* h, int algo, const float* d_Q, int n_queries,
                       int n_neighbors, int32_t* d_ids, float* d_dists, void* cuda_stream);

/* No counterpart in the reference. coCEOs-Est search over device-resident queries that
 * allocates no device memory, for callers that cannot let the library call cudaMalloc: a
 * host process that owns all device memory through its own arena (a database or search
 * engine embedding the index as a plugin), or a latency-critical serving loop where an
 * allocation could stall the device or fail mid-request. Same arguments and results as
 * ceos_search_device(h, CEOS_ALGO_COCEOS, ...), but asynchronous: the results are valid once
 * `cuda_stream` (NULL = the index's stream) has been synchronized.
 * It always runs the hash-table query kernel (the allocating search may pick the sorted one;
 * both sum every estimate in the same order, so the results are the same), and rejects with
 * CEOS_ERR_UNSUPPORTED an n_probed_vectors * n_probed_points beyond that kernel's table
 * capacity. On a split-precision index it needs the bfloat16 row copy, which the first
 * allocating split search makes: before that copy exists it returns CEOS_ERR_UNSUPPORTED;
 * afterwards it scans in bfloat16 and rescores the best 4 * n_neighbors in FP32, as
 * ceos_search_device does.
 * Scratch (padded queries, their projections, and per-CTA hash tables when a table does not
 * fit in shared memory) comes from one fixed 64 MiB device array that every GPU loading the
 * library holds until exit. A batch needing more than that is rejected with
 * CEOS_ERR_UNSUPPORTED (roughly n_queries * (n_features + n_proj * n_repeats) * 4 bytes
 * plus the tables): split it. The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress); make that first call before any stream capture. All calls
 * share the array and it keeps the last call's contents, so calls whose GPU work overlaps
 * (on different streams, or from different indexes on the same device) race: serialize
 * them. */
int ceos_search_coceos_est_device_noalloc(ceos_index* h, const float* d_Q, int n_queries,
                                          int n_neighbors, int32_t* d_ids, float* d_dists,
                                          void* cuda_stream);

/* ---- introspection (no reference counterpart; used by parity tests) ---- */
/* Buckets of a coCEOs-Est / CEOs-Hash index as [n_proj*n_repeats][2][top_m] ids and values
 * (end 0 = closest, values v; end 1 = furthest, values -v): the reference's matrix_P
 * (src/CEOs.cpp:417-428) / matrix_H (:819-828) in a column-end-major layout. */
int ceos_get_buckets(const ceos_index* h, int32_t* ids, float* vals);
/* Dense CEOs-Est projections as row-major n_points x (n_proj*n_repeats). */
int ceos_get_projections(const ceos_index* h, float* P);
/* The 3*n_repeats*fht_dim sign bits (1 = +1) in the reference's bit order. */
int ceos_get_sign_bits(const ceos_index* h, uint8_t* bits);
/* Per-phase device times (ms) of the last build/search, measured with CUDA events on the
 * index's stream; returns the number of phases written. Phase names via
 * ceos_timing_name. */
int ceos_last_timings(const ceos_index* h, float* ms, int max_phases);
const char* ceos_timing_name(const ceos_index* h, int phase);

/* ---- streamCEOs (src/streamCEOs.h:12-107) ------------------------------ */
/* streamCEOs(n_features): python/python_wrapper.cpp:52-53 */
int ceos_stream_create(int n_features, ceos_stream** out);
void ceos_stream_destroy(ceos_stream* h);
/* setIndexParam(n_proj, n_repeats=1, top_points=1, n_threads=-1, random_seed=-1):
 * python/python_wrapper.cpp:55-57 -> src/streamCEOs.h:53-70 (sets n_probed_vectors = top_m,
 * as the reference does). */
int ceos_stream_set_index_param(ceos_stream* h, int n_proj, int n_repeats, int top_points,
                                int n_threads, int random_seed);
int ceos_stream_set_threads(ceos_stream* h, int n_threads);
/* CEOS_PRECISION_* for the next estimate_search / hash_search (no counterpart in the
 * reference). */
int ceos_stream_set_precision(ceos_stream* h, int precision);
int ceos_stream_clear(ceos_stream* h);
int ceos_stream_set_query_param(ceos_stream* h, int n_probed_vectors, int n_probed_points,
                                int n_cand);
int ceos_stream_get_query_param(const ceos_stream* h, int* n_probed_vectors,
                                int* n_probed_points, int* n_cand);
/* build(dataset): python/python_wrapper.cpp:65 -> src/streamCEOs.cpp:9-161 */
int ceos_stream_build(ceos_stream* h, const float* X, int n_points);
/* update(new_dataset, n_delPoints=0): python/python_wrapper.cpp:66 ->
 * src/streamCEOs.cpp:174-369 (append at the back, delete n_del from the front). */
int ceos_stream_update(ceos_stream* h, const float* X_new, int n_new, int n_del);
/* estimate_search: python/python_wrapper.cpp:67-68 -> src/streamCEOs.cpp:378-612 */
int ceos_stream_estimate_search(ceos_stream* h, const float* Q, int n_queries, int n_neighbors,
                                int verbose, int32_t* ids, float* dists);
/* hash_search: python/python_wrapper.cpp:69-70 -> src/streamCEOs.cpp:621-877 */
int ceos_stream_hash_search(ceos_stream* h, const float* Q, int n_queries, int n_neighbors,
                            int verbose, int32_t* ids, float* dists);
/* Exact maintenance and random-id deletes (no reference counterpart: the reference
 * deletes only from the front, n_delPoints of src/streamCEOs.cpp:207-208, and refills a
 * bucket only from new points, leaving stale rows when too few remain, :337-352).
 * set_reserve(r >= 0) before build keeps top_points + r entries per column end; every
 * bucket is then the exact top-m over the live points after each update and delete
 * (a list that drops below top_m is refilled from all live rows). -1 (default) keeps
 * the reference's maintenance. */
int ceos_stream_set_reserve(ceos_stream* h, int reserve);
int ceos_stream_get_reserve(const ceos_stream* h, int* reserve);
/* Delete the points with the given current ids (0 .. size-1, duplicates ignored);
 * later ids move down, as erasing from the reference's deque would. Needs
 * set_reserve(>= 0) before build. CEOS_ERR_UPDATE_TOPM when fewer than top_points
 * points would remain. */
int ceos_stream_delete(ceos_stream* h, const int32_t* ids, int n_ids);
/* Current number of points (the reference's deque_X.size()). */
int ceos_stream_size(const ceos_stream* h, int* n_points);
int ceos_stream_get_buckets(const ceos_stream* h, int32_t* ids, float* vals);

/* ---- file ingestion ------------------------------------------------------
 * Build from a raw row-major float32 file holding at least n_points x n_features values: the
 * format the reference's loadbinData reads (src/Utilities.cpp:142-214), where the file is
 * mmapped and copied into an in-memory matrix before the build. Here the mapped rows stream
 * to the device through two pinned chunks, so the file never has to fit in host memory.
 * algo: CEOS_ALGO_DENSE (build), CEOS_ALGO_COCEOS (build_coCEOs_Est), CEOS_ALGO_HASH
 * (build_CEOs_Hash). A file with fewer rows fails with CEOS_ERR_ARG (the reference exits,
 * src/Utilities.cpp:171-175). */
int ceos_build_from_file(ceos_index* h, const char* path, int algo);
int ceos_stream_build_from_file(ceos_stream* h, const char* path, int n_points);

/* ---- save / load (no reference counterpart: the reference rebuilds every index) ----
 * A versioned binary file (magic "CEOSGB3", version 1) with the parameters, the rows in
 * logical order, the sign words and the built structures (buckets, or the dense CEOs-Est
 * projections; for streams with a reserve also the per-list counts and thresholds), closed by
 * an FNV-1a checksum. A loaded index is device resident and searches / updates exactly like
 * the saved one without rebuilding. Loading a file of the other kind, another version, or a
 * truncated or corrupt file fails with CEOS_ERR_ARG. */
/* Shape, precision and stream parameters of a handle (e.g. after a load). */
int ceos_get_shape(const ceos_index* h, int* n_points, int* n_features);
int ceos_get_precision(const ceos_index* h, int* precision);
int ceos_stream_get_index_param(const ceos_stream* h, int* n_proj, int* n_repeats,
                                int* top_points, int* seed, int* n_features);
int ceos_stream_get_precision(const ceos_stream* h, int* precision);
int ceos_save(const ceos_index* h, const char* path);
int ceos_load(const char* path, ceos_index** out);
int ceos_stream_save(const ceos_stream* h, const char* path);
int ceos_stream_load(const char* path, ceos_stream** out);

/* ---- ground truth (no reference counterpart in the library) -------------
 * Exact top-k maximum inner products of Q (nq x d) against X (n x d), row-major host
 * float32, computed on the GPU in FP64 (float products are exact in double; double
 * sums); ids and FP64 scores best first, ties towards the smaller id. Replaces the
 * faiss IndexFlatIP ground truth of the reference's scripts (test/utils.py:35-55),
 * for recall = |exact ∩ approx| / k (test/utils.py:27-32). k <= 1024. */
int ceos_bruteforce_fp64(const float* X, long n, int d, const float* Q, int nq, int k,
                         int32_t* ids, double* scores);

/* ---- serving loop (no reference counterpart) ----------------------------
 * The reference answers one blocking batch per call (python/python_wrapper.cpp:36-48,
 * :62-71). A server keeps a built index resident on the device and answers requests
 * submitted from any host thread. Each request is a block of queries with its own
 * n_neighbors and n_probed_vectors (n_probed_points and n_cand are the index's, as
 * set when the server is created), or, on a streamCEOs index, an update.
 *
 * One worker thread packs the queued query requests, in arrival order, into batches
 * of at most max_batch queries on n_slots device slots; a request larger than the
 * free room is split. A batch is launched as soon as a slot is free, so requests
 * that arrive while other batches run are admitted into the next slot that frees
 * up, and the slots' batches overlap on the device (continuous batching). Each slot
 * holds fixed device memory (slot_bytes in the stats); slots are created only while
 * they fit mem_budget_bytes. A batch (query upload, projection, the persistent query
 * kernel, result download) is replayed as a CUDA graph captured per (slot,
 * power-of-two batch size). An update waits until no batch is in flight, so every
 * request sees the index as of its place in the queue.
 *
 * A request's results are the same, bit for bit, whatever it is batched with, and
 * equal those of the index's own search with the same n_probed_vectors, n_neighbors
 * and precision.
 *
 * While a server exists, the index's own build, update, search, clear and set_*
 * calls return CEOS_ERR_BUSY. Destroy the server (it finishes queued work) before
 * the index. */
typedef struct ceos_server ceos_server;

typedef struct ceos_server_config {
  int algo;               /* CEOS_ALGO_COCEOS (coCEOs-Est; streamCEOs estimate_search) or
                             CEOS_ALGO_HASH (CEOs-Hash; streamCEOs hash_search) */
  int n_slots;            /* batches in flight, >= 1 */
  int max_batch;          /* queries per batch, >= 1 */
  int max_neighbors;      /* largest n_neighbors of a request */
  int max_probed_vectors; /* largest n_probed_vectors of a request */
  long long mem_budget_bytes; /* device bytes for the slots; 0 = no limit */
  int use_graphs;         /* 1 = replay batches as CUDA graphs, 0 = launch them directly */
} ceos_server_config;

typedef struct ceos_server_stats {
  long long requests;        /* query requests completed since the last reset */
  long long queries;         /* queries launched */
  long long batches;         /* batches launched */
  long long graph_launches;  /* batches launched as graph replays */
  long long graphs_captured; /* graphs captured (since creation) */
  long long updates;         /* updates applied */
  int slots;                 /* slots created under the memory budget */
  long long slot_bytes;      /* device bytes of one slot */
  double mean_batch_queries;
  double p50_ms, p90_ms, p99_ms, max_ms, mean_ms; /* request latency: submit to results written */
  double busy_s;             /* first submit to last completion since the last reset */
} ceos_server_stats;

/* Defaults: algo COCEOS, 4 slots, max_batch 256, max_neighbors 100,
 * max_probed_vectors 80, no budget, graphs on. */
int ceos_server_config_init(ceos_server_config* cfg);
int ceos_server_create(ceos_index* h, const ceos_server_config* cfg, ceos_server** out);
int ceos_server_create_stream(ceos_stream* h, const ceos_server_config* cfg, ceos_server** out);
/* Finishes queued work, then frees the server. */
void ceos_server_destroy(ceos_server* s);
/* Queue n_queries x n_features queries (copied at the call). n_probed_vectors <= 0
 * means the index's current value. ids / dists (n_queries x n_neighbors, best first)
 * are written before the request completes and must stay valid until then. */
int ceos_server_submit(ceos_server* s, const float* Q, int n_queries, int n_neighbors,
                       int n_probed_vectors, int32_t* ids, float* dists, uint64_t* ticket);
/* streamCEOs update (src/streamCEOs.cpp:174-369) in queue order; rows copied at the call. */
int ceos_server_submit_update(ceos_server* s, const float* X_new, int n_new, int n_del,
                              uint64_t* ticket);
/* Random-id delete (ceos_stream_delete) in queue order; ids copied at the call. */
int ceos_server_submit_delete(ceos_server* s, const int32_t* ids, int n_ids, uint64_t* ticket);
/* Block until the request completes (timeout_ms < 0: no limit); returns its status,
 * CEOS_ERR_TIMEOUT if it is still running. A completed ticket is released. */
int ceos_server_wait(ceos_server* s, uint64_t ticket, int timeout_ms);
int ceos_server_get_stats(ceos_server* s, ceos_server_stats* out);
int ceos_server_reset_stats(ceos_server* s);

#ifdef __cplusplus
}
#endif

#endif /* CEOS_GB300_H */
