// C ABI (include/ceos_gb300.h) over the host core (core.h).
//
// Validates parameters with the reference's rules and maps each entry point
// onto the index state; parameter semantics follow src/CEOs.h:52-81 and
// src/streamCEOs.h:40-70.
#include "core.h"

using namespace ceos_host;

extern "C" {

int ceos_abi_version(void) { return CEOS_ABI_VERSION; }
const char* ceos_last_error(void) { return g_err.c_str(); }
int ceos_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}
void ceos_set_log_level(int level) { g_log = level < 0 ? 0 : level; }

int ceos_debug_stall_tensor_products(int polls) {
  project_t5_set_stall(polls < 0 ? 0 : polls);
  return CEOS_OK;
}

int ceos_flush_l2(long bytes) {
  static DevBuf* flush = nullptr;
  if (bytes <= 0) return fail(CEOS_ERR_ARG, "bytes must be > 0");
  if (!flush) flush = new DevBuf();
  CUDA_TRY(flush->ensure((size_t)bytes));
  CUDA_TRY(cudaMemsetAsync(flush->p, 0x5a, (size_t)bytes, 0));
  CUDA_TRY(cudaDeviceSynchronize());
  return CEOS_OK;
}

// ---------------------------------------------------------------------------
int ceos_create(int n_points, int n_features, ceos_index** out) {
  if (!out) return fail(CEOS_ERR_ARG, "null output handle");
  *out = nullptr;
  if (n_points < 1 || n_features < 1)
    return fail(CEOS_ERR_ARG, "n_points (%d) and n_features (%d) must be >= 1", n_points, n_features);
  ceos_index* h = new ceos_index();
  h->n_points = n_points;
  h->core.n_features = n_features;
  h->core.set_param(256, 1, 100, -1, -1);  // class defaults, src/CEOs.h:24-29
  *out = h;
  return CEOS_OK;
}

void ceos_destroy(ceos_index* h) { delete h; }

int ceos_set_index_param(ceos_index* h, int n_proj, int n_repeats, int top_m, int n_threads,
                         int random_seed) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  if (n_proj < 1 || n_repeats < 1) return fail(CEOS_ERR_ARG, "n_proj and n_repeats must be >= 1");
  h->core.set_param(n_proj, n_repeats, top_m, n_threads, random_seed);
  h->core.p = top_m;  // n_probed_points = top_m (src/CEOs.h:69)
  return CEOS_OK;
}

int ceos_get_index_param(const ceos_index* h, int* n_proj, int* n_repeats, int* top_m,
                         int* n_threads, int* random_seed, int* fht_dim_out) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  const Core& c = h->core;
  if (n_proj) *n_proj = c.n_proj;
  if (n_repeats) *n_repeats = c.n_repeats;
  if (top_m) *top_m = c.top_m;
  if (n_threads) *n_threads = c.n_threads;
  if (random_seed) *random_seed = c.seed;
  if (fht_dim_out) *fht_dim_out = c.fht;
  return CEOS_OK;
}

int ceos_set_threads(ceos_index* h, int n_threads) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  h->core.n_threads = n_threads;
  return CEOS_OK;
}

int ceos_clear(ceos_index* h) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  if (h->core.device >= 0) cudaSetDevice(h->core.device);
  h->core.release_all();
  return CEOS_OK;
}

int ceos_set_query_param(ceos_index* h, int s, int p, int c) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  h->core.s = s;
  h->core.p = p;
  h->core.c = c;
  return CEOS_OK;
}

int ceos_get_query_param(const ceos_index* h, int* s, int* p, int* c) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (s) *s = h->core.s;
  if (p) *p = h->core.p;
  if (c) *c = h->core.c;
  return CEOS_OK;
}

int ceos_set_centering(ceos_index* h, int centering) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  h->core.centering = centering ? 1 : 0;
  return CEOS_OK;
}

int ceos_get_centering(const ceos_index* h, int* centering) {
  if (!h || !centering) return fail(CEOS_ERR_ARG, "null argument");
  *centering = h->core.centering;
  return CEOS_OK;
}

int ceos_set_precision(ceos_index* h, int precision) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  if (precision != CEOS_PRECISION_FP32 && precision != CEOS_PRECISION_SPLIT_BF16)
    return fail(CEOS_ERR_ARG, "unknown precision %d", precision);
  h->core.precision = precision;
  return CEOS_OK;
}

// Rows of a build come from host memory, or from a file when `path` is set.
static thread_local const char* g_build_path = nullptr;

static int index_build_common(ceos_index* h, const float* X, const char* what) {
  if (!h || (!X && !g_build_path)) return fail(CEOS_ERR_ARG, "null argument");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  Core& c = h->core;
  ST_TRY(c.check_param());
  ST_TRY(c.ensure_device());
  c.release_all();
  c.timer.begin(c.stream);
  c.n_rows = h->n_points;
  c.head = 0;
  c.cap_rows = h->n_points;
  CUDA_TRY(c.dX.ensure((size_t)c.n_rows * c.ldx * 4));
  if (g_build_path)
    ST_TRY(c.upload_rows_from_file(g_build_path, c.n_rows, c.dX.as<float>()));
  else
    ST_TRY(c.upload_rows(X, c.n_rows, c.dX.as<float>()));
  ST_TRY(c.upload_signs());
  c.proj_tensor = (c.precision == CEOS_PRECISION_SPLIT_BF16 && project_tc_supported(c.L)) ? 1 : 0;
  c.timer.mark("h2d");
  if (log_level() >= 1) {
    std::printf("%s\nn_points: %ld\nn_features: %d\nn_repeats: %d\nn_proj: %d\ntop_m: %d\nfhtDim: %d\n",
                what, c.n_rows, c.n_features, c.n_repeats, c.n_proj, c.top_m, c.fht);
  }
  return CEOS_OK;
}

static int ceos_build_coceos_est_or_hash(ceos_index* h, int algo);

int ceos_build(ceos_index* h, const float* X) {
  ST_TRY(index_build_common(h, X, "Building CEOs index..."));
  Core& c = h->core;
  const int Cc = c.C();
  CUDA_TRY(c.dP.ensure((size_t)Cc * c.n_rows * 4));
  ProjArgs a = c.proj_base();
  a.n_rows = c.n_rows;
  a.out = c.dP.as<float>();
  a.ld_out = c.n_rows;
  CUDA_TRY(launch_project(a, PROJ_COLS, c.L, c.sms, c.stream));
  c.timer.mark("project");
  CUDA_TRY(cudaStreamSynchronize(c.stream));
  c.timer.finish();
  c.built = B_DENSE;
  print_timings("CEOs build", c.timer);
  return CEOS_OK;
}

// CEOs-Hash centering (opt-in `centering`): the reference subtracts the
// n-vector of row means from every d-dimensional row (src/CEOs.cpp:721-728,
// `matX.rowwise().mean()`), which does not type-check as a column centering.
// Here the rows are centered by the d-vector of column means, computed in a
// fixed order (double sums per chunk of kCenterChunk rows, chunks added in
// order, mean rounded to float), before the projection; the rerank then uses
// the centered rows, as the reference's does, so reported scores are
// q . (x - mean). Queries are not centered.
constexpr long kCenterChunk = 4096;

static int center_rows(Core& c) {
  const long n = c.n_rows;
  const int d = c.n_features;
  const long chunks = (n + kCenterChunk - 1) / kCenterChunk;
  DevBuf part, mu;
  CUDA_TRY(part.ensure((size_t)chunks * d * 8));
  CUDA_TRY(launch_col_partial_sums(c.dX.as<float>(), n, d, c.ldx, kCenterChunk, part.as<double>(), c.stream));
  std::vector<double> hp((size_t)chunks * d);
  CUDA_TRY(cudaMemcpyAsync(hp.data(), part.p, hp.size() * 8, cudaMemcpyDeviceToHost, c.stream));
  CUDA_TRY(cudaStreamSynchronize(c.stream));
  std::vector<float> hm(d);
  for (int j = 0; j < d; ++j) {
    double s = 0.0;
    for (long b = 0; b < chunks; ++b) s += hp[(size_t)b * d + j];
    hm[j] = (float)(s / (double)n);
  }
  CUDA_TRY(mu.ensure((size_t)d * 4));
  CUDA_TRY(cudaMemcpyAsync(mu.p, hm.data(), (size_t)d * 4, cudaMemcpyHostToDevice, c.stream));
  CUDA_TRY(launch_center_rows(c.dX.as<float>(), n, d, c.ldx, mu.as<float>(), c.stream));
  CUDA_TRY(cudaStreamSynchronize(c.stream));
  return CEOS_OK;
}

static int build_buckets_api(ceos_index* h, const float* X, int kind, const char* what) {
  ST_TRY(index_build_common(h, X, what));
  Core& c = h->core;
  if (kind == B_HASH && c.centering) {
    ST_TRY(center_rows(c));
    c.timer.mark("centering");
  }
  const int st = c.build_buckets();
  if (st != CEOS_OK) {
    c.timer.clear();
    c.release_all();
    return st;
  }
  CUDA_TRY(cudaStreamSynchronize(c.stream));
  c.timer.finish();
  c.built = kind;
  print_timings(kind == B_COCEOS ? "coCEOs-Est build" : "CEOs-Hash build", c.timer);
  return CEOS_OK;
}

static int ceos_build_coceos_est_or_hash(ceos_index* h, int algo) {
  return algo == CEOS_ALGO_COCEOS
             ? build_buckets_api(h, nullptr, B_COCEOS, "Building coCEOs-Estimate index...")
             : build_buckets_api(h, nullptr, B_HASH, "Building CEOs-Hash index...");
}

int ceos_build_coceos_est(ceos_index* h, const float* X) {
  return build_buckets_api(h, X, B_COCEOS, "Building coCEOs-Estimate index...");
}

int ceos_build_ceos_hash(ceos_index* h, const float* X) {
  return build_buckets_api(h, X, B_HASH, "Building CEOs-Hash index...");
}

int ceos_build_from_file(ceos_index* h, const char* path, int algo) {
  if (!path) return fail(CEOS_ERR_ARG, "null path");
  if (algo != CEOS_ALGO_DENSE && algo != CEOS_ALGO_COCEOS && algo != CEOS_ALGO_HASH)
    return fail(CEOS_ERR_ARG, "unknown algo %d", algo);
  g_build_path = path;
  const int st = algo == CEOS_ALGO_DENSE ? ceos_build(h, nullptr)
                                         : ceos_build_coceos_est_or_hash(h, algo);
  g_build_path = nullptr;
  return st;
}

// Reference validation order: n_probed_points first, then n_probed_vectors
// (src/CEOs.cpp:452-461).
static int check_query(const Core& c, int built_kind, int algo_needs_points, long nq, int k,
                       int s_limit) {
  if (c.built != built_kind) return fail(CEOS_ERR_NOT_BUILT, "index is not built for this search");
  if (nq < 0 || k < 0) return fail(CEOS_ERR_ARG, "n_queries and n_neighbors must be >= 0");
  if (algo_needs_points && (c.p > c.top_m))
    return fail(CEOS_ERR_PROBED_POINTS,
                "Number of probed points must be smaller than number of indexed top-m points");
  if (c.p < 0 && algo_needs_points) return fail(CEOS_ERR_ARG, "n_probed_points must be >= 0");
  if (c.s > s_limit)
    return fail(CEOS_ERR_PROBED_VECTORS,
                "Number of probed vectors must be smaller than n_proj * n_repeats");
  if (c.s < 0 || c.c < 0) return fail(CEOS_ERR_ARG, "n_probed_vectors and n_cand must be >= 0");
  if (k > 8192 || c.c > 65536)
    return fail(CEOS_ERR_UNSUPPORTED, "n_neighbors > 8192 or n_cand > 65536 is not supported");
  return CEOS_OK;
}


int ceos_search(ceos_index* h, const float* Q, int nq, int k, int verbose, int32_t* ids,
                float* dists) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  Core& c = h->core;
  ST_TRY(check_query(c, B_DENSE, 0, nq, k, c.C()));
  if (nq == 0 || k == 0) return CEOS_OK;
  if (!Q || !ids || !dists) return fail(CEOS_ERR_ARG, "null buffer");
  ST_TRY(c.ensure_device());
  ST_TRY(c.search_dense(Q, nq, k, ids, dists, false));
  if (verbose) print_timings("CEOs search", c.timer);
  return CEOS_OK;
}

int ceos_search_coceos_est(ceos_index* h, const float* Q, int nq, int k, int verbose,
                           int32_t* ids, float* dists) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  Core& c = h->core;
  ST_TRY(check_query(c, B_COCEOS, 1, nq, k, c.C()));
  if (nq == 0 || k == 0) return CEOS_OK;
  if (!Q || !ids || !dists) return fail(CEOS_ERR_ARG, "null buffer");
  ST_TRY(c.ensure_device());
  ST_TRY(c.search_buckets(Q_ESTIMATE, Q, nq, k, ids, dists, false, nullptr));
  if (verbose) print_timings("coCEOs-Est search", c.timer);
  return CEOS_OK;
}

int ceos_search_ceos_hash(ceos_index* h, const float* Q, int nq, int k, int verbose,
                          int32_t* ids, float* dists) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  Core& c = h->core;
  ST_TRY(check_query(c, B_HASH, 1, nq, k, c.C()));
  if (nq == 0 || k == 0) return CEOS_OK;
  if (!Q || !ids || !dists) return fail(CEOS_ERR_ARG, "null buffer");
  ST_TRY(c.ensure_device());
  ST_TRY(c.search_buckets(Q_UNION, Q, nq, k, ids, dists, false, nullptr));
  if (verbose) print_timings("CEOs-Hash search", c.timer);
  return CEOS_OK;
}

int ceos_search_device(ceos_index* h, int algo, const float* dQ, int nq, int k, int32_t* d_ids,
                       float* d_dists, void* cuda_stream) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  Core& c = h->core;
  const int kind = algo == CEOS_ALGO_DENSE ? B_DENSE : algo == CEOS_ALGO_COCEOS ? B_COCEOS
                   : algo == CEOS_ALGO_HASH ? B_HASH : -1;
  if (kind < 0) return fail(CEOS_ERR_ARG, "unknown algorithm %d", algo);
  ST_TRY(check_query(c, kind, kind != B_DENSE, nq, k, c.C()));
  if (nq == 0 || k == 0) return CEOS_OK;
  if (!dQ || !d_ids || !d_dists) return fail(CEOS_ERR_ARG, "null buffer");
  ST_TRY(c.ensure_device());
  cudaStream_t user = reinterpret_cast<cudaStream_t>(cuda_stream);
  if (user) {
    // order the index stream after the caller's prior work
    cudaEvent_t ev;
    CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CUDA_TRY(cudaEventRecord(ev, user));
    CUDA_TRY(cudaStreamWaitEvent(c.stream, ev, 0));
    cudaEventDestroy(ev);
  }
  if (kind == B_DENSE) {
    ST_TRY(c.search_dense(dQ, nq, k, d_ids, d_dists, true));
  } else {
    ST_TRY(c.search_buckets(kind == B_COCEOS ? Q_ESTIMATE : Q_UNION, dQ, nq, k, d_ids, d_dists,
                            true, user));
  }
  return CEOS_OK;
}

int ceos_get_buckets(const ceos_index* h, int32_t* ids, float* vals) {
  if (!h || !ids || !vals) return fail(CEOS_ERR_ARG, "null argument");
  const Core& c = h->core;
  if (c.built != B_COCEOS && c.built != B_HASH) return fail(CEOS_ERR_NOT_BUILT, "no buckets built");
  const size_t cnt = (size_t)c.C() * 2 * c.top_m;
  CUDA_TRY(cudaSetDevice(c.device));
  CUDA_TRY(cudaMemcpy(ids, c.dBids.p, cnt * 4, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(vals, c.dBvals.p, cnt * 4, cudaMemcpyDeviceToHost));
  if (c.built == B_HASH) std::memset(vals, 0, cnt * 4);
  return CEOS_OK;
}

int ceos_get_projections(const ceos_index* h, float* P) {
  if (!h || !P) return fail(CEOS_ERR_ARG, "null argument");
  const Core& c = h->core;
  if (c.built != B_DENSE) return fail(CEOS_ERR_NOT_BUILT, "dense index not built");
  const int Cc = c.C();
  std::vector<float> colmajor((size_t)Cc * c.n_rows);
  CUDA_TRY(cudaSetDevice(c.device));
  CUDA_TRY(cudaMemcpy(colmajor.data(), c.dP.p, colmajor.size() * 4, cudaMemcpyDeviceToHost));
  for (long i = 0; i < c.n_rows; ++i)
    for (int col = 0; col < Cc; ++col) P[i * Cc + col] = colmajor[(size_t)col * c.n_rows + i];
  return CEOS_OK;
}

int ceos_get_sign_bits(const ceos_index* h, uint8_t* bits) {
  if (!h || !bits) return fail(CEOS_ERR_ARG, "null argument");
  if (h->core.bits.empty()) return fail(CEOS_ERR_NOT_BUILT, "signs are generated at build");
  std::memcpy(bits, h->core.bits.data(), h->core.bits.size());
  return CEOS_OK;
}

int ceos_last_timings(const ceos_index* h, float* ms, int max_phases) {
  if (!h) return 0;
  const Timer& t = h->core.timer;
  int n = std::min((int)t.ms.size(), max_phases);
  for (int i = 0; i < n; ++i) ms[i] = t.ms[i];
  return n;
}

const char* ceos_timing_name(const ceos_index* h, int phase) {
  if (!h || phase < 0 || phase >= (int)h->core.timer.names.size()) return "";
  return h->core.timer.names[phase].c_str();
}

// ---------------------------------------------------------------------------
// streamCEOs

int ceos_stream_create(int n_features, ceos_stream** out) {
  if (!out) return fail(CEOS_ERR_ARG, "null output handle");
  *out = nullptr;
  if (n_features < 1) return fail(CEOS_ERR_ARG, "n_features must be >= 1");
  ceos_stream* h = new ceos_stream();
  h->core.n_features = n_features;
  h->core.set_param(256, 1, 100, -1, -1);  // class defaults, src/streamCEOs.h:19-24
  *out = h;
  return CEOS_OK;
}

void ceos_stream_destroy(ceos_stream* h) { delete h; }

int ceos_stream_set_index_param(ceos_stream* h, int n_proj, int n_repeats, int top_points,
                                int n_threads, int random_seed) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  if (n_proj < 1 || n_repeats < 1) return fail(CEOS_ERR_ARG, "n_proj and n_repeats must be >= 1");
  h->core.set_param(n_proj, n_repeats, top_points, n_threads, random_seed);
  h->core.s = top_points;  // n_probed_vectors = top_m (src/streamCEOs.h:58)
  return CEOS_OK;
}

int ceos_stream_set_precision(ceos_stream* h, int precision) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  if (precision != CEOS_PRECISION_FP32 && precision != CEOS_PRECISION_SPLIT_BF16)
    return fail(CEOS_ERR_ARG, "unknown precision %d", precision);
  h->core.precision = precision;
  return CEOS_OK;
}

int ceos_stream_set_threads(ceos_stream* h, int n_threads) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  h->core.n_threads = n_threads;
  return CEOS_OK;
}

int ceos_stream_clear(ceos_stream* h) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  if (h->core.device >= 0) cudaSetDevice(h->core.device);
  h->core.release_all();
  return CEOS_OK;
}

int ceos_stream_set_query_param(ceos_stream* h, int s, int p, int c) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  h->core.s = s;
  h->core.p = p;
  h->core.c = c;
  return CEOS_OK;
}

int ceos_stream_get_query_param(const ceos_stream* h, int* s, int* p, int* c) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (s) *s = h->core.s;
  if (p) *p = h->core.p;
  if (c) *c = h->core.c;
  return CEOS_OK;
}

int ceos_stream_build(ceos_stream* h, const float* X, int n_points) {
  if (!h || (!X && !g_build_path)) return fail(CEOS_ERR_ARG, "null argument");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  if (n_points < 1) return fail(CEOS_ERR_ARG, "n_points must be >= 1");
  Core& c = h->core;
  ST_TRY(c.check_param());
  ST_TRY(c.ensure_device());
  c.release_all();
  c.timer.begin(c.stream);
  c.n_rows = n_points;
  c.head = 0;
  c.cap_rows = n_points;
  CUDA_TRY(c.dX.ensure((size_t)c.cap_rows * c.ldx * 4));
  if (g_build_path)
    ST_TRY(c.upload_rows_from_file(g_build_path, c.n_rows, c.dX.as<float>()));
  else
    ST_TRY(c.upload_rows(X, c.n_rows, c.dX.as<float>()));
  ST_TRY(c.upload_signs());
  c.proj_tensor = (c.precision == CEOS_PRECISION_SPLIT_BF16 && project_tc_supported(c.L)) ? 1 : 0;
  c.timer.mark("h2d");
  if (log_level() >= 1)
    std::printf("n_features: %d\nn_proj: %d\ntop_m: %d\nfhtDim: %d\nn_points: %ld\n", c.n_features,
                c.n_proj, c.top_m, c.fht, c.n_rows);
  const int st = c.build_buckets();
  if (st != CEOS_OK) {
    c.timer.clear();
    c.release_all();
    return st;
  }
  if (c.reserve >= 0) {
    std::vector<int> cnt((size_t)c.C() * 2, c.stride());
    CUDA_TRY(c.dCnt.ensure(cnt.size() * 4));
    CUDA_TRY(cudaMemcpyAsync(c.dCnt.p, cnt.data(), cnt.size() * 4, cudaMemcpyHostToDevice, c.stream));
    CUDA_TRY(c.dTau.ensure(cnt.size() * sizeof(uint2)));
    CUDA_TRY(launch_init_tau(c.C(), c.stride(), c.n_rows, c.dBids.as<int>(), c.dBvals.as<float>(),
                             c.dTau.as<uint2>(), c.stream));
  }
  CUDA_TRY(cudaStreamSynchronize(c.stream));
  c.timer.finish();
  c.built = B_STREAM;
  print_timings("streamCEOs build", c.timer);
  return CEOS_OK;
}

int ceos_stream_update(ceos_stream* h, const float* Xn, int b, int n_del) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  return ceos_host::stream_update(h, Xn, b, n_del);
}

}  // extern "C"

int ceos_host::stream_update(ceos_stream* h, const float* Xn, int b, int n_del) {
  Core& c = h->core;
  if (c.built != B_STREAM) return fail(CEOS_ERR_NOT_BUILT, "streamCEOs is not built");
  if (b < 0 || n_del < 0) return fail(CEOS_ERR_ARG, "n_new and n_delPoints must be >= 0");
  if (b > 0 && !Xn) return fail(CEOS_ERR_ARG, "null new rows");
  const long cur = c.n_rows;
  if (n_del > cur)
    return fail(CEOS_ERR_UPDATE_DEL,
                "Number of removed points must be smaller than the current number of points");
  if ((long)c.top_m > cur + b - n_del)
    return fail(CEOS_ERR_UPDATE_TOPM, "There is not enough indexed top-points for coCEOs after update");
  ST_TRY(c.ensure_device());
  c.timer.begin(c.stream);
  const int Cc = c.C();
  // new rows, padded, and their projections [C][b]
  CUDA_TRY(c.wNewX.ensure((size_t)std::max(b, 1) * c.ldx * 4));
  ST_TRY(c.upload_rows(Xn, b, c.wNewX.as<float>()));
  c.timer.mark("h2d");
  if (b > 0) {
    CUDA_TRY(c.wNewP.ensure((size_t)Cc * b * 4));
    ProjArgs a = c.proj_base();
    a.X = c.wNewX.as<float>();
    a.head = 0;
    a.cap_rows = LONG_MAX;
    a.n_rows = b;
    a.out = c.wNewP.as<float>();
    a.ld_out = b;
    CUDA_TRY(launch_project(a, PROJ_COLS, c.L, c.sms, c.stream));
  }
  c.timer.mark("project");
  DevBuf flags;
  if (c.reserve >= 0) {
    CUDA_TRY(flags.ensure((size_t)Cc * 2 * 4));
    CUDA_TRY(launch_stream_merge_exact(Cc, c.stride(), c.top_m, c.wNewP.as<float>(), b, cur, n_del,
                                       c.dBids.as<int>(), c.dBvals.as<float>(), c.dCnt.as<int>(),
                                       c.dTau.as<uint2>(), flags.as<unsigned>(), c.stream));
  } else {
    CUDA_TRY(launch_stream_merge(Cc, c.top_m, c.wNewP.as<float>(), b, cur, n_del, c.dBids.as<int>(),
                                 c.dBvals.as<float>(), c.stream));
  }
  c.timer.mark("merge");
  // append the rows to the ring, growing it when full
  if (cur + b > c.cap_rows) {
    const long ncap = std::max(2 * c.cap_rows, cur + b);
    DevBuf nx;
    CUDA_TRY(nx.ensure((size_t)ncap * c.ldx * 4));
    const size_t rowb = (size_t)c.ldx * 4;
    const long first = std::min(cur, c.cap_rows - c.head);
    CUDA_TRY(cudaMemcpyAsync(nx.p, c.dX.as<float>() + c.head * c.ldx, first * rowb,
                             cudaMemcpyDeviceToDevice, c.stream));
    if (cur > first)
      CUDA_TRY(cudaMemcpyAsync(nx.as<float>() + first * c.ldx, c.dX.p, (cur - first) * rowb,
                               cudaMemcpyDeviceToDevice, c.stream));
    CUDA_TRY(cudaStreamSynchronize(c.stream));
    c.dX.swap(nx);
    nx.release();
    c.cap_rows = ncap;
    c.head = 0;
    c.dXb.release();
    c.xb_valid = false;
  }
  if (b > 0) {
    const size_t rowb = (size_t)c.ldx * 4;
    long pos = (c.head + cur) % c.cap_rows;
    const long first = std::min((long)b, c.cap_rows - pos);
    CUDA_TRY(cudaMemcpyAsync(c.dX.as<float>() + pos * c.ldx, c.wNewX.p, first * rowb,
                             cudaMemcpyDeviceToDevice, c.stream));
    if (b > first)
      CUDA_TRY(cudaMemcpyAsync(c.dX.p, c.wNewX.as<float>() + first * c.ldx, (b - first) * rowb,
                               cudaMemcpyDeviceToDevice, c.stream));
    if (c.xb_valid) {  // keep the bfloat16 copy of the ring current
      CUDA_TRY(launch_to_bf16(c.dX.as<float>() + pos * c.ldx, first * (long)c.ldx,
                              c.dXb.as<uint16_t>() + pos * c.ldx, c.stream));
      if (b > first)
        CUDA_TRY(launch_to_bf16(c.dX.as<float>(), (b - first) * (long)c.ldx, c.dXb.as<uint16_t>(),
                                c.stream));
    }
  }
  c.head = (c.head + n_del) % c.cap_rows;
  c.n_rows = cur + b - n_del;
  c.timer.mark("append");
  if (c.reserve >= 0) {  // lists that fell below top_m: refill from all live rows
    int refilled = 0;
    ST_TRY(c.exact_refill(flags.as<unsigned>(), (int)std::min<long>(c.stride(), c.n_rows), c.stride(),
                          c.dCnt.as<int>(), c.dTau.as<uint2>(), &refilled));
    c.refilled_columns = refilled;
    if (refilled) c.timer.mark("refill");
  }
  CUDA_TRY(cudaStreamSynchronize(c.stream));
  c.timer.finish();
  if (log_level() >= 1) {
    std::printf("n_points (after update): %ld\n", c.n_rows);
    print_timings("streamCEOs update", c.timer);
  }
  return CEOS_OK;
}

extern "C" {

static int stream_search(ceos_stream* h, int mode, const float* Q, int nq, int k, int verbose,
                         int32_t* ids, float* dists) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  Core& c = h->core;
  // streamCEOs limits n_probed_vectors by n_proj (src/streamCEOs.cpp:386-390)
  ST_TRY(check_query(c, B_STREAM, 1, nq, k, c.n_proj));
  if (nq == 0 || k == 0) return CEOS_OK;
  if (!Q || !ids || !dists) return fail(CEOS_ERR_ARG, "null buffer");
  ST_TRY(c.ensure_device());
  ST_TRY(c.search_buckets(mode, Q, nq, k, ids, dists, false, nullptr));
  if (verbose) print_timings(mode == Q_ESTIMATE ? "streamCEOs-est search" : "streamCEOs-hash search", c.timer);
  return CEOS_OK;
}

int ceos_stream_estimate_search(ceos_stream* h, const float* Q, int nq, int k, int verbose,
                                int32_t* ids, float* dists) {
  return stream_search(h, Q_ESTIMATE, Q, nq, k, verbose, ids, dists);
}

int ceos_stream_hash_search(ceos_stream* h, const float* Q, int nq, int k, int verbose,
                            int32_t* ids, float* dists) {
  return stream_search(h, Q_UNION, Q, nq, k, verbose, ids, dists);
}

int ceos_stream_size(const ceos_stream* h, int* n_points) {
  if (!h || !n_points) return fail(CEOS_ERR_ARG, "null argument");
  *n_points = (int)h->core.n_rows;
  return CEOS_OK;
}

int ceos_stream_get_buckets(const ceos_stream* h, int32_t* ids, float* vals) {
  if (!h || !ids || !vals) return fail(CEOS_ERR_ARG, "null argument");
  const Core& c = h->core;
  if (c.built != B_STREAM) return fail(CEOS_ERR_NOT_BUILT, "streamCEOs is not built");
  // the first top_m entries of each list (the bucket; lists hold stride() entries)
  const size_t rows = (size_t)c.C() * 2, w = (size_t)c.top_m * 4, ld = (size_t)c.stride() * 4;
  CUDA_TRY(cudaSetDevice(c.device));
  CUDA_TRY(cudaMemcpy2D(ids, w, c.dBids.p, ld, w, rows, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy2D(vals, w, c.dBvals.p, ld, w, rows, cudaMemcpyDeviceToHost));
  return CEOS_OK;
}

int ceos_stream_build_from_file(ceos_stream* h, const char* path, int n_points) {
  if (!path) return fail(CEOS_ERR_ARG, "null path");
  g_build_path = path;
  const int st = ceos_stream_build(h, nullptr, n_points);
  g_build_path = nullptr;
  return st;
}

int ceos_stream_set_reserve(ceos_stream* h, int reserve) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  if (h->core.built != B_NONE) return fail(CEOS_ERR_ARG, "set the reserve before build");
  if (reserve < -1) return fail(CEOS_ERR_ARG, "reserve must be >= -1");
  h->core.reserve = reserve;
  return CEOS_OK;
}

int ceos_stream_get_reserve(const ceos_stream* h, int* reserve) {
  if (!h || !reserve) return fail(CEOS_ERR_ARG, "null argument");
  *reserve = h->core.reserve;
  return CEOS_OK;
}

int ceos_stream_delete(ceos_stream* h, const int32_t* ids, int n_ids) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  return ceos_host::stream_delete(h, ids, n_ids);
}

}  // extern "C"

int ceos_host::stream_delete(ceos_stream* h, const int32_t* ids, int n_ids) {
  Core& c = h->core;
  if (c.built != B_STREAM) return fail(CEOS_ERR_NOT_BUILT, "streamCEOs is not built");
  if (c.reserve < 0)
    return fail(CEOS_ERR_ARG, "random deletes need exact maintenance: call set_reserve before build");
  if (n_ids < 0 || (n_ids > 0 && !ids)) return fail(CEOS_ERR_ARG, "bad id list");
  std::vector<int> del(ids, ids + n_ids);
  std::sort(del.begin(), del.end());
  del.erase(std::unique(del.begin(), del.end()), del.end());
  if (del.empty()) return CEOS_OK;
  if (del.front() < 0 || del.back() >= c.n_rows)
    return fail(CEOS_ERR_ARG, "ids must be in [0, %ld)", c.n_rows);
  const long nd = (long)del.size();
  if ((long)c.top_m > c.n_rows - nd)
    return fail(CEOS_ERR_UPDATE_TOPM, "There is not enough indexed top-points for coCEOs after delete");
  ST_TRY(c.ensure_device());
  c.timer.begin(c.stream);
  const int Cc = c.C(), M = c.stride();
  DevBuf dDel, flags, nx;
  CUDA_TRY(dDel.ensure((size_t)nd * 4));
  CUDA_TRY(cudaMemcpyAsync(dDel.p, del.data(), nd * 4, cudaMemcpyHostToDevice, c.stream));
  CUDA_TRY(flags.ensure((size_t)Cc * 2 * 4));
  CUDA_TRY(launch_stream_delete(Cc, M, c.top_m, dDel.as<int>(), (int)nd, c.dBids.as<int>(),
                                c.dBvals.as<float>(), c.dCnt.as<int>(), c.dTau.as<uint2>(),
                                flags.as<unsigned>(), c.stream));
  c.timer.mark("buckets");
  // compact the surviving rows into a fresh ring (same capacity, head 0)
  CUDA_TRY(nx.ensure((size_t)c.cap_rows * c.ldx * 4));
  CUDA_TRY(launch_compact_rows(c.dX.as<float>(), c.head, c.cap_rows, c.n_rows, c.ldx, dDel.as<int>(),
                               (int)nd, nx.as<float>(), c.stream));
  CUDA_TRY(cudaStreamSynchronize(c.stream));
  c.dX.swap(nx);
  nx.release();
  c.head = 0;
  c.n_rows -= nd;
  if (c.xb_valid) {
    CUDA_TRY(launch_to_bf16(c.dX.as<float>(), c.n_rows * (long)c.ldx, c.dXb.as<uint16_t>(), c.stream));
  }
  c.timer.mark("rows");
  int refilled = 0;
  ST_TRY(c.exact_refill(flags.as<unsigned>(), (int)std::min<long>(M, c.n_rows), M, c.dCnt.as<int>(),
                        c.dTau.as<uint2>(), &refilled));
  c.timer.mark("refill");
  CUDA_TRY(cudaStreamSynchronize(c.stream));
  c.timer.finish();
  c.refilled_columns = refilled;
  if (log_level() >= 1) {
    std::printf("n_points (after delete): %ld\nrefilled columns: %d\n", c.n_rows, refilled);
    print_timings("streamCEOs delete", c.timer);
  }
  return CEOS_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free search.
//
// Some callers cannot let this library call cudaMalloc: a host process that
// owns every byte of device memory through its own arena (a database or
// search-engine plugin host), or a latency-critical serving loop in which an
// allocation could stall the device or fail in the middle of a request. For
// them, ceos_search_coceos_est_device_noalloc takes its scratch (the padded
// queries, their projections and, when a query's hash table does not fit in
// shared memory, the per-CTA tables) from the fixed array below instead of
// allocating. The array is a file-scope __device__ object, so every GPU that
// loads this library holds it until the process exits.
constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;  // 64 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[128] = {};

// Device address of g_noalloc_scratch on `dev` (which must be current). In
// host code the symbol itself is only a host-side stand-in, so the address is
// looked up once per device with cudaGetSymbolAddress and cached.
int noalloc_scratch(int dev, void** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (dev < 0 || dev >= 128) return fail(CEOS_ERR_ARG, "device ordinal %d out of range", dev);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(CEOS_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return CEOS_OK;
}

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }
}  // namespace

extern "C" int ceos_search_coceos_est_device_noalloc(ceos_index* h, const float* d_Q, int nq,
                                                     int k, int32_t* d_ids, float* d_dists,
                                                     void* cuda_stream) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.attached) return fail(CEOS_ERR_BUSY, "the index is owned by a server");
  Core& c = h->core;
  ST_TRY(check_query(c, B_COCEOS, 1, nq, k, c.C()));
  if (nq == 0 || k == 0) return CEOS_OK;
  if (!d_Q || !d_ids || !d_dists) return fail(CEOS_ERR_ARG, "null buffer");
  CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = cuda_stream ? reinterpret_cast<cudaStream_t>(cuda_stream) : c.stream;
  // Scratch layout: padded queries | query projections | per-CTA hash tables.
  QueryArgs q;
  q.nq = nq;
  q.d = c.n_features;
  q.ldx = c.ldx;
  q.C = c.C();
  q.s = c.s;
  q.p = c.p;
  q.m = c.stride();
  q.c = c.c;
  q.k = k;
  q.X = c.dX.as<float>();
  q.head = c.head;
  q.cap_rows = c.cap_rows;
  q.n_points = c.n_rows;
  q.bids = c.dBids.as<int>();
  q.bvals = c.dBvals.as<float>();
  q.distinct_ids = 1;
  q.out_ids = d_ids;
  q.out_d = d_dists;
  if (c.precision == CEOS_PRECISION_SPLIT_BF16) {
    // The split form scans the bfloat16 row copy; making that copy allocates,
    // so this entry point only uses one that an earlier search already made.
    if (!c.xb_valid)
      return fail(CEOS_ERR_UNSUPPORTED,
                  "split-precision index without its bfloat16 row copy: run one allocating "
                  "split search (ceos_search_device or a host search) first");
    q.Xb = c.dXb.as<uint16_t>();
    q.rescore = 4 * k;
  }
  const long tc = table_capacity(c.s, c.p);
  if (tc < 0) return fail(CEOS_ERR_UNSUPPORTED, "n_probed_vectors * n_probed_points too large");
  q.table_cap = (int)tc;
  q.table_in_smem = 1;
  size_t smem = query_buckets_smem(q, Q_ESTIMATE);
  int per_sm;
  if (smem > c.smem_optin) {
    q.table_in_smem = 0;
    smem = query_buckets_smem(q, Q_ESTIMATE);
    if (smem > c.smem_optin)
      return fail(CEOS_ERR_UNSUPPORTED, "query working set exceeds shared memory");
  }
  per_sm = c.query_blocks_per_sm(Q_ESTIMATE, smem, q.table_in_smem != 0);
  const int grid = (int)std::max<long>(1, std::min<long>(nq, (long)c.sms * std::max(per_sm, 1)));
  const size_t qbytes = al256((size_t)nq * c.ldx * 4);
  const size_t pbytes = al256((size_t)nq * c.C() * 4);
  const size_t tbytes = q.table_in_smem ? 0 : (size_t)grid * tc * 8;
  const size_t need = qbytes + pbytes + tbytes;
  if (need > kNoAllocScratchBytes)
    return fail(CEOS_ERR_UNSUPPORTED,
                "this batch needs %zu bytes of scratch; the allocation-free search is limited to %zu "
                "bytes (n_queries * (n_features + n_proj * n_repeats) * 4 plus hash tables): split "
                "the batch",
                need, kNoAllocScratchBytes);
  void* base = nullptr;
  ST_TRY(noalloc_scratch(c.device, &base));
  unsigned char* sc = static_cast<unsigned char*>(base);
  float* qpad = reinterpret_cast<float*>(sc);
  float* qproj = reinterpret_cast<float*>(sc + qbytes);
  q.gtable = q.table_in_smem ? nullptr : reinterpret_cast<uint64_t*>(sc + qbytes + pbytes);
  q.Q = qpad;
  q.qproj = qproj;
  // Every buffer above is fully written before it is read (the hash tables
  // are reset per query inside the kernel), so no clearing is needed.
  CUDA_TRY(launch_pad_rows(d_Q, nq, c.n_features, qpad, c.ldx, st));
  ProjArgs a = c.query_proj_base();
  a.X = qpad;
  a.head = 0;
  a.cap_rows = LONG_MAX;
  a.n_rows = nq;
  a.out = qproj;
  CUDA_TRY(launch_project(a, PROJ_ROWS, c.L, c.sms, st));
  CUDA_TRY(launch_query_buckets(q, Q_ESTIMATE, grid, smem, st));
  return CEOS_OK;
}
