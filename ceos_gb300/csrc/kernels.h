// Launch interface between the host layer (capi.cu) and the kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ceos {

enum ProjMode { PROJ_ROWS = 0, PROJ_COLS = 1, PROJ_EMIT = 2 };

struct ProjArgs {
  // input rows: row `i` of the work list is X[((row_map ? row_map[i] : i) + head) mod cap_rows]
  const float* X = nullptr;
  long ldx = 0;
  const long* row_map = nullptr;
  long n_rows = 0;
  long head = 0;
  long cap_rows = 0;
  int d = 0, D = 0, R = 0;
  const uint32_t* signs = nullptr;  // [R][3][max(F/32,1)] words, bit j set => +1
  // PROJ_ROWS: out[row * R*D + col]; PROJ_COLS: out[slot * ld_out + row]
  float* out = nullptr;
  long ld_out = 0;
  const int* col_slot = nullptr;  // PROJ_COLS: column -> output slot (-1 = skip); null = identity
  // PROJ_EMIT
  const uint32_t* th = nullptr;  // [C][2] key thresholds (close: fkey(v), far: fkey(-v))
  // [C] float prefilter of th: a value v can clear the close end only if
  // v >= thf.x and the far end only if v <= thf.y (see emit_bounds)
  const float2* thf = nullptr;
  unsigned* cnt = nullptr;       // [C][2] candidate counters
  uint64_t* cand = nullptr;      // [C][2][cap] packed keys
  int cap = 0;
  long id_base = 0;
  const unsigned char* col_active = nullptr;  // optional per-column enable
  // 1 = split-precision tensor-core transform (project_tc.cu) where supported
  int tensor = 0;
};

cudaError_t launch_project(const ProjArgs& a, int mode, int L, int num_sms, cudaStream_t st);
// Split-precision tensor-core projection (fhtDim 256 and 1024).
bool project_tc_supported(int L);
cudaError_t launch_project_tc(const ProjArgs& a, int mode, int L, int num_sms, cudaStream_t st);
// fhtDim 1024 on tcgen05 (project_t5.cu); project_t5_take_faults returns and
// clears the number of CTAs whose bounded waits gave up (-1 on a CUDA error),
// synchronizing the stream.
cudaError_t launch_project_t5(const ProjArgs& a, int mode, cudaStream_t st, int num_sms);
int project_t5_take_faults(cudaStream_t st);
// test hook: polls > 0 makes the following launches issue no products and
// give up each wait after `polls` polls (0: normal operation)
void project_t5_set_stall(int polls);

// ---- selection (select.cu) ----
// Per column of the row-major sample samp[S][C]: u32 key thresholds, the lower
// edge of the 16-bit key prefix holding each end's rank-`rank` key (so at least
// `rank` sampled values pass), and their float prefilter bounds (thf, see
// ProjArgs::thf).
cudaError_t launch_sample_thresholds(const float* samp, long S, int C, int rank, uint32_t* th,
                                     float2* thf, cudaStream_t st);
// Per column end: top-m of the emitted candidates -> buckets; flags failures.
cudaError_t launch_finish_buckets(const uint64_t* cand, const unsigned* cnt, int cap, int C, int m,
                                  int* bids, float* bvals, unsigned* fail, cudaStream_t st);
// Exact top-m of dumped full columns (fallback / refill): vals [slots][ld] -> the
// flagged ends of col_of_slot's bucket lists (stride lds), cnt[end] = m and the
// completeness threshold tau[end] if given.
cudaError_t launch_exact_buckets(const float* vals, long n, long ld, int n_slots,
                                 const int* col_of_slot, const unsigned* fail, int m, int lds,
                                 int* bids, float* bvals, int* cnt, uint2* tau, cudaStream_t st);
// Completeness thresholds of freshly built lists of M entries over n rows.
cudaError_t launch_init_tau(int C, int M, long n, const int* bids, const float* bvals, uint2* tau,
                            cudaStream_t st);

// ---- queries (query.cu) ----
struct QueryArgs {
  const float* Q = nullptr;  // [nq][ldx] (zero padded) device queries
  const float* qproj = nullptr;  // [nq][C]
  int nq = 0, d = 0, ldx = 0, C = 0;
  int s = 0, p = 0, m = 0, c = 0, k = 0;
  const float* X = nullptr;  // ring of rows, stride ldx
  long head = 0, cap_rows = 0;
  long n_points = 0;
  const int* bids = nullptr;    // [C][2][m]
  const float* bvals = nullptr; // [C][2][m]
  const float* P = nullptr;     // dense CEOs-Est projections [C][n]
  // split precision: bfloat16 copy of the rows (same ring layout, stride ldx)
  // and the number of scan winners rescored in FP32 (0 = plain FP32 rerank)
  const uint16_t* Xb = nullptr;
  int rescore = 0;
  // with per-query k (q_k), query q rescores rescore_per_k * k_q (<= rescore)
  int rescore_per_k = 0;
  int* out_ids = nullptr;
  float* out_d = nullptr;
  // optional per-query parameters (serving batches that mix requests): probes
  // s_q <= s, neighbours k_q <= k, and the offset of query q's k_q results in
  // out_ids / out_d. Null = every query uses s and k at offset q * k.
  const int* q_s = nullptr;
  const int* q_k = nullptr;
  const long* q_off = nullptr;
  const int* q_cap = nullptr;  // per-query hash-table capacity (<= table_cap)
  // optional device-side query count (graph replays of a fixed-capacity batch)
  const int* d_nq = nullptr;
  // 1 when every bucket column holds distinct ids (CEOs / coCEOs indexes); a
  // streamCEOs index can keep stale rows that repeat an id within a column
  int distinct_ids = 0;
  // hash table (estimate / union), in shared memory when table_in_smem
  int table_cap = 0;
  int table_in_smem = 0;
  uint64_t* gtable = nullptr;   // [grid][table_cap] workspace when not in smem
  // dense path
  const int* probes = nullptr;  // [nq][s] tags in pop order
  float* est = nullptr;         // [nq][n]
  int* probes_out = nullptr;
  // sort-based estimate accumulation (k_query_sorted): 2 x grid x sort_cap
  // (id, value) pairs, every CTA's first buffer, then every CTA's second;
  // ids below 2^id_bits
  int2* sort_scratch = nullptr;
  long sort_cap = 0;
  int id_bits = 0;
};

enum QueryMode { Q_ESTIMATE = 0, Q_UNION = 1 };

cudaError_t launch_query_buckets(const QueryArgs& a, int mode, int grid, size_t smem, cudaStream_t st);
// Sort-based coCEOs-Est search (distinct ids per column): the probed (id, value)
// pairs ordered by id (one stable scatter into 1024-id partitions summed in
// per-warp shared-memory tables when ids are below 2^20, else a stable LSD radix
// sort and run sums), every sum taken in probe order; top-c, rerank, top-k.
cudaError_t launch_query_sorted(const QueryArgs& a, int grid, size_t smem, cudaStream_t st);
size_t query_sorted_smem(const QueryArgs& a);
int query_sorted_blocks_per_sm(size_t smem);
// true when the estimate search is faster with its hash table in shared memory
// (two CTAs per SM) than sorted; a.table_cap must be set
bool query_table_preferred(const QueryArgs& a);
size_t query_buckets_smem(const QueryArgs& a, int mode);
int query_buckets_blocks_per_sm(int mode, size_t smem, bool table_in_smem);
cudaError_t launch_probe_select(const QueryArgs& a, cudaStream_t st);
cudaError_t launch_dense_estimate(const QueryArgs& a, int q0, int nq_chunk, cudaStream_t st);
cudaError_t launch_dense_select_rerank(const QueryArgs& a, int q0, int nq_chunk, cudaStream_t st);

// ---- streaming (stream.cu) ----
cudaError_t launch_stream_merge(int C, int m, const float* newP, long b, long cur, int n_del,
                                int* bids, float* bvals, cudaStream_t st);
// Exact maintenance (lists of up to M = top_m + reserve entries, cnt valid per end,
// completeness threshold tau per end): merge the entries surviving the FIFO delete
// with the new points, keep the best M that rank at or above tau; flag[end] = 1
// when fewer than m remain.
cudaError_t launch_stream_merge_exact(int C, int M, int m, const float* newP, long b, long cur,
                                      int n_del, int* bids, float* bvals, int* cnt, uint2* tau,
                                      unsigned* flag, cudaStream_t st);
// Random deletes: drop entries whose id is in del (sorted, distinct, nd ids), shift
// the other ids down by the number of deleted ids below them, keep list order;
// flag[end] = 1 when fewer than m remain.
cudaError_t launch_stream_delete(int C, int M, int m, const int* del, int nd, int* bids,
                                 float* bvals, int* cnt, uint2* tau, unsigned* flag,
                                 cudaStream_t st);
// Row compaction of the ring after random deletes: dst row j (stride ldx) = the
// j-th surviving row of the ring (head, cap) of n rows.
cudaError_t launch_compact_rows(const float* X, long head, long cap, long n, int ldx,
                                const int* del, int nd, float* dst, cudaStream_t st);

// ---- CEOs-Hash centering (stream.cu) ----
// per-chunk column sums in double, rows [b*chunk, (b+1)*chunk) summed in order
cudaError_t launch_col_partial_sums(const float* X, long n, int d, int ldx, long chunk, double* partial,
                                    cudaStream_t st);
cudaError_t launch_center_rows(float* X, long n, int d, int ldx, const float* mu, cudaStream_t st);

// ---- misc ----
cudaError_t launch_pad_rows(const float* src, long n, int d, float* dst, int ldx, cudaStream_t st);
// bfloat16 copy (round to nearest even) of n rows of stride ldx
cudaError_t launch_to_bf16(const float* src, long n_elems, uint16_t* dst, cudaStream_t st);

}  // namespace ceos
