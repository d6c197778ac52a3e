// Two-ended top-m selection per projection column (the bucket build),
// src/CEOs.cpp:377-432 (coCEOs-Est), :779-831 (CEOs-Hash) and
// src/streamCEOs.cpp:88-150.
//
// The reference keeps two bounded min-heaps per column while scanning all n
// projections. Here the selection is split so that the full projection
// matrix is never stored:
//   1. sample thresholds: a strided sample of S rows is projected (PROJ_COLS)
//      and, per column, the rank-r_s value of each end is taken as a key
//      threshold (k_sample_thresholds). When S = n the threshold is exact.
//   2. the full projection runs in PROJ_EMIT mode, appending every value whose
//      key clears a threshold to that column end's candidate list.
//   3. k_finish_buckets picks the exact top-m of each candidate list (a
//      block-wide value-histogram select on packed (value, id) keys, then a
//      bitonic sort) and writes the bucket best first, as the reference pops
//      its heap into rows m-1 .. 0.
// A column end whose list came out short (< m) or overflowed is flagged; the
// host then dumps those full columns and k_exact_buckets selects them exactly.
#include "kernels.h"
#include "common.cuh"

namespace ceos {

__global__ void __launch_bounds__(256) k_sample_thresholds(const float* samp, long S, int rank,
                                                          uint32_t* th) {
  __shared__ uint32_t hist[256];
  __shared__ uint32_t scratch[8];
  const int c = blockIdx.x;
  const float* col = samp + (long)c * S;
  const uint32_t t_hi = block_radix_threshold<uint32_t>(
      [&](long i) { return fkey(col[i]); }, S, rank, hist, scratch);
  const uint32_t t_lo = block_radix_threshold<uint32_t>(
      [&](long i) { return fkey(-col[i]); }, S, rank, hist, scratch);
  if (threadIdx.x == 0) {
    th[2 * c] = t_hi;
    th[2 * c + 1] = t_lo;
  }
}

cudaError_t launch_sample_thresholds(const float* samp, long S, int C, int rank, uint32_t* th,
                                     cudaStream_t st) {
  k_sample_thresholds<<<C, 256, 0, st>>>(samp, S, rank, th);
  return cudaGetLastError();
}

// Dynamic shared memory of the per-column-end selections: sorted output
// (next_pow2(K) keys), the value histogram and the threshold-bin buffer.
constexpr int kSelMaybe = 1024;
static size_t sel_smem(int K) {
  int cap = 1;
  while (cap < K) cap <<= 1;
  return (size_t)cap * 8 + (size_t)kHistBins * 4 + (size_t)kSelMaybe * 8;
}

__global__ void __launch_bounds__(256) k_finish_buckets(const uint64_t* cand, const unsigned* cnt,
                                                       int cap, int m, int* bids, float* bvals,
                                                       unsigned* fail) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ uint32_t scratch[16];
  const int out_cap = next_pow2(m);
  uint64_t* s_out = reinterpret_cast<uint64_t*>(sm);
  uint32_t* hist = reinterpret_cast<uint32_t*>(sm + (size_t)out_cap * 8);
  uint64_t* maybe = reinterpret_cast<uint64_t*>(hist + kHistBins);
  const long ce = blockIdx.x;  // 2 * column + end
  const unsigned n = cnt[ce];
  if (n < (unsigned)m || n > (unsigned)cap) {
    if (threadIdx.x == 0) fail[ce] = 1u;
    return;
  }
  const uint64_t* list = cand + ce * cap;
  block_topk_hist_sorted(
      [&](long i, float& v, int& id) {
        const uint64_t k = list[i];
        v = key_val(k);
        id = key_id(k);
        return true;
      },
      (long)n, m, s_out, out_cap, hist, maybe, kSelMaybe, scratch);
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    const uint64_t k = s_out[i];
    bids[ce * m + i] = key_id(k);
    bvals[ce * m + i] = key_val(k);
  }
}

cudaError_t launch_finish_buckets(const uint64_t* cand, const unsigned* cnt, int cap, int C, int m,
                                  int* bids, float* bvals, unsigned* fail, cudaStream_t st) {
  const size_t smem = sel_smem(m);
  cudaError_t e =
      cudaFuncSetAttribute(k_finish_buckets, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_finish_buckets<<<2 * C, 256, smem, st>>>(cand, cnt, cap, m, bids, bvals, fail);
  return cudaGetLastError();
}

// Exact selection over a full dumped column (rows 0..n-1 of slot): the best
// m of the column end, written at stride `lds` (>= m) of the bucket lists,
// and m into cnt[column end] when cnt is given, with the list's completeness
// threshold (its last entry, or none when the list holds all n rows) into tau.
__global__ void __launch_bounds__(512) k_exact_buckets(const float* vals, long n, long ld,
                                                      const int* col_of_slot, const unsigned* fail,
                                                      int m, int lds, int* bids, float* bvals,
                                                      int* cnt, uint2* tau) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ uint32_t scratch[16];
  const int out_cap = next_pow2(m);
  uint64_t* s_out = reinterpret_cast<uint64_t*>(sm);
  uint32_t* hist = reinterpret_cast<uint32_t*>(sm + (size_t)out_cap * 8);
  uint64_t* maybe = reinterpret_cast<uint64_t*>(hist + kHistBins);
  const int slot = blockIdx.x >> 1;
  const int end = blockIdx.x & 1;
  const int col = col_of_slot[slot];
  const long ce = 2L * col + end;
  if (!fail[ce]) return;
  const float* v = vals + (long)slot * ld;
  block_topk_hist_sorted(
      [&](long i, float& x, int& id) {
        x = end ? -v[i] : v[i];
        id = (int)i;
        return true;
      },
      n, m, s_out, out_cap, hist, maybe, kSelMaybe, scratch);
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    const uint64_t k = s_out[i];
    bids[ce * lds + i] = key_id(k);
    bvals[ce * lds + i] = key_val(k);
  }
  if (cnt && threadIdx.x == 0) cnt[ce] = m;
  if (tau && threadIdx.x == 0)
    tau[ce] = (n > m) ? tau_of(key_val(s_out[m - 1]), key_id(s_out[m - 1])) : tau_none();
}

cudaError_t launch_exact_buckets(const float* vals, long n, long ld, int n_slots,
                                 const int* col_of_slot, const unsigned* fail, int m, int lds,
                                 int* bids, float* bvals, int* cnt, uint2* tau, cudaStream_t st) {
  const size_t smem = sel_smem(m);
  cudaError_t e =
      cudaFuncSetAttribute(k_exact_buckets, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_exact_buckets<<<2 * n_slots, 512, smem, st>>>(vals, n, ld, col_of_slot, fail, m, lds, bids,
                                                  bvals, cnt, tau);
  return cudaGetLastError();
}

// Thresholds of freshly built lists: the last of the M entries, or none when
// the list holds all n rows.
__global__ void k_init_tau(long n_ends, int M, long n, const int* bids, const float* bvals,
                           uint2* tau) {
  for (long ce = (long)blockIdx.x * blockDim.x + threadIdx.x; ce < n_ends;
       ce += (long)gridDim.x * blockDim.x)
    tau[ce] = n > M ? tau_of(bvals[ce * M + M - 1], bids[ce * M + M - 1]) : tau_none();
}

cudaError_t launch_init_tau(int C, int M, long n, const int* bids, const float* bvals, uint2* tau,
                            cudaStream_t st) {
  const long ends = 2L * C;
  k_init_tau<<<(unsigned)((ends + 255) / 256), 256, 0, st>>>(ends, M, n, bids, bvals, tau);
  return cudaGetLastError();
}

}  // namespace ceos
