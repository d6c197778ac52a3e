// Two-ended top-m selection per projection column (the bucket build),
// src/CEOs.cpp:377-432 (coCEOs-Est), :779-831 (CEOs-Hash) and
// src/streamCEOs.cpp:88-150.
//
// The reference keeps two bounded min-heaps per column while scanning all n
// projections. Here the selection is split so that the full projection
// matrix is never stored:
//   1. sample thresholds: a strided sample of S rows is projected (PROJ_ROWS)
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

// Sample thresholds. The S sampled rows' projections arrive row-major
// (samp[i * C + col], coalesced writes from the projection). One block owns 32
// adjacent columns: lane l of every warp handles column c0 + l, and warp w of
// kThWarps reads rows w, w + kThWarps, ..., so each warp load is one 128-byte
// line. Every 8-bit digit pass builds, per column, the histograms of both
// ends at once: the close end ranks k = fkey(v), the far end fkey(-v) = ~k.
// Histograms are
// per column (padded to 257 bins, so lanes on equal digits hit different
// banks); lanes of a warp never share a column, so increments only collide
// across warps. The threshold of an end is the lower edge of the 16-bit key
// prefix that holds its rank-`rank` key from the top (every key when
// S <= rank). Which threshold a column gets changes how many candidates the
// emission pass appends, never the selected buckets.
constexpr int kThCols = 32;
constexpr int kThWarps = 32;
constexpr int kThBins = 257;

__global__ void __launch_bounds__(kThWarps * 32) k_sample_thresholds(const float* samp, long S,
                                                                    int C, int rank, uint32_t* th,
                                                                    float2* thf) {
  extern __shared__ __align__(16) uint32_t s_hist[];  // [2][kThCols][kThBins]
  __shared__ uint32_t s_prefix[2][kThCols], s_remaining[2][kThCols], s_done[2][kThCols];
  __shared__ uint32_t s_scratch[2][kThCols][4];
  __shared__ int s_all_done;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c0 = blockIdx.x * kThCols;
  const int col = c0 + lane;
  const bool all = rank <= 0 || S <= rank;  // every sampled key passes
  if (threadIdx.x < 2 * kThCols) {
    const int end = threadIdx.x / kThCols, c = threadIdx.x % kThCols;
    s_prefix[end][c] = 0u;
    s_remaining[end][c] = (uint32_t)(rank > 0 ? rank : 0);
    s_done[end][c] = (all || c0 + c >= C) ? 1u : 0u;
  }
  if (threadIdx.x == 0) s_all_done = all ? 1 : 0;
  __syncthreads();
  uint32_t mask = 0u;
  // two digit passes: the threshold is the lower edge of the 16-bit key prefix
  // holding the rank-`rank` key (a column end that resolves in the first pass
  // gets its exact key), so at least `rank` sampled keys clear it
  for (int shift = 24; shift >= 16 && !s_all_done; shift -= 8) {
    for (int b = threadIdx.x; b < 2 * kThCols * kThBins; b += blockDim.x) s_hist[b] = 0u;
    __syncthreads();
    const bool act0 = !s_done[0][lane], act1 = !s_done[1][lane];
    const uint32_t p0 = s_prefix[0][lane], p1 = s_prefix[1][lane];
    uint32_t* h0 = s_hist + lane * kThBins;
    uint32_t* h1 = s_hist + (kThCols + lane) * kThBins;
    if (col < C && (act0 || act1)) {
      const float* src = samp + col;
      for (long i = warp; i < S; i += kThWarps) {
        const uint32_t k = fkey(__ldg(src + i * C));
        if (act0 && (k & mask) == p0) atomicAdd(h0 + ((k >> shift) & 255u), 1u);
        if (act1 && (~k & mask) == p1) atomicAdd(h1 + ((~k >> shift) & 255u), 1u);
      }
    }
    __syncthreads();
    // warp w scans columns w, w + kThWarps, ..., both ends
    for (int c = warp; c < kThCols; c += kThWarps)
      for (int end = 0; end < 2; ++end)
        if (!s_done[end][c])
          radix_scan_hist(s_hist + (end * kThCols + c) * kThBins, s_remaining[end][c],
                          s_scratch[end][c]);
    __syncthreads();
    if (threadIdx.x < 2 * kThCols) {
      const int end = threadIdx.x / kThCols, c = threadIdx.x % kThCols;
      if (!s_done[end][c]) {
        // the histogram held every remaining key of this end and more than
        // `remaining` of them, so a bin was found
        const uint32_t* sc = s_scratch[end][c];
        s_prefix[end][c] |= sc[0] << shift;
        s_remaining[end][c] -= sc[1];
        if (sc[2] == s_remaining[end][c]) s_done[end][c] = 1u;
      }
    }
    mask |= 255u << shift;
    __syncthreads();
    if (threadIdx.x == 0) {
      int d = 1;
      for (int c = 0; c < 2 * kThCols; ++c) d &= (int)s_done[c / kThCols][c % kThCols];
      s_all_done = d;
    }
    __syncthreads();
  }
  if (warp == 0 && col < C) {
    const uint2 t = all ? make_uint2(0u, 0u) : make_uint2(s_prefix[0][lane], s_prefix[1][lane]);
    th[2 * col] = t.x;
    th[2 * col + 1] = t.y;
    thf[col] = emit_bounds(t);
  }
}

cudaError_t launch_sample_thresholds(const float* samp, long S, int C, int rank, uint32_t* th,
                                     float2* thf, cudaStream_t st) {
  const size_t smem = (size_t)2 * kThCols * kThBins * 4;
  cudaError_t e = cudaFuncSetAttribute(k_sample_thresholds,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_sample_thresholds<<<(C + kThCols - 1) / kThCols, kThWarps * 32, smem, st>>>(samp, S, C, rank,
                                                                              th, thf);
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
  block_topk_hist_sorted<true>(
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
  block_topk_hist_sorted<true>(
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
