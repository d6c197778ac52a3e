// streamCEOs::update bucket maintenance (src/streamCEOs.cpp:262-358).
//
// Per column end, the reference rebuilds its heap from
//   * every stored bucket row whose id survives the FIFO delete (id >= n_del),
//     stale rows included (rows that an earlier update could not refill keep
//     their old contents and are read back as-is), and
//   * the new points, with ids continuing after the pre-update size,
// keeps the best m, and writes them back best first with ids shifted by
// -n_del. When fewer than m items remain, only that many rows are rewritten
// and the rows after them keep their previous contents.
//
// GPU form: one CTA per (column, end); the survivors and the new points'
// projections (column-major [C][b]) form one key stream for the block top-m.
#include <cuda_bf16.h>

#include "kernels.h"
#include "common.cuh"

namespace ceos {

constexpr int kMergeMaybe = 1024;

__global__ void __launch_bounds__(512) k_stream_merge(int m, const float* newP, long b, long cur,
                                                     int n_del, int* bids, float* bvals) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ uint32_t scratch[16];
  const int out_cap = next_pow2(2 * m);
  uint64_t* s_out = reinterpret_cast<uint64_t*>(sm);
  uint32_t* hist = reinterpret_cast<uint32_t*>(sm + (size_t)out_cap * 8);
  uint64_t* maybe = reinterpret_cast<uint64_t*>(hist + kHistBins);
  const long ce = blockIdx.x;
  const int col = (int)(ce >> 1);
  const int end = (int)(ce & 1);
  int* ids = bids + ce * m;
  float* vals = bvals + ce * m;
  const float* np = newP + (long)col * b;
  auto get = [&](long i, float& v, int& id) -> bool {
    if (i < m) {
      id = ids[i];
      v = vals[i];
      return id >= n_del;
    }
    const long t = i - m;
    v = end ? -np[t] : np[t];
    id = (int)(cur + t);
    return true;
  };
  const int cnt = block_topk_hist_sorted<true>(get, (long)m + b, m, s_out, out_cap, hist, maybe,
                                         kMergeMaybe, scratch);
  // the sort ends with a barrier, so every read of ids/vals is done
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
    const uint64_t k = s_out[i];
    ids[i] = key_id(k) - n_del;
    vals[i] = key_val(k);
  }
}

cudaError_t launch_stream_merge(int C, int m, const float* newP, long b, long cur, int n_del,
                                int* bids, float* bvals, cudaStream_t st) {
  int out_cap = 1;
  while (out_cap < 2 * m) out_cap <<= 1;
  const size_t smem = (size_t)out_cap * 8 + (size_t)kHistBins * 4 + (size_t)kMergeMaybe * 8;
  cudaError_t e =
      cudaFuncSetAttribute(k_stream_merge, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_stream_merge<<<2 * C, 512, smem, st>>>(m, newP, b, cur, n_del, bids, bvals);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Exact maintenance (no reference counterpart): each column end keeps the exact
// best cnt (<= M = top_m + reserve) points of the live set, best first, and a
// completeness threshold tau: every live point outside the list ranks below
// tau. A random delete drops entries (tau stays valid). An update merges the
// entries surviving the FIFO delete with the new points and keeps those that
// rank at or above tau, since an unseen old point may beat a new point below
// it; a full list of M moves tau up to its last entry. A list that falls below
// top_m entries is flagged and refilled from all live points by the host
// (exact column dump).

__global__ void __launch_bounds__(512) k_stream_merge_exact(int M, int m, const float* newP, long b,
                                                           long cur, int n_del, int* bids,
                                                           float* bvals, int* cnt, uint2* tau,
                                                           unsigned* flag) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ uint32_t scratch[16];
  const int out_cap = next_pow2(M);
  uint64_t* s_out = reinterpret_cast<uint64_t*>(sm);
  uint32_t* hist = reinterpret_cast<uint32_t*>(sm + (size_t)out_cap * 8);
  uint64_t* maybe = reinterpret_cast<uint64_t*>(hist + kHistBins);
  const long ce = blockIdx.x;
  const int col = (int)(ce >> 1);
  const int end = (int)(ce & 1);
  int* ids = bids + ce * M;
  float* vals = bvals + ce * M;
  const int n_old = cnt[ce];
  const float* np = newP + (long)col * b;
  auto get = [&](long i, float& v, int& id) -> bool {
    if (i < n_old) {
      id = ids[i];
      v = vals[i];
      return id >= n_del;
    }
    const long t = i - n_old;
    v = end ? -np[t] : np[t];
    id = (int)(cur + t);
    return true;
  };
  const int got = block_topk_hist_sorted<true>(get, (long)n_old + b, M, s_out, out_cap, hist, maybe,
                                         kMergeMaybe, scratch);
  // the sorted result is certified up to its first entry below tau
  const uint2 t = tau[ce];
  __shared__ int first_below;
  if (threadIdx.x == 0) first_below = got;
  __syncthreads();
  for (int i = threadIdx.x; i < got; i += blockDim.x)
    if (!tau_certifies(t, key_val(s_out[i]), key_id(s_out[i]))) atomicMin(&first_below, i);
  __syncthreads();
  const int kept = first_below;
  for (int i = threadIdx.x; i < M; i += blockDim.x) {
    const uint64_t k = s_out[i];
    ids[i] = i < kept ? key_id(k) - n_del : -1;
    vals[i] = i < kept ? key_val(k) : 0.0f;
  }
  if (threadIdx.x == 0) {
    uint2 nt = t;
    if (kept == M) nt = tau_of(key_val(s_out[M - 1]), key_id(s_out[M - 1]));
    if (!tau_is_none(nt)) nt.y = (uint32_t)((int)nt.y - n_del);
    tau[ce] = nt;
    cnt[ce] = kept;
    flag[ce] = kept < m ? 1u : 0u;
  }
}

cudaError_t launch_stream_merge_exact(int C, int M, int m, const float* newP, long b, long cur,
                                      int n_del, int* bids, float* bvals, int* cnt, uint2* tau,
                                      unsigned* flag, cudaStream_t st) {
  int out_cap = 1;
  while (out_cap < M) out_cap <<= 1;
  const size_t smem = (size_t)out_cap * 8 + (size_t)kHistBins * 4 + (size_t)kMergeMaybe * 8;
  cudaError_t e = cudaFuncSetAttribute(k_stream_merge_exact,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_stream_merge_exact<<<2 * C, 512, smem, st>>>(M, m, newP, b, cur, n_del, bids, bvals, cnt, tau,
                                                 flag);
  return cudaGetLastError();
}

// Number of deleted ids (sorted, distinct) below id.
__device__ __forceinline__ int deleted_below(const int* del, int nd, int id) {
  int lo = 0, hi = nd;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (del[mid] < id) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(256) k_stream_delete(int M, int m, const int* del, int nd,
                                                      int* bids, float* bvals, int* cnt,
                                                      uint2* tau, unsigned* flag) {
  __shared__ int warp_sum[8];
  __shared__ int base_s;
  const long ce = blockIdx.x;
  int* ids = bids + ce * M;
  float* vals = bvals + ce * M;
  const int n = cnt[ce];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) base_s = 0;
  __syncthreads();
  // in-order compaction, one chunk of blockDim entries at a time; every output
  // position is at or before its input position and before the next chunk
  for (int c0 = 0; c0 < n; c0 += blockDim.x) {
    const int i = c0 + threadIdx.x;
    int id = -1;
    float v = 0.0f;
    bool keep = false;
    if (i < n) {
      id = ids[i];
      v = vals[i];
      const int below = deleted_below(del, nd, id);
      keep = !(below < nd && del[below] == id);
      id -= below;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) warp_sum[warp] = __popc(bal);
    __syncthreads();
    int off = base_s;
    for (int w = 0; w < warp; ++w) off += warp_sum[w];
    off += __popc(bal & ((1u << lane) - 1u));
    __syncthreads();  // every read of this chunk precedes the writes
    if (keep) {
      ids[off] = id;
      vals[off] = v;
    }
    if (threadIdx.x == blockDim.x - 1) {
      int tot = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += warp_sum[w];
      base_s += tot;
    }
    __syncthreads();
  }
  const int kept = base_s;
  for (int i = kept + threadIdx.x; i < n; i += blockDim.x) {
    ids[i] = -1;
    vals[i] = 0.0f;
  }
  if (threadIdx.x == 0) {
    uint2 t = tau[ce];
    if (!tau_is_none(t)) t.y = (uint32_t)((int)t.y - deleted_below(del, nd, (int)t.y));
    tau[ce] = t;
    cnt[ce] = kept;
    flag[ce] = kept < m ? 1u : 0u;
  }
}

cudaError_t launch_stream_delete(int C, int M, int m, const int* del, int nd, int* bids,
                                 float* bvals, int* cnt, uint2* tau, unsigned* flag,
                                 cudaStream_t st) {
  k_stream_delete<<<2 * C, 256, 0, st>>>(M, m, del, nd, bids, bvals, cnt, tau, flag);
  return cudaGetLastError();
}

// dst row j <- ring row (head + old_j) mod cap, old_j = j + #{deleted ids <= old_j}:
// with f(k) = del[k] - k non-decreasing (sorted distinct ids), the number of
// deleted ids below the j-th survivor is the count of k with f(k) <= j.
__global__ void k_compact_rows(const float4* X, long head, long cap, long n_new, int ldx4,
                               const int* del, int nd, float4* dst) {
  const long total = n_new * (long)ldx4;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long)gridDim.x * blockDim.x) {
    const long j = t / ldx4;
    const int c = (int)(t - j * ldx4);
    int lo = 0, hi = nd;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if ((long)del[mid] - mid <= j) lo = mid + 1; else hi = mid;
    }
    long r = head + j + lo;
    if (r >= cap) r -= cap;
    dst[t] = X[r * ldx4 + c];
  }
}

cudaError_t launch_compact_rows(const float* X, long head, long cap, long n, int ldx,
                                const int* del, int nd, float* dst, cudaStream_t st) {
  const long n_new = n - nd;
  if (n_new <= 0) return cudaSuccess;
  long blocks = (n_new * (ldx / 4) + 255) / 256;
  if (blocks > 8192) blocks = 8192;
  k_compact_rows<<<(unsigned)blocks, 256, 0, st>>>(reinterpret_cast<const float4*>(X), head, cap,
                                                   n_new, ldx / 4, del, nd,
                                                   reinterpret_cast<float4*>(dst));
  return cudaGetLastError();
}

// Column means for CEOs-Hash centering, in a fixed order: block b sums rows
// [b * chunk, (b + 1) * chunk) of every column sequentially in double; the
// host adds the per-chunk sums in chunk order.
__global__ void k_col_partial_sums(const float* X, long n, int d, int ldx, long chunk, double* partial) {
  const long r0 = (long)blockIdx.x * chunk;
  const long r1 = min(n, r0 + chunk);
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    double s = 0.0;
    for (long r = r0; r < r1; ++r) s += (double)X[r * ldx + j];
    partial[(long)blockIdx.x * d + j] = s;
  }
}

cudaError_t launch_col_partial_sums(const float* X, long n, int d, int ldx, long chunk, double* partial,
                                    cudaStream_t st) {
  const long blocks = (n + chunk - 1) / chunk;
  if (blocks <= 0) return cudaSuccess;
  k_col_partial_sums<<<(unsigned)blocks, 128, 0, st>>>(X, n, d, ldx, chunk, partial);
  return cudaGetLastError();
}

__global__ void k_center_rows(float* X, long n, int d, int ldx, const float* mu) {
  const long total = n * (long)d;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long r = i / d;
    const int j = (int)(i % d);
    X[r * ldx + j] -= mu[j];
  }
}

cudaError_t launch_center_rows(float* X, long n, int d, int ldx, const float* mu, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  long blocks = (n * d + 255) / 256;
  if (blocks > 8192) blocks = 8192;
  k_center_rows<<<(unsigned)blocks, 256, 0, st>>>(X, n, d, ldx, mu);
  return cudaGetLastError();
}

// Copy rows into a zero-padded row stride (ldx >= d, multiple of 4).
__global__ void k_pad_rows(const float* src, long n, int d, float* dst, int ldx) {
  const long total = n * (long)ldx;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long)gridDim.x * blockDim.x) {
    const long r = i / ldx;
    const int j = (int)(i % ldx);
    dst[i] = j < d ? src[r * d + j] : 0.0f;
  }
}

cudaError_t launch_pad_rows(const float* src, long n, int d, float* dst, int ldx, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  long blocks = (n * ldx + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  k_pad_rows<<<(unsigned)blocks, 256, 0, st>>>(src, n, d, dst, ldx);
  return cudaGetLastError();
}

// bfloat16 rows for the split-precision scan (round to nearest, ties to even).
__global__ void k_to_bf16(const float* src, long n, uint16_t* dst) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    dst[i] = __bfloat16_as_ushort(__float2bfloat16_rn(src[i]));
}

cudaError_t launch_to_bf16(const float* src, long n_elems, uint16_t* dst, cudaStream_t st) {
  if (n_elems <= 0) return cudaSuccess;
  long blocks = (n_elems + 255) / 256;
  if (blocks > 8192) blocks = 8192;
  k_to_bf16<<<(unsigned)blocks, 256, 0, st>>>(src, n_elems, dst);
  return cudaGetLastError();
}

}  // namespace ceos
