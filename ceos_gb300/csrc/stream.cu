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
#include "kernels.h"
#include "common.cuh"

namespace ceos {

__global__ void __launch_bounds__(512) k_stream_merge(int m, const float* newP, long b, long cur,
                                                     int n_del, int* bids, float* bvals) {
  extern __shared__ __align__(16) uint64_t s_out[];
  __shared__ uint32_t hist[256];
  __shared__ uint32_t scratch[8];
  const long ce = blockIdx.x;
  const int col = (int)(ce >> 1);
  const int end = (int)(ce & 1);
  int* ids = bids + ce * m;
  float* vals = bvals + ce * m;
  const float* np = newP + (long)col * b;
  auto get = [&](long i) -> uint64_t {
    if (i < m) {
      const int id = ids[i];
      return id >= n_del ? pack_key(vals[i], id) : 0ull;
    }
    const long t = i - m;
    const float v = np[t];
    return pack_key(end ? -v : v, (int)(cur + t));
  };
  const int out_cap = next_pow2(2 * m);
  const int cnt = block_topk_sorted(get, (long)m + b, m, s_out, out_cap, hist, scratch);
  // block_topk_sorted ends with a barrier, so every read of ids/vals is done.
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
  const size_t smem = (size_t)out_cap * 8;
  cudaError_t e =
      cudaFuncSetAttribute(k_stream_merge, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_stream_merge<<<2 * C, 512, smem, st>>>(m, newP, b, cur, n_del, bids, bvals);
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

}  // namespace ceos
