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
  const int cnt = block_topk_hist_sorted(get, (long)m + b, m, s_out, out_cap, hist, maybe,
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
