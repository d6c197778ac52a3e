// Exact maximum-inner-product ground truth in FP64 on the GPU, for recall.
//
// The reference's scripts take their ground truth from faiss IndexFlatIP
// (test/utils.py:35-55) and score recall as |exact ∩ approx| / k per query
// (test/utils.py:27-32). Here the inner products are computed in FP64: the
// product of two floats is exact in double, the sums are double, so the
// ranking is exact up to the order of the double additions. Ties are broken
// towards the smaller id.
//
// Two kernels per chunk of queries:
//   k_bf_scores : tiled X (n x d) . Q^T -> S [chunk][n] doubles (FP64 FMA);
//   k_bf_topk   : per query, the K-th largest score by a radix select over
//                 order-preserving 64-bit keys, then the keys above it plus the
//                 smallest-id ties, sorted.
#include "common.cuh"
#include "core.h"

using namespace ceos_host;

namespace {

constexpr int kRowsT = 128;  // rows per tile
constexpr int kQT = 32;      // queries per tile
constexpr int kDT = 32;      // feature chunk
constexpr int kTieCap = 4096;

__global__ void __launch_bounds__(256) k_bf_scores(const float* __restrict__ X, long n, int d,
                                                  const float* __restrict__ Q, int nq,
                                                  double* __restrict__ S) {
  __shared__ float xs[kRowsT][kDT + 1];
  __shared__ float qs[kQT][kDT + 1];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const long row0 = (long)blockIdx.x * kRowsT;
  const int q0 = blockIdx.y * kQT;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int d0 = 0; d0 < d; d0 += kDT) {
    for (int e = threadIdx.x; e < kRowsT * kDT; e += blockDim.x) {
      const int r = e / kDT, c = e % kDT;
      const long row = row0 + r;
      xs[r][c] = (row < n && d0 + c < d) ? X[row * d + d0 + c] : 0.0f;
    }
    for (int e = threadIdx.x; e < kQT * kDT; e += blockDim.x) {
      const int r = e / kDT, c = e % kDT;
      qs[r][c] = (q0 + r < nq && d0 + c < d) ? Q[(long)(q0 + r) * d + d0 + c] : 0.0f;
    }
    __syncthreads();
#pragma unroll 4
    for (int c = 0; c < kDT; ++c) {
      double xv[4], qv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) xv[i] = (double)xs[tx + 32 * i][c];
#pragma unroll
      for (int j = 0; j < 4; ++j) qv[j] = (double)qs[ty + 8 * j][c];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(xv[i], qv[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int q = q0 + ty + 8 * j;
    if (q >= nq) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long row = row0 + tx + 32 * i;
      if (row < n) S[(long)q * n + row] = acc[i][j];
    }
  }
}

__device__ __forceinline__ uint64_t dkey(double v) {
  const uint64_t u = (uint64_t)__double_as_longlong(v);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

// One block per query of the chunk: S row `blockIdx.x` (S already offset to
// the chunk's first query by the launch), results at out + blockIdx.x * K.
__global__ void __launch_bounds__(1024) k_bf_topk(const double* __restrict__ S, long n, int K,
                                                 int32_t* ids, double* scores, unsigned* overflow) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ uint32_t hist[256];
  __shared__ uint32_t scratch[16];
  double* lv = reinterpret_cast<double*>(sm);            // [K] values above the threshold
  int* li = reinterpret_cast<int*>(lv + K);               // [K] their ids
  int* ties = li + K;                                     // [kTieCap] ids at the threshold
  const double* s = S + (long)blockIdx.x * n;
  const long KK = min((long)K, n);
  const uint64_t T = block_radix_threshold<uint64_t>([&](long i) { return dkey(s[i]); }, n,
                                                     (int)KK, hist, scratch);
  if (threadIdx.x == 0) {
    scratch[8] = 0;
    scratch[9] = 0;
  }
  __syncthreads();
  for (long i = threadIdx.x; i < n; i += blockDim.x) {
    const uint64_t k = dkey(s[i]);
    if (k > T) {
      const uint32_t pos = atomicAdd(&scratch[8], 1u);
      if (pos < (uint32_t)K) {
        lv[pos] = s[i];
        li[pos] = (int)i;
      }
    } else if (k == T) {
      const uint32_t pos = atomicAdd(&scratch[9], 1u);
      if (pos < (uint32_t)kTieCap) ties[pos] = (int)i;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int na = (int)min(scratch[8], (uint32_t)K);
    const int nt = (int)min(scratch[9], (uint32_t)kTieCap);
    if (scratch[9] > (uint32_t)kTieCap || scratch[8] > (uint32_t)K) atomicAdd(overflow, 1u);
    // smallest-id ties fill the remaining places
    for (int a = 1; a < nt; ++a) {
      const int v = ties[a];
      int b = a - 1;
      while (b >= 0 && ties[b] > v) {
        ties[b + 1] = ties[b];
        --b;
      }
      ties[b + 1] = v;
    }
    for (int t = 0; t < nt && na < (int)KK; ++t) {
      lv[na] = s[ties[t]];
      li[na] = ties[t];
      ++na;
    }
    // sort by (score desc, id asc)
    for (int a = 1; a < na; ++a) {
      const double v = lv[a];
      const int id = li[a];
      int b = a - 1;
      while (b >= 0 && (lv[b] < v || (lv[b] == v && li[b] > id))) {
        lv[b + 1] = lv[b];
        li[b + 1] = li[b];
        --b;
      }
      lv[b + 1] = v;
      li[b + 1] = id;
    }
    for (int t = 0; t < K; ++t) {
      ids[(long)blockIdx.x * K + t] = t < na ? li[t] : 0;
      scores[(long)blockIdx.x * K + t] = t < na ? lv[t] : 0.0;
    }
  }
}

}  // namespace

extern "C" int ceos_bruteforce_fp64(const float* X, long n, int d, const float* Q, int nq, int k,
                                    int32_t* ids, double* scores) {
  if (!X || !Q || !ids || !scores) return fail(CEOS_ERR_ARG, "null argument");
  if (n < 1 || d < 1 || nq < 0 || k < 1) return fail(CEOS_ERR_ARG, "n, d, k must be >= 1 and nq >= 0");
  if (k > 1024) return fail(CEOS_ERR_UNSUPPORTED, "k > 1024 is not supported");
  if (n > INT_MAX) return fail(CEOS_ERR_UNSUPPORTED, "n > 2^31-1 is not supported");
  if (nq == 0) return CEOS_OK;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count < 1) {
    cudaGetLastError();
    return fail(CEOS_ERR_NO_DEVICE, "no CUDA device is visible; the brute-force oracle runs on the GPU");
  }
  cudaStream_t st;
  CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct Guard {
    cudaStream_t s;
    ~Guard() { cudaStreamDestroy(s); }
  } guard{st};
  DevBuf dX, dQ, dS, dI, dV, dOv;
  CUDA_TRY(dX.ensure((size_t)n * d * 4));
  CUDA_TRY(dQ.ensure((size_t)nq * d * 4));
  CUDA_TRY(cudaMemcpyAsync(dX.p, X, (size_t)n * d * 4, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(dQ.p, Q, (size_t)nq * d * 4, cudaMemcpyHostToDevice, st));
  // query chunk so that the score block stays near 4 GB
  const long chunk = std::max(1L, std::min<long>(nq, ((4L << 30) / ((long)n * 8)) / kQT * kQT));
  const long qc = std::max(chunk, (long)std::min(nq, kQT));
  CUDA_TRY(dS.ensure((size_t)qc * n * 8));
  CUDA_TRY(dI.ensure((size_t)nq * k * 4));
  CUDA_TRY(dV.ensure((size_t)nq * k * 8));
  CUDA_TRY(dOv.ensure(4));
  CUDA_TRY(cudaMemsetAsync(dOv.p, 0, 4, st));
  const size_t smem = (size_t)k * 12 + (size_t)kTieCap * 4;
  CUDA_TRY(cudaFuncSetAttribute(k_bf_topk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  for (long q0 = 0; q0 < nq; q0 += qc) {
    const int m = (int)std::min(qc, nq - q0);
    dim3 grid((unsigned)((n + kRowsT - 1) / kRowsT), (unsigned)((m + kQT - 1) / kQT));
    k_bf_scores<<<grid, 256, 0, st>>>(dX.as<float>(), n, d, dQ.as<float>() + q0 * d, m,
                                      dS.as<double>());
    CUDA_TRY(cudaGetLastError());
    k_bf_topk<<<m, 1024, smem, st>>>(dS.as<double>(), n, k, dI.as<int32_t>() + q0 * k,
                                     dV.as<double>() + q0 * k, dOv.as<unsigned>());
    CUDA_TRY(cudaGetLastError());
  }
  unsigned ov = 0;
  CUDA_TRY(cudaMemcpyAsync(ids, dI.p, (size_t)nq * k * 4, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(scores, dV.p, (size_t)nq * k * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(&ov, dOv.p, 4, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (ov) return fail(CEOS_ERR_DEVICE_LIMIT, "more than %d exactly tied scores at the k-th place", kTieCap);
  return CEOS_OK;
}
