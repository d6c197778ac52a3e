// Query kernels.
//
//  k_query_buckets<Q_ESTIMATE>: coCEOs-Est / streamCEOs.estimate_search
//     (src/CEOs.cpp:450-694, src/streamCEOs.cpp:378-612)
//  k_query_buckets<Q_UNION>   : CEOs-Hash / streamCEOs.hash_search
//     (src/CEOs.cpp:850-1066, src/streamCEOs.cpp:621-877)
//  k_probe_select + k_dense_estimate + k_dense_select_rerank: CEOs-Est
//     (src/CEOs.cpp:107-297)
//
// One CTA owns one query at a time (persistent grid, queries strided by
// gridDim.x). Per query:
//  1. probe selection: the s columns of largest |projection| (abs computed as
//     the reference does: v < 0 ? -v : v), tagged +-(col+1), consumed in the
//     reference's heap pop order (worst first) - the order the estimate sums
//     are accumulated in.
//  2. estimate: for each probed column in that order, its first p bucket
//     entries are accumulated into an open-addressing hash table keyed by
//     point id (in shared memory when it fits, else in a per-CTA L2-resident
//     workspace). Within one column the ids are distinct, so each table
//     value receives its terms in exactly the reference's order; a barrier
//     separates columns. Values start at -0.0, so the first addition
//     reproduces the reference's "assign on first sight".
//  3. top-c candidates by estimate (block radix select on packed keys).
//  4. exact rerank: one thread per candidate computes the inner product as a
//     sequential FMA chain over the row, then the block selects the top-k,
//     written best first with zero fill past the number of results
//     (src/CEOs.cpp:659-666).
#include "kernels.h"
#include "common.cuh"

namespace ceos {

constexpr int kQueryThreads = 512;
constexpr uint64_t kEmptySlot = (0x80000000ull << 32) | 0xffffffffull;  // id -1, value -0.0

CEOS_DEV float abs_ref(float v) { return v < 0 ? -v : v; }

CEOS_DEV const float* row_ptr(const QueryArgs& a, int id) {
  long r = a.head + id;
  if (r >= a.cap_rows) r -= a.cap_rows;
  return a.X + r * (long)a.ldx;
}

// Sequential FMA inner product over ldx (multiple of 4) floats; padding
// columns are zero on both sides and leave the sum unchanged.
CEOS_DEV float dot_seq(const float* __restrict__ q, const float* __restrict__ x, int ldx) {
  const float4* x4 = reinterpret_cast<const float4*>(x);
  const float4* q4 = reinterpret_cast<const float4*>(q);
  float s = 0.0f;
  for (int j = 0; j < (ldx >> 2); ++j) {
    const float4 xv = __ldg(x4 + j);
    const float4 qv = q4[j];
    s = __fmaf_rn(qv.x, xv.x, s);
    s = __fmaf_rn(qv.y, xv.y, s);
    s = __fmaf_rn(qv.z, xv.z, s);
    s = __fmaf_rn(qv.w, xv.w, s);
  }
  return s;
}

CEOS_DEV int slot_id(uint64_t w) { return (int)(uint32_t)(w & 0xffffffffu); }
CEOS_DEV float slot_val(uint64_t w) { return __uint_as_float((uint32_t)(w >> 32)); }

// Find or insert `id`; returns the slot index. The capacity exceeds the
// number of insertions, so a free slot always exists; the probe sequence is
// still bounded by the capacity and returns -1 if it ever ran out.
CEOS_DEV int table_slot(uint64_t* t, int cap, int id) {
  const uint32_t h = (uint32_t)id * 0x9E3779B1u;
  int s = (int)(((uint64_t)h * (uint32_t)cap) >> 32);
  int* keys = reinterpret_cast<int*>(t);
  for (int probe = 0; probe < cap; ++probe) {
    const int cur = *reinterpret_cast<volatile int*>(&keys[2 * s]);
    if (cur == id) return s;
    if (cur == -1) {
      const int prev = atomicCAS(&keys[2 * s], -1, id);
      if (prev == -1 || prev == id) return s;
    }
    s = (s + 1 == cap) ? 0 : s + 1;
  }
  return -1;
}

struct QLayout {
  size_t qv, pkeys, probes, topk, cand, region, total;
};

__host__ __device__ inline int np2(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline QLayout q_layout(const QueryArgs& a, int mode) {
  QLayout L;
  size_t o = 0;
  L.qv = o;
  o = al16(o + (size_t)a.ldx * 4);
  L.pkeys = o;
  o = al16(o + (size_t)np2(a.s > 0 ? a.s : 1) * 8);
  L.probes = o;
  o = al16(o + (size_t)(a.s > 0 ? a.s : 1) * 4);
  L.topk = o;
  o = al16(o + (size_t)np2(a.k > 0 ? a.k : 1) * 8);
  L.cand = o;
  if (mode == Q_ESTIMATE) o = al16(o + (size_t)(a.c > 0 ? a.c : 1) * 4);
  L.region = o;
  size_t region = 0;
  if (a.table_in_smem) region = (size_t)a.table_cap * 8;
  if (mode == Q_ESTIMATE) {
    const size_t rk = (size_t)np2(a.c > 0 ? a.c : 1) * 8;
    if (rk > region) region = rk;
  }
  o = al16(o + region);
  L.total = o;
  return L;
}

size_t query_buckets_smem(const QueryArgs& a, int mode) { return q_layout(a, mode).total; }

template <int MODE>
__global__ void __launch_bounds__(kQueryThreads) k_query_buckets(QueryArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ uint32_t hist[256];
  __shared__ uint32_t scratch[8];
  const QLayout Lq = q_layout(a, MODE);
  float* qv = reinterpret_cast<float*>(sm + Lq.qv);
  uint64_t* pkeys = reinterpret_cast<uint64_t*>(sm + Lq.pkeys);
  int* probes = reinterpret_cast<int*>(sm + Lq.probes);
  uint64_t* topk = reinterpret_cast<uint64_t*>(sm + Lq.topk);
  int* cand = reinterpret_cast<int*>(sm + Lq.cand);
  uint64_t* region = reinterpret_cast<uint64_t*>(sm + Lq.region);
  uint64_t* table = a.table_in_smem ? region : a.gtable + (long)blockIdx.x * a.table_cap;
  const int cap = a.table_cap;
  const int s_cap = np2(a.s > 0 ? a.s : 1);
  const int k_cap = np2(a.k > 0 ? a.k : 1);

  for (int q = blockIdx.x; q < a.nq; q += gridDim.x) {
    for (int j = threadIdx.x; j < a.ldx; j += blockDim.x) qv[j] = a.Q[(long)q * a.ldx + j];
    // ---- 1. probes ----
    const float* qp = a.qproj + (long)q * a.C;
    const int ns = block_topk_sorted([&](long i) { return pack_key(abs_ref(qp[i]), (int)i); },
                                     (long)a.C, a.s, pkeys, s_cap, hist, scratch);
    for (int j = threadIdx.x; j < ns; j += blockDim.x) {
      const int col = key_id(pkeys[ns - 1 - j]);
      probes[j] = qp[col] < 0 ? -(col + 1) : (col + 1);
    }
    for (int i = threadIdx.x; i < cap; i += blockDim.x) table[i] = kEmptySlot;
    __syncthreads();
    // ---- 2. estimate / union ----
    for (int j = 0; j < ns; ++j) {
      const int tag = probes[j];
      const int col = (tag < 0 ? -tag : tag) - 1;
      const long base = (2L * col + (tag < 0 ? 1 : 0)) * a.m;
      for (int e = threadIdx.x; e < a.p; e += blockDim.x) {
        const int id = __ldg(a.bids + base + e);
        // streamCEOs can keep stale bucket rows whose id is no longer a live
        // point; they are skipped (the reference reads out of range there).
        if ((unsigned)id >= (unsigned long)a.n_points) continue;
        const int sl = table_slot(table, cap, id);
        if (sl < 0) continue;
        if (MODE == Q_ESTIMATE) {
          const float v = __ldg(a.bvals + base + e);
          atomicAdd(reinterpret_cast<float*>(&table[sl]) + 1, v);
        }
      }
      if (MODE == Q_ESTIMATE) __syncthreads();
    }
    __syncthreads();
    int nres;
    if (MODE == Q_ESTIMATE) {
      // ---- 3. top-c candidates ----
      auto getc = [&](long i) -> uint64_t {
        const uint64_t w = *reinterpret_cast<volatile uint64_t*>(&table[i]);
        const int id = slot_id(w);
        return id < 0 ? 0ull : pack_key(slot_val(w), id);
      };
      const uint64_t T = block_radix_threshold<uint64_t>(getc, (long)cap, a.c, hist, scratch);
      if (threadIdx.x == 0) scratch[5] = 0;
      __syncthreads();
      for (int i = threadIdx.x; i < cap; i += blockDim.x) {
        const uint64_t k = getc(i);
        if (k != 0 && k >= T) {
          const uint32_t pos = atomicAdd(&scratch[5], 1u);
          if (pos < (uint32_t)a.c) cand[pos] = key_id(k);
        }
      }
      __syncthreads();
      const int nc = (int)min(scratch[5], (uint32_t)(a.c > 0 ? a.c : 0));
      __syncthreads();
      // ---- 4. rerank ----
      uint64_t* rk = region;
      for (int i = threadIdx.x; i < nc; i += blockDim.x) {
        const int id = cand[i];
        rk[i] = pack_key(dot_seq(qv, row_ptr(a, id), a.ldx), id);
      }
      __syncthreads();
      nres = block_topk_sorted([&](long i) { return rk[i]; }, (long)nc, a.k, topk, k_cap, hist,
                               scratch);
    } else {
      // ---- union rerank in place over the table slots ----
      for (int i = threadIdx.x; i < cap; i += blockDim.x) {
        const uint64_t w = *reinterpret_cast<volatile uint64_t*>(&table[i]);
        const int id = slot_id(w);
        table[i] = id < 0 ? 0ull : pack_key(dot_seq(qv, row_ptr(a, id), a.ldx), id);
      }
      __syncthreads();
      nres = block_topk_sorted(
          [&](long i) { return *reinterpret_cast<volatile uint64_t*>(&table[i]); }, (long)cap, a.k,
          topk, k_cap, hist, scratch);
    }
    for (int i = threadIdx.x; i < a.k; i += blockDim.x) {
      a.out_ids[(long)q * a.k + i] = i < nres ? key_id(topk[i]) : 0;
      a.out_d[(long)q * a.k + i] = i < nres ? key_val(topk[i]) : 0.0f;
    }
    __syncthreads();
  }
}

cudaError_t launch_query_buckets(const QueryArgs& a, int mode, int grid, size_t smem,
                                 cudaStream_t st) {
  if (a.nq <= 0) return cudaSuccess;
  cudaError_t e;
  if (mode == Q_ESTIMATE) {
    e = cudaFuncSetAttribute(k_query_buckets<Q_ESTIMATE>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_query_buckets<Q_ESTIMATE><<<grid, kQueryThreads, smem, st>>>(a);
  } else {
    e = cudaFuncSetAttribute(k_query_buckets<Q_UNION>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    k_query_buckets<Q_UNION><<<grid, kQueryThreads, smem, st>>>(a);
  }
  return cudaGetLastError();
}

int query_buckets_blocks_per_sm(int mode, size_t smem) {
  int n = 0;
  cudaError_t e;
  if (mode == Q_ESTIMATE) {
    e = cudaFuncSetAttribute(k_query_buckets<Q_ESTIMATE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_query_buckets<Q_ESTIMATE>, kQueryThreads, smem);
  } else {
    e = cudaFuncSetAttribute(k_query_buckets<Q_UNION>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_query_buckets<Q_UNION>, kQueryThreads, smem);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n;
}

// ---------------------------------------------------------------------------
// Dense CEOs-Est.

__global__ void __launch_bounds__(256) k_probe_select(QueryArgs a) {
  extern __shared__ __align__(16) uint64_t pk[];
  __shared__ uint32_t hist[256];
  __shared__ uint32_t scratch[8];
  const int q = blockIdx.x;
  const float* qp = a.qproj + (long)q * a.C;
  const int s_cap = np2(a.s > 0 ? a.s : 1);
  const int ns = block_topk_sorted([&](long i) { return pack_key(abs_ref(qp[i]), (int)i); },
                                   (long)a.C, a.s, pk, s_cap, hist, scratch);
  for (int j = threadIdx.x; j < a.s; j += blockDim.x) {
    int tag = 0;
    if (j < ns) {
      const int col = key_id(pk[ns - 1 - j]);
      tag = qp[col] < 0 ? -(col + 1) : (col + 1);
    }
    a.probes_out[(long)q * a.s + j] = tag;
  }
}

cudaError_t launch_probe_select(const QueryArgs& a, cudaStream_t st) {
  if (a.nq <= 0 || a.s <= 0) return cudaSuccess;
  const size_t smem = (size_t)np2(a.s) * 8;
  k_probe_select<<<a.nq, 256, smem, st>>>(a);
  return cudaGetLastError();
}

// est[q][i] = 0 (+/-) P[col_1][i] (+/-) ... in probe pop order
// (src/CEOs.cpp:208-219: vecEst starts at zero, += close, -= far).
__global__ void __launch_bounds__(256) k_dense_estimate(QueryArgs a, int q0) {
  extern __shared__ int tags[];
  const int qi = blockIdx.y;
  const int q = q0 + qi;
  for (int j = threadIdx.x; j < a.s; j += blockDim.x) tags[j] = a.probes[(long)q * a.s + j];
  __syncthreads();
  const long n = a.n_points;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    float e = 0.0f;
    for (int j = 0; j < a.s; ++j) {
      const int tag = tags[j];
      if (tag == 0) continue;
      const int col = (tag < 0 ? -tag : tag) - 1;
      const float v = __ldg(a.P + (long)col * n + i);
      e = tag < 0 ? e - v : e + v;
    }
    a.est[(long)qi * n + i] = e;
  }
}

cudaError_t launch_dense_estimate(const QueryArgs& a, int q0, int nq_chunk, cudaStream_t st) {
  if (nq_chunk <= 0) return cudaSuccess;
  long bx = (a.n_points + 255) / 256;
  if (bx > 1024) bx = 1024;
  dim3 grid((unsigned)bx, (unsigned)nq_chunk);
  k_dense_estimate<<<grid, 256, (size_t)(a.s > 0 ? a.s : 1) * 4, st>>>(a, q0);
  return cudaGetLastError();
}

// Top-c over all n estimates of one query, then the exact rerank and top-k.
__global__ void __launch_bounds__(kQueryThreads) k_dense_select_rerank(QueryArgs a, int q0) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ uint32_t hist[256];
  __shared__ uint32_t scratch[8];
  const int qi = blockIdx.x;
  const int q = q0 + qi;
  const int k_cap = np2(a.k > 0 ? a.k : 1);
  const int c_cap = np2(a.c > 0 ? a.c : 1);
  float* qv = reinterpret_cast<float*>(sm);
  uint64_t* topk = reinterpret_cast<uint64_t*>(sm + al16((size_t)a.ldx * 4));
  uint64_t* rk = topk + k_cap;
  int* cand = reinterpret_cast<int*>(rk + c_cap);
  for (int j = threadIdx.x; j < a.ldx; j += blockDim.x) qv[j] = a.Q[(long)q * a.ldx + j];
  const float* est = a.est + (long)qi * a.n_points;
  auto gete = [&](long i) { return pack_key(est[i], (int)i); };
  const uint64_t T = block_radix_threshold<uint64_t>(gete, a.n_points, a.c, hist, scratch);
  if (threadIdx.x == 0) scratch[5] = 0;
  __syncthreads();
  for (long i = threadIdx.x; i < a.n_points; i += blockDim.x) {
    const uint64_t k = gete(i);
    if (k >= T) {
      const uint32_t pos = atomicAdd(&scratch[5], 1u);
      if (pos < (uint32_t)a.c) cand[pos] = (int)i;
    }
  }
  __syncthreads();
  const int nc = (int)min(scratch[5], (uint32_t)(a.c > 0 ? a.c : 0));
  __syncthreads();
  for (int i = threadIdx.x; i < nc; i += blockDim.x) {
    const int id = cand[i];
    rk[i] = pack_key(dot_seq(qv, row_ptr(a, id), a.ldx), id);
  }
  __syncthreads();
  const int nres =
      block_topk_sorted([&](long i) { return rk[i]; }, (long)nc, a.k, topk, k_cap, hist, scratch);
  for (int i = threadIdx.x; i < a.k; i += blockDim.x) {
    a.out_ids[(long)q * a.k + i] = i < nres ? key_id(topk[i]) : 0;
    a.out_d[(long)q * a.k + i] = i < nres ? key_val(topk[i]) : 0.0f;
  }
}

cudaError_t launch_dense_select_rerank(const QueryArgs& a, int q0, int nq_chunk, cudaStream_t st) {
  if (nq_chunk <= 0) return cudaSuccess;
  const int k_cap = np2(a.k > 0 ? a.k : 1);
  const int c_cap = np2(a.c > 0 ? a.c : 1);
  const size_t smem = al16((size_t)a.ldx * 4) + (size_t)k_cap * 8 + (size_t)c_cap * 8 +
                      (size_t)(a.c > 0 ? a.c : 1) * 4;
  cudaError_t e = cudaFuncSetAttribute(k_dense_select_rerank,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_dense_select_rerank<<<nq_chunk, kQueryThreads, smem, st>>>(a, q0);
  return cudaGetLastError();
}

}  // namespace ceos
