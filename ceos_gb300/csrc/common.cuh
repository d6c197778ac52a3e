// Shared device helpers for the CEOs GPU library (sm_103a).
//
// Ordering convention used by every selection in this library (buckets,
// probes, candidates, final top-k): items are ranked by value through the
// order-preserving uint32 image of the float (`fkey`, so -0 ranks below +0),
// and ties on value go to the smaller id. Packing (fkey(value), ~id) into one
// 64-bit word makes every key unique, so "top-K" is always exactly defined and
// a radix select on the packed key never stalls on ties.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define CEOS_DEV __device__ __forceinline__

namespace ceos {

constexpr int kWarp = 32;

CEOS_DEV uint32_t fkey(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

CEOS_DEV float fkey_inv(uint32_t k) {
  uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  return __uint_as_float(u);
}

// Packed rank key: larger key = better item.
CEOS_DEV uint64_t pack_key(float v, int id) {
  return ((uint64_t)fkey(v) << 32) | (uint64_t)(0xffffffffu - (uint32_t)id);
}
CEOS_DEV uint64_t pack_key_u(uint32_t vkey, int id) {
  return ((uint64_t)vkey << 32) | (uint64_t)(0xffffffffu - (uint32_t)id);
}
CEOS_DEV int key_id(uint64_t k) { return (int)(0xffffffffu - (uint32_t)(k & 0xffffffffu)); }
CEOS_DEV float key_val(uint64_t k) { return fkey_inv((uint32_t)(k >> 32)); }

// ---------------------------------------------------------------------------
// Block-level radix select.
//
// Finds the largest threshold T such that at least min(K, N') of the N'
// nonzero keys produced by `get(i)` are >= T, i.e. T is the K-th largest key.
// With unique keys (the packed 64-bit form) exactly min(K, N') keys are >= T. Keys are visited through a functor so
// the same routine serves keys in shared memory, keys computed on the fly from
// global memory, and hash-table slots (a functor may return 0 for "no item";
// 0 is never a valid key because ids are < 2^31).
//
// `hist` must point to 256 uint32 of shared memory; `scratch` to 4 uint32 of
// shared memory. All threads of the block must call it.
template <typename KeyT, typename GetKey>
__device__ KeyT block_radix_threshold(GetKey get, long N, int K, uint32_t* hist,
                                      uint32_t* scratch) {
  if (K <= 0) return ~(KeyT)0;  // nothing selected
  KeyT prefix = 0, mask = 0;
  uint32_t remaining = (uint32_t)K;
  for (int shift = (int)sizeof(KeyT) * 8 - 8; shift >= 0; shift -= 8) {
    for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    for (long i = threadIdx.x; i < N; i += blockDim.x) {
      const KeyT k = get(i);
      if (k != 0 && (k & mask) == prefix) atomicAdd(&hist[(uint32_t)(k >> shift) & 255u], 1u);
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      // Suffix scan over 256 bins by one warp: lane l owns bins [8l, 8l+8).
      const int lane = threadIdx.x;
      uint32_t loc[8];
      uint32_t s = 0;
#pragma unroll
      for (int j = 7; j >= 0; --j) {
        loc[j] = hist[lane * 8 + j];
        s += loc[j];
      }
      // inclusive suffix sum of per-lane totals (lanes above me)
      uint32_t above = 0;
      uint32_t t = s;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_down_sync(0xffffffffu, t, o);
        if (lane + o < 32) t += v;
      }
      above = t - s;  // count in bins of higher lanes
      // find the bin b where cumulative count from the top reaches `remaining`
      uint32_t acc = above;
      int found = -1;
      uint32_t before = 0, inbin = 0;
#pragma unroll
      for (int j = 7; j >= 0; --j) {
        if (found < 0 && acc + loc[j] >= remaining && acc < remaining) {
          found = lane * 8 + j;
          before = acc;
          inbin = loc[j];
        }
        acc += loc[j];
      }
      if (found >= 0) {
        scratch[0] = (uint32_t)found;
        scratch[1] = before;
        scratch[2] = inbin;
      }
      // total < remaining (N < K): handled below via scratch[3]
      const uint32_t total = __shfl_sync(0xffffffffu, t, 0);
      if (lane == 0) scratch[3] = total;
    }
    __syncthreads();
    const uint32_t total = scratch[3];
    if (total < remaining) {
      // Fewer candidates than requested under this prefix: take them all.
      __syncthreads();
      return prefix;
    }
    const uint32_t b = scratch[0], before = scratch[1], inbin = scratch[2];
    __syncthreads();
    prefix |= (KeyT)b << shift;
    mask |= (KeyT)255 << shift;
    remaining -= before;
    if (inbin == remaining) break;
  }
  return prefix;
}

// In-place bitonic sort (descending) of n = power-of-two 64-bit keys in
// shared memory. All threads of the block must call it.
__device__ inline void block_bitonic_sort_desc(uint64_t* a, int n) {
  for (int k = 2; k <= n; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        int ixj = i ^ j;
        if (ixj > i) {
          uint64_t x = a[i], y = a[ixj];
          bool desc = ((i & k) == 0);
          if (desc ? (x < y) : (x > y)) {
            a[i] = y;
            a[ixj] = x;
          }
        }
      }
      __syncthreads();
    }
  }
}

// Select the top-K (K <= cap) of N keys into `out` (shared memory, `cap` =
// power of two >= K) sorted descending; unused tail slots are 0. Returns the
// number of selected keys (min(N', K), N' = number of nonzero keys).
// hist: 256 u32 smem, scratch: 8 u32 smem.
template <typename GetKey>
__device__ int block_topk_sorted(GetKey get, long N, int K, uint64_t* out, int cap,
                                 uint32_t* hist, uint32_t* scratch) {
  const uint64_t T = block_radix_threshold<uint64_t>(get, N, K, hist, scratch);
  for (int i = threadIdx.x; i < cap; i += blockDim.x) out[i] = 0;
  if (threadIdx.x == 0) scratch[4] = 0;
  __syncthreads();
  for (long i = threadIdx.x; i < N; i += blockDim.x) {
    const uint64_t k = get(i);
    if (k != 0 && k >= T) {
      uint32_t pos = atomicAdd(&scratch[4], 1u);
      if (pos < (uint32_t)cap) out[pos] = k;
    }
  }
  __syncthreads();
  int cnt = (int)min(scratch[4], (uint32_t)K);
  __syncthreads();
  block_bitonic_sort_desc(out, cap);
  return cnt;
}

CEOS_DEV int next_pow2(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

}  // namespace ceos
