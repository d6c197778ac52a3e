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

// Completeness threshold of an exactly maintained bucket list (x = fkey of the
// value, y = id as a signed int): every live point outside the list ranks below
// it, so list entries that rank at or above it are the exact top of the live
// set. kTauNone certifies everything (the list holds every live point).
constexpr uint32_t kTauNoneId = 0x7fffffffu;
CEOS_DEV uint2 tau_none() { return make_uint2(0u, kTauNoneId); }
CEOS_DEV bool tau_is_none(uint2 t) { return t.x == 0u && t.y == kTauNoneId; }
CEOS_DEV uint2 tau_of(float v, int id) { return make_uint2(fkey(v), (uint32_t)id); }
// (v, id) ranks at or above the threshold
CEOS_DEV bool tau_certifies(uint2 t, float v, int id) {
  const uint32_t k = fkey(v);
  return k > t.x || (k == t.x && id <= (int)t.y);
}
CEOS_DEV float key_val(uint64_t k) { return fkey_inv((uint32_t)(k >> 32)); }

// Smallest float b with fkey(v) >= k  =>  v >= b for every non-NaN v: the
// float of the key itself, -inf for keys at or below fkey(-inf) and +inf for
// keys above fkey(+inf). The only non-NaN v with v >= b but fkey(v) < k is
// v = -0 when b = +0, so a float test against b is a superset test.
CEOS_DEV float key_lower_bound(uint32_t k) {
  if (k <= 0x007fffffu) return __uint_as_float(0xff800000u);  // -inf
  if (k > 0xff800000u) return __uint_as_float(0x7f800000u);   // +inf
  return fkey_inv(k);
}
// Float prefilter of a (close, far) threshold pair: fkey(v) >= t.x implies
// v >= bounds.x, and fkey(-v) >= t.y implies v <= bounds.y.
CEOS_DEV float2 emit_bounds(uint2 t) {
  return make_float2(key_lower_bound(t.x), -key_lower_bound(t.y));
}

// One digit step of a radix select, run by warp 0 of the block on a complete
// 256-bin histogram: finds the bin b where the count of keys taken from the
// top reaches `remaining` and writes scratch[0] = b, scratch[1] = keys in bins
// above b, scratch[2] = keys in b, scratch[3] = all keys in the histogram.
__device__ inline void radix_scan_hist(const uint32_t* hist, uint32_t remaining,
                                       uint32_t* scratch) {
  // lane l owns bins [8l, 8l+8)
  const int lane = threadIdx.x & 31;
  uint32_t loc[8];
  uint32_t s = 0;
#pragma unroll
  for (int j = 7; j >= 0; --j) {
    loc[j] = hist[lane * 8 + j];
    s += loc[j];
  }
  // inclusive suffix sum of per-lane totals (lanes above me)
  uint32_t t = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t v = __shfl_down_sync(0xffffffffu, t, o);
    if (lane + o < 32) t += v;
  }
  uint32_t acc = t - s;  // count in bins of higher lanes
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
  // total < remaining (fewer keys than requested): the caller takes them all
  const uint32_t total = __shfl_sync(0xffffffffu, t, 0);
  if (lane == 0) scratch[3] = total;
}

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
    if (threadIdx.x < 32) radix_scan_hist(hist, remaining, scratch);
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


// ---------------------------------------------------------------------------
// Block-level top-K by value histogram.
//
// Exact top-K (under the packed (value, id) order) of N items delivered by
// `get(i, v, id) -> bool`. Three passes over the items instead of up to eight
// radix passes:
//   1. min / max / count of the values;
//   2. a 2048-bin histogram on a LINEAR scale over [min, max], which spreads
//      clustered values over many counters (a radix digit of the float key
//      puts most of them on one shared-memory counter);
//   3. compaction: items in bins above the threshold bin go straight to `out`,
//      items of the threshold bin to `maybe`, which is then sorted by packed
//      key to take the missing ones.
// The bin index is a weakly increasing function of the value, so every item
// of a higher bin ranks above every item of a lower bin, and ties in value
// land in the same bin where the packed key orders them. Degenerate value
// ranges, non-finite values and an oversized threshold bin fall back to the
// radix select. `out` (at least K slots) receives min(K, valid) keys,
// unsorted; with unique keys they are exactly the top-K.
//
// Shared memory: hist = kHistBins u32, maybe = maybe_cap u64 (power of two),
// scratch = 16 u32. All threads of the block must call it; blockDim.x must be
// a multiple of 32.
constexpr int kHistBins = 2048;
// items loaded per thread before they are used, in the histogram and
// compaction passes (the items usually come from L2 or HBM)
constexpr int kTopkU = 2;

CEOS_DEV uint32_t warp_reserve(bool want, uint32_t* counter) {
  const unsigned m = __ballot_sync(0xffffffffu, want);
  uint32_t base = 0;
  const int lane = threadIdx.x & 31;
  if (m) {
    const int leader = __ffs(m) - 1;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
  }
  return base + __popc(m & ((1u << lane) - 1u));
}

// pre (optional): min key, max key and count of the valid items, already
// known to the caller; pass 1 is then skipped.
//
// kBinOrder: on the histogram path, items above the threshold bin are
// scattered to the output segment of their bin (bins in descending order,
// offsets from the suffix scan of the histogram) instead of being appended,
// and each bin's few items are then insertion-sorted, so that `out` comes out
// sorted descending without a block-wide sort. scratch[12] = 1 reports a
// sorted result; it is 0 when a path without bin order was taken or a bin
// holds more than kBinSortMax items (the caller sorts then).
// kLoadsU: items each thread loads before it uses them in the passes (more
// when the items come from HBM, at the cost of registers).
constexpr int kBinSortMax = 24;
template <bool kBinOrder = false, int kLoadsU = kTopkU, typename GetItem>
__device__ int block_topk_hist(GetItem get, long N, int K, uint64_t* out, uint32_t* hist,
                               uint64_t* maybe, int maybe_cap, uint32_t* scratch,
                               const uint32_t* pre = nullptr, const int2* pf_items = nullptr) {
  // pf_items: the items as 8-byte records in global memory, when get() reads
  // them there; each round of loads then prefetches the next round into L2,
  // one 128-byte line (16 items) per thread
  auto pf_round = [&](long next) {
    if (pf_items == nullptr) return;
    const long i = next + 16L * threadIdx.x;
    if (16 * threadIdx.x < kLoadsU * blockDim.x && i < N)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(pf_items + i));
  };
  const int lane = threadIdx.x & 31;
  if (kBinOrder && threadIdx.x == 0) {
    scratch[12] = 0u;
    scratch[13] = 0u;
  }
  // ---- pass 1: min / max keys and count ----
  if (threadIdx.x == 0) {
    scratch[0] = pre ? pre[0] : 0xffffffffu;  // min key
    scratch[1] = pre ? pre[1] : 0u;           // max key
    scratch[2] = pre ? pre[2] : 0u;           // valid count
    scratch[3] = 0u;                          // out count
    scratch[4] = 0u;                          // maybe count
  }
  __syncthreads();
  if (!pre) {
    uint32_t lo = 0xffffffffu, hi = 0u, cnt = 0u;
    for (long base = 0; base < N; base += kLoadsU * blockDim.x) {
      float v[kLoadsU];
      int id[kLoadsU];
      bool ok[kLoadsU];
#pragma unroll
      for (int u = 0; u < kLoadsU; ++u) {
        const long i = base + u * blockDim.x + threadIdx.x;
        v[u] = 0.f;
        id[u] = 0;
        ok[u] = i < N && get(i, v[u], id[u]);
      }
#pragma unroll
      for (int u = 0; u < kLoadsU; ++u) {
        if (ok[u]) {
          const uint32_t k = fkey(v[u]);
          lo = min(lo, k);
          hi = max(hi, k);
          ++cnt;
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
      cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if (lane == 0) {
      atomicMin(&scratch[0], lo);
      atomicMax(&scratch[1], hi);
      atomicAdd(&scratch[2], cnt);
    }
  }
  __syncthreads();
  const uint32_t nvalid = scratch[2];
  const float vmin = fkey_inv(scratch[0]), vmax = fkey_inv(scratch[1]);
  if (K <= 0 || nvalid == 0) return 0;
  if (nvalid <= (uint32_t)K) {
    for (long base = 0; base < N; base += blockDim.x) {
      const long i = base + threadIdx.x;
      float v = 0.f;
      int id = 0;
      const bool ok = i < N && get(i, v, id);
      const uint32_t pos = warp_reserve(ok, &scratch[3]);
      if (ok) out[pos] = pack_key(v, id);
    }
    __syncthreads();
    return (int)nvalid;
  }
  const float range = vmax - vmin;
  const bool linear = (range > 0.0f) && isfinite(range) && isfinite(vmin) && isfinite(vmax);
  if (!linear) {
    const uint64_t T = block_radix_threshold<uint64_t>(
        [&](long i) -> uint64_t {
          float v;
          int id;
          return get(i, v, id) ? pack_key(v, id) : 0ull;
        },
        N, K, hist, scratch + 8);
    for (long base = 0; base < N; base += blockDim.x) {
      const long i = base + threadIdx.x;
      float v = 0.f;
      int id = 0;
      const bool ok = i < N && get(i, v, id) && pack_key(v, id) >= T;
      const uint32_t pos = warp_reserve(ok, &scratch[3]);
      if (ok && pos < (uint32_t)K) out[pos] = pack_key(v, id);
    }
    __syncthreads();
    return K;
  }
  const float scale = (float)kHistBins / range;
  auto bin_of = [&](float v) -> int {
    const int b = (int)((v - vmin) * scale);
    return b < 0 ? 0 : (b >= kHistBins ? kHistBins - 1 : b);
  };
  // ---- pass 2: histogram ----
  for (int b = threadIdx.x; b < kHistBins; b += blockDim.x) hist[b] = 0;
  __syncthreads();
  for (long base = 0; base < N; base += kLoadsU * blockDim.x) {
    pf_round(base + kLoadsU * blockDim.x);
    float v[kLoadsU];
    int id[kLoadsU];
    bool ok[kLoadsU];
#pragma unroll
    for (int u = 0; u < kLoadsU; ++u) {
      const long i = base + u * blockDim.x + threadIdx.x;
      v[u] = 0.f;
      id[u] = 0;
      ok[u] = i < N && get(i, v[u], id[u]);
    }
#pragma unroll
    for (int u = 0; u < kLoadsU; ++u)
      if (ok[u]) atomicAdd(&hist[bin_of(v[u])], 1u);
  }
  __syncthreads();
  // ---- threshold bin: block-wide suffix scan over the bins ----
  {
    // thread t owns bins [t*per, (t+1)*per); warps combine their totals
    const int per = (kHistBins + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per;
    uint32_t mine = 0;
    for (int j = 0; j < per; ++j)
      if (b0 + j < kHistBins) mine += hist[b0 + j];
    uint32_t t = mine;  // inclusive suffix sum within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_down_sync(0xffffffffu, t, o);
      if (lane + o < 32) t += v;
    }
    __shared__ uint32_t warp_tot[32];
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    if (lane == 0) warp_tot[warp] = t;
    __syncthreads();
    uint32_t above_warps = 0;
    for (int w = warp + 1; w < nwarps; ++w) above_warps += warp_tot[w];
    uint32_t acc = above_warps + (t - mine);  // items in bins above mine
    for (int j = per - 1; j >= 0; --j) {
      if (b0 + j >= kHistBins) continue;
      const uint32_t h = hist[b0 + j];
      if (acc < (uint32_t)K && acc + h >= (uint32_t)K) {
        scratch[5] = (uint32_t)(b0 + j);
        scratch[6] = acc;  // items above the threshold bin
        scratch[7] = h;    // items in it
      }
      // bin order: the bin's output offset (items in higher bins) becomes its
      // scatter cursor (each thread rewrites only its own bins)
      if constexpr (kBinOrder) hist[b0 + j] = acc;
      acc += h;
    }
  }
  __syncthreads();
  const int tb = (int)scratch[5];
  const uint32_t above = scratch[6], inbin = scratch[7];
  const uint32_t need = (uint32_t)K - above;
  const bool fits = inbin <= (uint32_t)maybe_cap;
  // ---- pass 3: compaction ----
  for (long base = 0; base < N; base += kLoadsU * blockDim.x) {
    pf_round(base + kLoadsU * blockDim.x);
    float v[kLoadsU];
    int id[kLoadsU];
    bool ok[kLoadsU];
#pragma unroll
    for (int u = 0; u < kLoadsU; ++u) {
      const long i = base + u * blockDim.x + threadIdx.x;
      v[u] = 0.f;
      id[u] = 0;
      ok[u] = i < N && get(i, v[u], id[u]);
    }
#pragma unroll
    for (int u = 0; u < kLoadsU; ++u) {
      const int b = ok[u] ? bin_of(v[u]) : -1;
      const bool sure = ok[u] && b > tb;
      const bool cand = ok[u] && b == tb && fits;
      if constexpr (kBinOrder) {
        if (sure) out[atomicAdd(&hist[b], 1u)] = pack_key(v[u], id[u]);
      } else {
        const uint32_t p1 = warp_reserve(sure, &scratch[3]);
        if (sure) out[p1] = pack_key(v[u], id[u]);
      }
      const uint32_t p2 = warp_reserve(cand, &scratch[4]);
      if (cand) maybe[p2] = pack_key(v[u], id[u]);
    }
  }
  // bin order scattered the items above the threshold bin to out[0, above)
  // without the append counter; later appends go after them
  if (kBinOrder && threadIdx.x == 0) scratch[3] = above;
  __syncthreads();
  if (fits) {
    int np = 1;
    while (np < (int)inbin) np <<= 1;
    for (int i = (int)inbin + threadIdx.x; i < np; i += blockDim.x) maybe[i] = 0ull;
    __syncthreads();
    block_bitonic_sort_desc(maybe, np);
    for (uint32_t i = threadIdx.x; i < need; i += blockDim.x) out[above + i] = maybe[i];
    if constexpr (kBinOrder) {
      // bin b > tb now holds out[end(b + 1), end(b)), end = its final cursor
      for (int b = tb + 1 + threadIdx.x; b < kHistBins; b += blockDim.x) {
        const uint32_t lo = (b + 1 < kHistBins) ? hist[b + 1] : 0u, hi = hist[b];
        if (hi - lo > (uint32_t)kBinSortMax) {
          scratch[13] = 1u;
          continue;
        }
        for (uint32_t i = lo + 1; i < hi; ++i) {
          const uint64_t x = out[i];
          uint32_t j = i;
          while (j > lo && out[j - 1] < x) {
            out[j] = out[j - 1];
            --j;
          }
          out[j] = x;
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) scratch[12] = scratch[13] ? 0u : 1u;
    }
    __syncthreads();
  } else {
    // threshold bin too large for the buffer: radix select inside it
    auto getb = [&](long i) -> uint64_t {
      float v;
      int id;
      return (get(i, v, id) && bin_of(v) == tb) ? pack_key(v, id) : 0ull;
    };
    const uint64_t T = block_radix_threshold<uint64_t>(getb, N, (int)need, hist, scratch + 8);
    for (long base = 0; base < N; base += blockDim.x) {
      const long i = base + threadIdx.x;
      const uint64_t k = i < N ? getb(i) : 0ull;
      const bool ok = k != 0 && k >= T;
      const uint32_t pos = warp_reserve(ok, &scratch[3]);
      if (ok && pos < (uint32_t)K) out[pos] = k;
    }
    __syncthreads();
  }
  return K;
}

// block_topk_hist followed by a descending sort: out[0..ret) best first,
// out[ret..out_cap) zero. out_cap is a power of two >= K. kBinOrder (for large
// K, e.g. bucket lists) orders the result by histogram bins and sorts within
// bins, falling back to the block-wide bitonic sort; small K (probes, final
// top-k) is cheaper with the bitonic sort alone.
template <bool kBinOrder = false, typename GetItem>
__device__ int block_topk_hist_sorted(GetItem get, long N, int K, uint64_t* out, int out_cap,
                                      uint32_t* hist, uint64_t* maybe, int maybe_cap,
                                      uint32_t* scratch) {
  const int cnt = block_topk_hist<kBinOrder>(get, N, K, out, hist, maybe, maybe_cap, scratch);
  const bool sorted = kBinOrder && scratch[12] != 0u;
  for (int i = cnt + threadIdx.x; i < out_cap; i += blockDim.x) out[i] = 0ull;
  __syncthreads();
  if (!sorted) block_bitonic_sort_desc(out, out_cap);
  return cnt;
}

CEOS_DEV int next_pow2(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

}  // namespace ceos
