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
//     point id (keys and values in two arrays; in shared memory when it fits,
//     else in a per-CTA L2-resident workspace). Within one column the ids are
//     distinct, so each table value receives its terms in exactly the
//     reference's order; a barrier separates columns. A value starts as its
//     first term (the reference's "assign on first sight").
//  3. top-c candidates by estimate (block histogram select on packed keys).
//  4. exact rerank: groups of 8 lanes compute one inner product each (lane g
//     accumulates the float4 chunks g, g+8, ... with FMA, then a butterfly
//     over the 8 lanes), then the block selects the top-k, written best first
//     with zero fill past the number of results (src/CEOs.cpp:659-666).
#include <climits>

#include "kernels.h"
#include "common.cuh"

namespace ceos {

constexpr int kQueryThreads = 512;

CEOS_DEV float abs_ref(float v) { return v < 0 ? -v : v; }

CEOS_DEV const float* row_ptr(const QueryArgs& a, int id) {
  long r = a.head + id;
  if (r >= a.cap_rows) r -= a.cap_rows;
  return a.X + r * (long)a.ldx;
}

CEOS_DEV const uint16_t* row_ptr_bf16(const QueryArgs& a, int id) {
  long r = a.head + id;
  if (r >= a.cap_rows) r -= a.cap_rows;
  return a.Xb + r * (long)a.ldx;
}

// Inner product of a query with one row, in the library's canonical order:
// the row is split into float4 chunks; lane g (0..7) of an 8-lane group
// accumulates chunks g, g+8, g+16, ... as a sequential FMA chain
// (s = fma(q_j, x_j, s) over the chunk's 4 elements, chunk by chunk), then the
// 8 partial sums are combined by a butterfly (xor 4, then 2, then 1). Padding
// columns are zero on both sides and leave every partial sum unchanged. The
// oracle computes the same order, so scores are bit-exact between the two.
// An 8-lane group reads 128 contiguous bytes per load, so a warp moves four
// rows' chunks per instruction (coalesced, few outstanding requests per byte).
CEOS_DEV float dot_g8(const float* __restrict__ q, const float* __restrict__ x, int n4, int g,
                      bool active) {
  const float4* x4 = reinterpret_cast<const float4*>(x);
  const float4* q4 = reinterpret_cast<const float4*>(q);
  float s = 0.0f;
  if (active) {
    int c = g;
    for (; c + 24 < n4; c += 32) {
      float4 xv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) xv[u] = __ldcg(x4 + c + 8 * u);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float4 qv = q4[c + 8 * u];
        s = __fmaf_rn(qv.x, xv[u].x, s);
        s = __fmaf_rn(qv.y, xv[u].y, s);
        s = __fmaf_rn(qv.z, xv[u].z, s);
        s = __fmaf_rn(qv.w, xv[u].w, s);
      }
    }
    for (; c < n4; c += 8) {
      const float4 xv = __ldcg(x4 + c);
      const float4 qv = q4[c];
      s = __fmaf_rn(qv.x, xv.x, s);
      s = __fmaf_rn(qv.y, xv.y, s);
      s = __fmaf_rn(qv.z, xv.z, s);
      s = __fmaf_rn(qv.w, xv.w, s);
    }
  }
  s = s + __shfl_xor_sync(0xffffffffu, s, 4);
  s = s + __shfl_xor_sync(0xffffffffu, s, 2);
  s = s + __shfl_xor_sync(0xffffffffu, s, 1);
  return s;
}

// Prefetch into L2 the rows of candidates keys[i0 .. i0 + 8) (lane l: row
// i0 + l / 4, its 128-byte line l % 4), one step of a warp's rerank loop
// ahead. Long candidate lists of short rows only: at 8000 candidates of 512
// bytes per query it took 2.6% off the search, at 2000 it added 1.7%, and on
// 3840-byte rows (4000 candidates) it cost 9%.
constexpr int kRerankPrefetchMin = 3072;
template <typename RowPtr>
CEOS_DEV void prefetch_rows(const uint64_t* keys, int n, int i0, int row_bytes, RowPtr row) {
  const int lane = threadIdx.x & 31;
  const int i = i0 + (lane >> 2);
  if (i >= n || row_bytes > 512) return;
  const char* p = reinterpret_cast<const char*>(row(key_id(keys[i])));
  for (int off = 128 * (lane & 3); off < row_bytes; off += 512)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p + off));
}

// Approximate score for the split-precision scan: like dot_g8 but over
// 8-element chunks of the bfloat16 row (16 bytes per lane per load); chunk c
// goes to lane c mod 8, each lane a sequential FMA chain, then the butterfly.
CEOS_DEV float dot_g8_bf16(const float* __restrict__ q, const uint16_t* __restrict__ x, int n8,
                           int g, bool active) {
  const uint4* x8 = reinterpret_cast<const uint4*>(x);
  const float4* q4 = reinterpret_cast<const float4*>(q);
  float s = 0.0f;
  auto acc8 = [&](const uint4 w, int c) {
    const float4 qa = q4[2 * c], qb = q4[2 * c + 1];
    s = __fmaf_rn(qa.x, __uint_as_float(w.x << 16), s);
    s = __fmaf_rn(qa.y, __uint_as_float(w.x & 0xffff0000u), s);
    s = __fmaf_rn(qa.z, __uint_as_float(w.y << 16), s);
    s = __fmaf_rn(qa.w, __uint_as_float(w.y & 0xffff0000u), s);
    s = __fmaf_rn(qb.x, __uint_as_float(w.z << 16), s);
    s = __fmaf_rn(qb.y, __uint_as_float(w.z & 0xffff0000u), s);
    s = __fmaf_rn(qb.z, __uint_as_float(w.w << 16), s);
    s = __fmaf_rn(qb.w, __uint_as_float(w.w & 0xffff0000u), s);
  };
  if (active) {
    int c = g;
    // four loads in flight, then the FMAs in chunk order
    for (; c + 24 < n8; c += 32) {
      uint4 w[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) w[u] = __ldcg(x8 + c + 8 * u);
#pragma unroll
      for (int u = 0; u < 4; ++u) acc8(w[u], c + 8 * u);
    }
    for (; c < n8; c += 8) acc8(__ldcg(x8 + c), c);
  }
  s = s + __shfl_xor_sync(0xffffffffu, s, 4);
  s = s + __shfl_xor_sync(0xffffffffu, s, 2);
  s = s + __shfl_xor_sync(0xffffffffu, s, 1);
  return s;
}

// dot_g8_bf16 of one query with two rows at once (each row's sum in exactly
// dot_g8_bf16's order): an 8-lane group keeps twice as many loads in flight.
CEOS_DEV void dot_g8_bf16_2(const float* __restrict__ q, const uint16_t* __restrict__ xa,
                            const uint16_t* __restrict__ xb, int n8, int g, float& sa, float& sb) {
  const uint4* a8 = reinterpret_cast<const uint4*>(xa);
  const uint4* b8 = reinterpret_cast<const uint4*>(xb);
  const float4* q4 = reinterpret_cast<const float4*>(q);
  float s0 = 0.0f, s1 = 0.0f;
  auto acc8 = [&](float& s, const uint4 w, int c) {
    const float4 qa = q4[2 * c], qb = q4[2 * c + 1];
    s = __fmaf_rn(qa.x, __uint_as_float(w.x << 16), s);
    s = __fmaf_rn(qa.y, __uint_as_float(w.x & 0xffff0000u), s);
    s = __fmaf_rn(qa.z, __uint_as_float(w.y << 16), s);
    s = __fmaf_rn(qa.w, __uint_as_float(w.y & 0xffff0000u), s);
    s = __fmaf_rn(qb.x, __uint_as_float(w.z << 16), s);
    s = __fmaf_rn(qb.y, __uint_as_float(w.z & 0xffff0000u), s);
    s = __fmaf_rn(qb.z, __uint_as_float(w.w << 16), s);
    s = __fmaf_rn(qb.w, __uint_as_float(w.w & 0xffff0000u), s);
  };
  int c = g;
  for (; c + 24 < n8; c += 32) {
    uint4 wa[4], wb[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      wa[u] = __ldcg(a8 + c + 8 * u);
      wb[u] = __ldcg(b8 + c + 8 * u);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      acc8(s0, wa[u], c + 8 * u);
      acc8(s1, wb[u], c + 8 * u);
    }
  }
  for (; c < n8; c += 8) {
    const uint4 wa = __ldcg(a8 + c), wb = __ldcg(b8 + c);
    acc8(s0, wa, c);
    acc8(s1, wb, c);
  }
  s0 = s0 + __shfl_xor_sync(0xffffffffu, s0, 4);
  s1 = s1 + __shfl_xor_sync(0xffffffffu, s1, 4);
  s0 = s0 + __shfl_xor_sync(0xffffffffu, s0, 2);
  s1 = s1 + __shfl_xor_sync(0xffffffffu, s1, 2);
  s0 = s0 + __shfl_xor_sync(0xffffffffu, s0, 1);
  s1 = s1 + __shfl_xor_sync(0xffffffffu, s1, 1);
  sa = s0;
  sb = s1;
}

// Split-precision rerank of keys[0..n) in place (approximate bfloat16
// scores): eight rows per warp at a time, two per 8-lane group; a slot past n
// re-reads the last candidate's row (the result is dropped).
template <typename RowPtr>
CEOS_DEV void rerank_bf16_inplace(uint64_t* keys, int n, const float* qv, int ldx, RowPtr row) {
  const int lane = threadIdx.x & 31;
  const int g = lane & 7;
  const int grp = lane >> 3;
  const int warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const int n8 = ldx >> 3;
  const bool pf = n >= kRerankPrefetchMin;
  for (int base = warp * 8; base < n; base += nw * 8) {
    if (pf) prefetch_rows(keys, n, base + nw * 8, ldx * 2, row);
    const int i0 = base + grp, i1 = base + 4 + grp;
    const bool a0 = i0 < n, a1 = i1 < n;
    const int id0 = key_id(keys[a0 ? i0 : n - 1]);
    const int id1 = key_id(keys[a1 ? i1 : n - 1]);
    float d0, d1;
    dot_g8_bf16_2(qv, row(id0), row(id1), n8, g, d0, d1);
    if (g == 0) {
      if (a0) keys[i0] = pack_key(d0, id0);
      if (a1) keys[i1] = pack_key(d1, id1);
    }
  }
}

// dot_g8 of one query with two rows at once (each row's sum in exactly
// dot_g8's order): an 8-lane group keeps twice as many loads in flight.
CEOS_DEV void dot_g8_2(const float* __restrict__ q, const float* __restrict__ xa,
                       const float* __restrict__ xb, int n4, int g, float& sa, float& sb) {
  const float4* a4 = reinterpret_cast<const float4*>(xa);
  const float4* b4 = reinterpret_cast<const float4*>(xb);
  const float4* q4 = reinterpret_cast<const float4*>(q);
  float s0 = 0.0f, s1 = 0.0f;
  int c = g;
  for (; c + 24 < n4; c += 32) {
    float4 va[4], vb[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      va[u] = __ldcg(a4 + c + 8 * u);
      vb[u] = __ldcg(b4 + c + 8 * u);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float4 qv = q4[c + 8 * u];
      s0 = __fmaf_rn(qv.x, va[u].x, s0);
      s0 = __fmaf_rn(qv.y, va[u].y, s0);
      s0 = __fmaf_rn(qv.z, va[u].z, s0);
      s0 = __fmaf_rn(qv.w, va[u].w, s0);
      s1 = __fmaf_rn(qv.x, vb[u].x, s1);
      s1 = __fmaf_rn(qv.y, vb[u].y, s1);
      s1 = __fmaf_rn(qv.z, vb[u].z, s1);
      s1 = __fmaf_rn(qv.w, vb[u].w, s1);
    }
  }
  for (; c < n4; c += 8) {
    const float4 va = __ldcg(a4 + c), vb = __ldcg(b4 + c);
    const float4 qv = q4[c];
    s0 = __fmaf_rn(qv.x, va.x, s0);
    s0 = __fmaf_rn(qv.y, va.y, s0);
    s0 = __fmaf_rn(qv.z, va.z, s0);
    s0 = __fmaf_rn(qv.w, va.w, s0);
    s1 = __fmaf_rn(qv.x, vb.x, s1);
    s1 = __fmaf_rn(qv.y, vb.y, s1);
    s1 = __fmaf_rn(qv.z, vb.z, s1);
    s1 = __fmaf_rn(qv.w, vb.w, s1);
  }
  s0 = s0 + __shfl_xor_sync(0xffffffffu, s0, 4);
  s1 = s1 + __shfl_xor_sync(0xffffffffu, s1, 4);
  s0 = s0 + __shfl_xor_sync(0xffffffffu, s0, 2);
  s1 = s1 + __shfl_xor_sync(0xffffffffu, s1, 2);
  s0 = s0 + __shfl_xor_sync(0xffffffffu, s0, 1);
  s1 = s1 + __shfl_xor_sync(0xffffffffu, s1, 1);
  sa = s0;
  sb = s1;
}

// Rerank keys[0..n) in place: each holds a candidate id (packed key); it is
// replaced by pack_key(<q, x_id>, id). Each warp scores eight rows at a time,
// two per 8-lane group. A slot past n re-reads the last candidate's row (its
// loads must stay global-memory loads of a real row; the result is dropped).
template <typename RowPtr>
CEOS_DEV void rerank_inplace(uint64_t* keys, int n, const float* qv, int ldx, RowPtr row) {
  const int lane = threadIdx.x & 31;
  const int g = lane & 7;
  const int grp = lane >> 3;
  const int warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const int n4 = ldx >> 2;
  const bool pf = n >= kRerankPrefetchMin;
  for (int base = warp * 8; base < n; base += nw * 8) {
    if (pf) prefetch_rows(keys, n, base + nw * 8, ldx * 4, row);
    const int i0 = base + grp, i1 = base + 4 + grp;
    const bool a0 = i0 < n, a1 = i1 < n;
    const int id0 = key_id(keys[a0 ? i0 : n - 1]);
    const int id1 = key_id(keys[a1 ? i1 : n - 1]);
    float d0, d1;
    dot_g8_2(qv, row(id0), row(id1), n4, g, d0, d1);
    if (g == 0) {
      if (a0) keys[i0] = pack_key(d0, id0);
      if (a1) keys[i1] = pack_key(d1, id1);
    }
  }
}

// Final scoring of a candidate list (keys hold candidate ids): exact FP32
// rerank, or (split precision) the bfloat16 scan followed by an exact rescore
// of the scan's best `a.rescore`, staged in `resc`. Returns the number of
// leading keys that hold exact scores: n, or min(n, a.rescore) after the
// rescored keys are copied to the front.
CEOS_DEV int score_candidates(const QueryArgs& a, int rq, uint64_t* keys, int n, const float* qv,
                              uint64_t* resc, uint32_t* hist, uint64_t* maybe, int maybe_cap,
                              uint32_t* scratch) {
  if (a.Xb == nullptr || rq <= 0) {
    rerank_inplace(keys, n, qv, a.ldx, [&](int id) { return row_ptr(a, id); });
    __syncthreads();
    return n;
  }
  rerank_bf16_inplace(keys, n, qv, a.ldx, [&](int id) { return row_ptr_bf16(a, id); });
  __syncthreads();
  const int nr = block_topk_hist(
      [&](long i, float& v, int& id) {
        const uint64_t k = keys[i];
        v = key_val(k);
        id = key_id(k);
        return true;
      },
      (long)n, rq, resc, hist, maybe, maybe_cap, scratch);
  rerank_inplace(resc, nr, qv, a.ldx, [&](int id) { return row_ptr(a, id); });
  __syncthreads();
  for (int i = threadIdx.x; i < nr; i += blockDim.x) keys[i] = resc[i];
  __syncthreads();
  return nr;
}


// Shared-memory table accesses with explicit .shared instructions (a table
// pointer carried through lambdas is otherwise treated as generic, and
// generic-address atomics on shared memory are far slower).
CEOS_DEV unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
CEOS_DEV int ld_volatile_shared(unsigned a) {
  int v;
  asm volatile("ld.volatile.shared.b32 %0, [%1];" : "=r"(v) : "r"(a));
  return v;
}
CEOS_DEV int cas_shared(unsigned a, int cmp, int val) {
  int old;
  asm volatile("atom.shared.cas.b32 %0, [%1], %2, %3;" : "=r"(old) : "r"(a), "r"(cmp), "r"(val) : "memory");
  return old;
}
CEOS_DEV void red_add_shared(unsigned a, float v) {
  asm volatile("red.shared.add.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}

// Find or insert `id`; returns the slot index. Open addressing with double
// hashing over a prime capacity (so every probe sequence visits every slot):
// at the load factors a shared-memory table runs at, probe lengths have a
// geometric tail instead of linear probing's clustered one, which matters
// because every probed column ends at a barrier that waits for the longest
// insertion. The capacity exceeds the number of insertions, so a free slot
// always exists; the sequence is still bounded and returns -1 if it ran out.
//
// In shared memory the table is two arrays, keys[cap] (int32 ids, -1 = empty)
// and vals[cap] (float sums), so that the random key probes spread over all 32
// banks; in global memory slot s is the pair (keys[2s], value), one sector.
// `fresh` reports that this call inserted the id.
template <bool SMEM>
CEOS_DEV int table_slot(int* keys, int cap, int id, bool& fresh) {
  const uint32_t h1 = (uint32_t)id * 0x9E3779B1u;
  const uint32_t h2 = ((uint32_t)id ^ 0x5bd1e995u) * 0x85EBCA6Bu;
  int s = (int)(((uint64_t)h1 * (uint32_t)cap) >> 32);
  const int step = 1 + (int)(((uint64_t)h2 * (uint32_t)(cap - 1)) >> 32);
  const unsigned base = SMEM ? smem_u32(keys) : 0u;
  fresh = false;
  for (int probe = 0; probe < cap; ++probe) {
    int cur;
    if (SMEM)
      cur = ld_volatile_shared(base + 4u * (unsigned)s);  // shared: keys array
    else
      cur = *reinterpret_cast<volatile int*>(&keys[2 * s]);  // global: (key, value) pairs
    if (cur == id) return s;
    if (cur == -1) {
      const int prev = SMEM ? cas_shared(base + 4u * (unsigned)s, -1, id) : atomicCAS(&keys[2 * s], -1, id);
      if (prev == -1) {
        fresh = true;
        return s;
      }
      if (prev == id) return s;
    }
    s += step;
    if (s >= cap) s -= cap;
  }
  return -1;
}

// Add v to the value of slot `sl`. Within one probed column every id is
// distinct when `distinct` holds, so no other thread touches the slot during
// the column and a plain read-modify-write is exact; a fresh slot takes v
// itself (its sum starts at the additive identity -0.0f, and -0.0f + v == v),
// stored without reading. Otherwise (streamCEOs, whose stale rows may repeat
// an id) the add is atomic on a value initialised to -0.0f.
template <bool SMEM>
CEOS_DEV void table_add(float* vals, int sl, float v, bool distinct, bool fresh) {
  float* val = vals + (SMEM ? sl : 2 * sl);
  if (distinct) {
    *reinterpret_cast<volatile float*>(val) = fresh ? v : *reinterpret_cast<volatile float*>(val) + v;
  } else if (SMEM) {
    red_add_shared(smem_u32(val), v);
  } else {
    atomicAdd(val, v);
  }
}

struct QLayout {
  size_t qv, pkeys, probes, topk, resc, cand, hist, maybe, table, total;
};

constexpr int kMaybe = 1024;  // threshold-bin buffer of the histogram top-K

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
  L.resc = o;
  o = al16(o + (size_t)(a.rescore > 0 ? a.rescore : 0) * 8);
  L.cand = o;
  if (mode == Q_ESTIMATE) o = al16(o + (size_t)(a.c > 0 ? a.c : 1) * 8);
  L.hist = o;
  o = al16(o + (size_t)kHistBins * 4);
  L.maybe = o;
  o = al16(o + (size_t)kMaybe * 8);
  L.table = o;
  if (a.table_in_smem) o = al16(o + (size_t)a.table_cap * 8);
  L.total = o;
  return L;
}

size_t query_buckets_smem(const QueryArgs& a, int mode) { return q_layout(a, mode).total; }

constexpr int kPrefetch = 4;  // bucket columns in flight
constexpr int kEPT = 2;       // bucket entries per thread per column on the prefetch path

// MINB = CTAs per SM the register budget is sized for: 1 (128 registers per
// thread) when a shared-memory table leaves room for one CTA, 2 (64 registers)
// when two CTAs fit, so that the latency-bound accumulation has 32 warps per SM.
template <int MODE, bool SMEM_TABLE, int MINB>
__global__ void __launch_bounds__(kQueryThreads, MINB) k_query_buckets(QueryArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ uint32_t scratch[16];
  const QLayout Lq = q_layout(a, MODE);
  float* qv = reinterpret_cast<float*>(sm + Lq.qv);
  uint64_t* pkeys = reinterpret_cast<uint64_t*>(sm + Lq.pkeys);
  int* probes = reinterpret_cast<int*>(sm + Lq.probes);
  uint64_t* topk = reinterpret_cast<uint64_t*>(sm + Lq.topk);
  uint64_t* resc = reinterpret_cast<uint64_t*>(sm + Lq.resc);
  uint64_t* cand = reinterpret_cast<uint64_t*>(sm + Lq.cand);
  uint32_t* hist = reinterpret_cast<uint32_t*>(sm + Lq.hist);
  uint64_t* maybe = reinterpret_cast<uint64_t*>(sm + Lq.maybe);
  // The table pointer's address space is fixed per instantiation so that
  // shared-memory tables get shared (not generic) loads and atomics.
  const int cap_max = a.table_cap;
  // Shared-memory tables are two arrays (keys, then values) so that random key
  // probes spread over all banks; global tables interleave (key, value) so
  // that a slot is one 32-byte sector. Slot i: tkeys[kS * i], tvals[kS * i].
  constexpr int kS = SMEM_TABLE ? 1 : 2;
  int* tkeys = SMEM_TABLE ? reinterpret_cast<int*>(sm + Lq.table)
                          : reinterpret_cast<int*>(a.gtable + (long)blockIdx.x * cap_max);
  float* tvals = SMEM_TABLE ? reinterpret_cast<float*>(tkeys + cap_max) : reinterpret_cast<float*>(tkeys) + 1;
  const int s_cap = np2(a.s > 0 ? a.s : 1);
  const int k_cap = np2(a.k > 0 ? a.k : 1);
  const unsigned long npts = (unsigned long)a.n_points;

  const int nq = a.d_nq ? min(*a.d_nq, a.nq) : a.nq;
  for (int q = blockIdx.x; q < nq; q += gridDim.x) {
    const int sq = a.q_s ? min(a.q_s[q], a.s) : a.s;
    const int kq = a.q_k ? min(a.q_k[q], a.k) : a.k;
    const long oq = a.q_off ? a.q_off[q] : (long)q * a.k;
    // per-query table capacity (a prime sized for this query's probes)
    const int cap = a.q_cap ? min(a.q_cap[q], cap_max) : cap_max;
    const int rq = (a.q_k && a.rescore_per_k > 0) ? min(a.rescore, a.rescore_per_k * kq) : a.rescore;
    for (int j = threadIdx.x; j < a.ldx; j += blockDim.x) qv[j] = a.Q[(long)q * a.ldx + j];
    // ---- 1. probes: top-s |projection|, consumed worst first ----
    const float* qp = a.qproj + (long)q * a.C;
    const int ns = block_topk_hist_sorted(
        [&](long i, float& v, int& id) {
          v = abs_ref(qp[i]);
          id = (int)i;
          return true;
        },
        (long)a.C, sq, pkeys, s_cap, hist, maybe, kMaybe, scratch);
    for (int j = threadIdx.x; j < ns; j += blockDim.x) {
      const int col = key_id(pkeys[ns - 1 - j]);
      probes[j] = qp[col] < 0 ? -(col + 1) : (col + 1);
    }
    for (int i = threadIdx.x; i < cap; i += blockDim.x) {
      tkeys[kS * i] = -1;
      if (!a.distinct_ids) tvals[kS * i] = -0.0f;
    }
    __syncthreads();
    // ---- 2. ordered accumulation / union of the probed bucket prefixes ----
    auto insert = [&](int id, float v) {
      if ((unsigned long)(unsigned)id >= npts) return;  // stale streamCEOs row
      bool fresh;
      const int sl = table_slot<SMEM_TABLE>(tkeys, cap, id, fresh);
      if (sl < 0) return;
      if (MODE == Q_ESTIMATE) table_add<SMEM_TABLE>(tvals, sl, v, a.distinct_ids != 0, fresh);
    };
    if (a.p <= kEPT * (int)blockDim.x) {
      int pid[kPrefetch][kEPT];
      float pv[kPrefetch][kEPT];
      auto load = [&](int j, int (&ids)[kEPT], float (&vs)[kEPT]) {
        const int tag = probes[j];
        const int col = (tag < 0 ? -tag : tag) - 1;
        const long base = (2L * col + (tag < 0 ? 1 : 0)) * a.m;
#pragma unroll
        for (int t = 0; t < kEPT; ++t) {
          const int e = threadIdx.x + t * blockDim.x;
          ids[t] = -1;
          vs[t] = 0.0f;
          if (e < a.p) {
            ids[t] = __ldg(a.bids + base + e);
            if (MODE == Q_ESTIMATE) vs[t] = __ldg(a.bvals + base + e);
          }
        }
      };
#pragma unroll
      for (int u = 0; u < kPrefetch; ++u)
        if (u < ns) load(u, pid[u], pv[u]);
      for (int j0 = 0; j0 < ns; j0 += kPrefetch) {
#pragma unroll
        for (int u = 0; u < kPrefetch; ++u) {
          const int j = j0 + u;
          if (j < ns) {
#pragma unroll
            for (int t = 0; t < kEPT; ++t)
              if (pid[u][t] != -1) insert(pid[u][t], pv[u][t]);
            if (j + kPrefetch < ns) load(j + kPrefetch, pid[u], pv[u]);
            if (MODE == Q_ESTIMATE) __syncthreads();
          }
        }
      }
    } else {
      for (int j = 0; j < ns; ++j) {
        const int tag = probes[j];
        const int col = (tag < 0 ? -tag : tag) - 1;
        const long base = (2L * col + (tag < 0 ? 1 : 0)) * a.m;
        for (int e = threadIdx.x; e < a.p; e += blockDim.x)
          insert(__ldg(a.bids + base + e), MODE == Q_ESTIMATE ? __ldg(a.bvals + base + e) : 0.0f);
        if (MODE == Q_ESTIMATE) __syncthreads();
      }
    }
    __syncthreads();
    int nres;
    if (MODE == Q_ESTIMATE) {
      // ---- 3. top-c candidates by estimate ----
      const int nc = block_topk_hist(
          [&](long i, float& v, int& id) {
            id = reinterpret_cast<volatile int*>(tkeys)[kS * i];
            v = reinterpret_cast<volatile float*>(tvals)[kS * i];
            return id >= 0;
          },
          (long)cap, a.c, cand, hist, maybe, kMaybe, scratch);
      // ---- 4. rerank (exact, or bfloat16 scan + exact rescore), in place ----
      const int ns2 = score_candidates(a, rq, cand, nc, qv, resc, hist, maybe, kMaybe, scratch);
      nres = block_topk_hist_sorted(
          [&](long i, float& v, int& id) {
            const uint64_t k = cand[i];
            v = key_val(k);
            id = key_id(k);
            return true;
          },
          (long)ns2, kq, topk, k_cap, hist, maybe, kMaybe, scratch);
    } else {
      // ---- union rerank in place over the table slots ----
      if (a.Xb != nullptr && rq > 0) {
        // split precision: bfloat16 scan over the slots, exact rescore of the best
        const int lane = threadIdx.x & 31;
        const int g = lane & 7;
        const int grp = lane >> 3;
        const int warp = threadIdx.x >> 5;
        const int nw = blockDim.x >> 5;
        for (int base = warp * 4; base < cap; base += nw * 4) {
          const int i = base + grp;
          const int id = i < cap ? reinterpret_cast<volatile int*>(tkeys)[kS * i] : -1;
          const bool active = id >= 0;
          const float d = dot_g8_bf16(qv, active ? row_ptr_bf16(a, id) : nullptr, a.ldx >> 3, g, active);
          if (active && g == 0) tvals[kS * i] = d;
        }
        __syncthreads();
        const int nr = block_topk_hist(
            [&](long i, float& v, int& id) {
              id = reinterpret_cast<volatile int*>(tkeys)[kS * i];
              v = reinterpret_cast<volatile float*>(tvals)[kS * i];
              return id >= 0;
            },
            (long)cap, rq, resc, hist, maybe, kMaybe, scratch);
        rerank_inplace(resc, nr, qv, a.ldx, [&](int id) { return row_ptr(a, id); });
        __syncthreads();
        nres = block_topk_hist_sorted(
            [&](long i, float& v, int& id) {
              v = key_val(resc[i]);
              id = key_id(resc[i]);
              return true;
            },
            (long)nr, kq, topk, k_cap, hist, maybe, kMaybe, scratch);
      } else {
      {
        const int lane = threadIdx.x & 31;
        const int g = lane & 7;
        const int grp = lane >> 3;
        const int warp = threadIdx.x >> 5;
        const int nw = blockDim.x >> 5;
        for (int base = warp * 4; base < cap; base += nw * 4) {
          const int i = base + grp;
          const int id = i < cap ? reinterpret_cast<volatile int*>(tkeys)[kS * i] : -1;
          const bool active = id >= 0;
          const float d = dot_g8(qv, active ? row_ptr(a, id) : qv, a.ldx >> 2, g, active);
          if (active && g == 0) tvals[kS * i] = d;
        }
      }
      __syncthreads();
      nres = block_topk_hist_sorted(
          [&](long i, float& v, int& id) {
            id = reinterpret_cast<volatile int*>(tkeys)[kS * i];
            v = reinterpret_cast<volatile float*>(tvals)[kS * i];
            return id >= 0;
          },
          (long)cap, kq, topk, k_cap, hist, maybe, kMaybe, scratch);
      }
    }
    for (int i = threadIdx.x; i < kq; i += blockDim.x) {
      a.out_ids[oq + i] = i < nres ? key_id(topk[i]) : 0;
      a.out_d[oq + i] = i < nres ? key_val(topk[i]) : 0.0f;
    }
    __syncthreads();
  }
}

template <int MODE, bool SM, int MINB>
static cudaError_t launch_qb(const QueryArgs& a, int grid, size_t smem, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(k_query_buckets<MODE, SM, MINB>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_query_buckets<MODE, SM, MINB><<<grid, kQueryThreads, smem, st>>>(a);
  return cudaGetLastError();
}

// Two CTAs per SM when their shared memory fits (the 64-register variant).
static bool two_per_sm(size_t smem) {
  int dev = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return 2 * (smem + 1024) <= (size_t)per_sm;
}

template <int MODE>
static cudaError_t launch_mode(const QueryArgs& a, int grid, size_t smem, cudaStream_t st) {
  if (!a.table_in_smem) return launch_qb<MODE, false, 2>(a, grid, smem, st);
  return two_per_sm(smem) ? launch_qb<MODE, true, 2>(a, grid, smem, st)
                          : launch_qb<MODE, true, 1>(a, grid, smem, st);
}

cudaError_t launch_query_buckets(const QueryArgs& a, int mode, int grid, size_t smem,
                                 cudaStream_t st) {
  if (a.nq <= 0) return cudaSuccess;
  return mode == Q_ESTIMATE ? launch_mode<Q_ESTIMATE>(a, grid, smem, st)
                            : launch_mode<Q_UNION>(a, grid, smem, st);
}

template <int MODE, bool SM, int MINB>
static int occ_qb(size_t smem) {
  int n = 0;
  cudaError_t e = cudaFuncSetAttribute(k_query_buckets<MODE, SM, MINB>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_query_buckets<MODE, SM, MINB>,
                                                      kQueryThreads, smem);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n;
}

template <int MODE>
static int occ_mode(size_t smem, bool table_in_smem) {
  if (!table_in_smem) return occ_qb<MODE, false, 2>(smem);
  return two_per_sm(smem) ? occ_qb<MODE, true, 2>(smem) : occ_qb<MODE, true, 1>(smem);
}

int query_buckets_blocks_per_sm(int mode, size_t smem, bool table_in_smem) {
  return mode == Q_ESTIMATE ? occ_mode<Q_ESTIMATE>(smem, table_in_smem)
                            : occ_mode<Q_UNION>(smem, table_in_smem);
}

// ---------------------------------------------------------------------------
// Sort-based coCEOs-Est accumulation.
//
// The estimate of an id is the sum of its values over the probed columns in
// probe order (src/CEOs.cpp:562-610). Instead of a hash table, the CTA
// gathers the s x p probed (id, value) pairs in probe order into a per-CTA
// scratch and brings equal ids together with stable scatters (one contiguous
// segment per warp, warp-private digit offsets, lanes ranked by ballots), so
// that the pairs of one id stay in probe order and their sums are the
// reference's (first value as is, then added term by term):
//   * ids below 2^20 (partitioned accumulation): ONE stable scatter by
//     id >> 10 into at most 1024 partitions of 1024 ids. Each warp then
//     walks the partitions of its share (a contiguous run of the scattered
//     pairs) 32 pairs at a time, summing into a shared-memory table of 1024
//     floats indexed by id & 1023; a one-byte tag per slot names the
//     partition whose id the slot holds. Lanes that hit the same slot are
//     applied by the lowest of them in lane order (a match per 32 pairs);
//     when a pair of a later partition reaches a slot, the slot's finished
//     sum is written out first, and the remaining slots are written out at
//     the end;
//   * larger ids: a stable LSD radix sort (8-bit digits) and in-order sums
//     over each run of equal ids.
// Entries whose id is not a live point (stale streamCEOs rows) are mapped to
// id n_points and dropped. The sums form a compact candidate list for the
// top-c; rerank and top-k are as in k_query_buckets.

constexpr int kRadixBins = 256;
constexpr int kSortWarps = kQueryThreads / 32;
constexpr int kPartTableBits = 10;                // ids per accumulation table
constexpr int kPartTable = 1 << kPartTableBits;
constexpr int kPartMaxBits = 10;                  // partitions: at most 1024
constexpr int kPartIdBits = kPartTableBits + kPartMaxBits;
// shared-memory region of the sort phase (aliases cand / hist / maybe)
constexpr size_t kPartCountsBytes = (size_t)kSortWarps * (1 << kPartMaxBits) * 4;  // digit counts
constexpr size_t kPartTablesBytes = (size_t)kSortWarps * kPartTable * 4;           // alias the counts
constexpr size_t kPartTagOff = kPartCountsBytes > kPartTablesBytes ? kPartCountsBytes : kPartTablesBytes;
constexpr size_t kPartStageOff = kPartTagOff + (size_t)kSortWarps * kPartTable;    // one byte per slot
constexpr size_t kPartStartOff = kPartStageOff + (size_t)kSortWarps * 32 * 8;
constexpr size_t kPartRegion = kPartStartOff + (((size_t)(1 << kPartMaxBits) + 1) * 4 + 15) / 16 * 16;
constexpr size_t kLsdRegion = (size_t)2 * kSortWarps * kRadixBins * 4;

struct SLayout {
  size_t qv, pkeys, probes, topk, resc, cand, hist, maybe, rhist, total;
};

__host__ __device__ inline SLayout s_layout(const QueryArgs& a) {
  SLayout L;
  size_t o = 0;
  L.qv = o;
  o = al16(o + (size_t)a.ldx * 4);
  L.pkeys = o;
  o = al16(o + (size_t)np2(a.s > 0 ? a.s : 1) * 8);
  L.probes = o;
  o = al16(o + (size_t)(a.s > 0 ? a.s : 1) * 4);
  L.topk = o;
  o = al16(o + (size_t)np2(a.k > 0 ? a.k : 1) * 8);
  L.resc = o;
  o = al16(o + (size_t)(a.rescore > 0 ? a.rescore : 0) * 8);
  L.cand = o;
  o = al16(o + (size_t)(a.c > 0 ? a.c : 1) * 8);
  L.hist = o;
  o = al16(o + (size_t)kHistBins * 4);
  L.maybe = o;
  o = al16(o + (size_t)kMaybe * 8);
  // the digit tables, partition starts and accumulation tables are live only
  // during the sort and the sums, when cand / hist / maybe are not: they
  // share that space (sized for either path, so that a launch configured for
  // one index size stays valid as a stream index grows)
  L.rhist = L.cand;
  const size_t rend = al16(L.rhist + (kPartRegion > kLsdRegion ? kPartRegion : kLsdRegion));
  L.total = o > rend ? o : rend;
  return L;
}

size_t query_sorted_smem(const QueryArgs& a) { return s_layout(a).total; }

template <int MINB>
__global__ void __launch_bounds__(kQueryThreads, MINB) k_query_sorted(QueryArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ uint32_t scratch[16];
  __shared__ int wsum[kQueryThreads / 32];
  __shared__ int wcnt[kQueryThreads / 32];
  const SLayout Lq = s_layout(a);
  float* qv = reinterpret_cast<float*>(sm + Lq.qv);
  uint64_t* pkeys = reinterpret_cast<uint64_t*>(sm + Lq.pkeys);
  int* probes = reinterpret_cast<int*>(sm + Lq.probes);
  uint64_t* topk = reinterpret_cast<uint64_t*>(sm + Lq.topk);
  uint64_t* resc = reinterpret_cast<uint64_t*>(sm + Lq.resc);
  uint64_t* cand = reinterpret_cast<uint64_t*>(sm + Lq.cand);
  uint32_t* hist = reinterpret_cast<uint32_t*>(sm + Lq.hist);
  uint64_t* maybe = reinterpret_cast<uint64_t*>(sm + Lq.maybe);
  // digit counts per warp segment: [2][kSortWarps][kRadixBins], the current
  // pass's table and the next pass's, filled while this pass scatters
  int* rh_all = reinterpret_cast<int*>(sm + Lq.rhist);
  const int s_cap = np2(a.s > 0 ? a.s : 1);
  const int k_cap = np2(a.k > 0 ? a.k : 1);
  const int npts = (int)a.n_points;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // the first scatter pass writes bufA: the buffers of all CTAs' first passes
  // (the only pass of the partitioned accumulation) form one contiguous range
  int2* bufA = a.sort_scratch + (long)blockIdx.x * a.sort_cap;
  int2* bufB = a.sort_scratch + ((long)gridDim.x + blockIdx.x) * a.sort_cap;

  const int nq = a.d_nq ? min(*a.d_nq, a.nq) : a.nq;
  for (int q = blockIdx.x; q < nq; q += gridDim.x) {
    const int sq = a.q_s ? min(a.q_s[q], a.s) : a.s;
    const int kq = a.q_k ? min(a.q_k[q], a.k) : a.k;
    const long oq = a.q_off ? a.q_off[q] : (long)q * a.k;
    const int rq = (a.q_k && a.rescore_per_k > 0) ? min(a.rescore, a.rescore_per_k * kq) : a.rescore;
    for (int j = threadIdx.x; j < a.ldx; j += blockDim.x) qv[j] = a.Q[(long)q * a.ldx + j];
    // ---- 1. probes: top-s |projection|, consumed worst first ----
    // (taken from a.probes when k_probe_select chose them for every query of
    // the launch beforehand: same selection, same order)
    int ns;
    if (a.probes != nullptr && a.q_s == nullptr) {
      ns = a.s;
      for (int j = threadIdx.x; j < ns; j += blockDim.x) probes[j] = a.probes[(long)q * a.s + j];
    } else {
      const float* qp = a.qproj + (long)q * a.C;
      ns = block_topk_hist_sorted(
          [&](long i, float& v, int& id) {
            v = abs_ref(qp[i]);
            id = (int)i;
            return true;
          },
          (long)a.C, sq, pkeys, s_cap, hist, maybe, kMaybe, scratch);
      for (int j = threadIdx.x; j < ns; j += blockDim.x) {
        const int col = key_id(pkeys[ns - 1 - j]);
        probes[j] = qp[col] < 0 ? -(col + 1) : (col + 1);
      }
    }
    __syncthreads();
    // ---- 2. digit counts of the probed pairs ----
    // Pair t = j * p + e is entry e of the j-th probed column (probe order).
    // Warp w owns the probed columns [jw0, jw1), a contiguous run of pairs;
    // it counts its run's first-pass digits, and the first scatter pass below
    // reads the same run straight from the bucket table (no gathered copy).
    const int E = ns * a.p;
    constexpr int kU = 8;  // independent loads in flight per thread in every pass
    const int seg = (E + kSortWarps - 1) / kSortWarps;
    const int jw0 = (int)((long)warp * ns / kSortWarps), jw1 = (int)((long)(warp + 1) * ns / kSortWarps);
    // partitioned accumulation: digit = id >> tb (hb bits); else 8-bit LSD digits
    const bool part = a.id_bits <= kPartIdBits;
    const int tb = min(a.id_bits, kPartTableBits);
    const int hb = part ? a.id_bits - tb : 8;
    const int nbins = 1 << hb;
    const int dshift0 = part ? tb : 0;
    for (int i = threadIdx.x; i < (part ? kSortWarps * nbins : 2 * kSortWarps * kRadixBins); i += blockDim.x)
      rh_all[i] = 0;
    __syncthreads();
    auto column = [&](int j, const int*& bid, const float*& bval) {
      const int tag = probes[j];
      const int col = (tag < 0 ? -tag : tag) - 1;
      const long base = (2L * col + (tag < 0 ? 1 : 0)) * a.m;
      bid = a.bids + base;
      bval = a.bvals + base;
    };
    {
      int* myh0 = rh_all + warp * nbins;
      for (int j = jw0; j < jw1; ++j) {
        const int* bid;
        const float* bval;
        column(j, bid, bval);
        for (int e0 = 0; e0 < a.p; e0 += 32 * kU) {
          int id[kU];
#pragma unroll
          for (int u = 0; u < kU; ++u) {
            const int e = e0 + 32 * u + lane;
            id[u] = e < a.p ? __ldg(bid + e) : 0;
          }
#pragma unroll
          for (int u = 0; u < kU; ++u) {
            if (e0 + 32 * u + lane < a.p) {
              const int i = (unsigned)id[u] >= (unsigned)npts ? npts : id[u];  // stale row: dropped below
              atomicAdd(&myh0[(i >> dshift0) & (nbins - 1)], 1);
            }
          }
        }
      }
    }
    __syncthreads();
    // ---- 3. stable scatter(s) by id digits ----
    int2* src = bufB;
    int2* dst = bufA;
    const int w0 = min(E, warp * seg), w1 = min(E, w0 + seg);
    int* pstart = reinterpret_cast<int*>(sm + Lq.rhist + kPartStartOff);
    const int npass = part ? 1 : (a.id_bits + 7) / 8;
    int cur = 0;
    for (int ps = 0; ps < npass; ++ps, cur ^= 1) {
      const int shift = part ? tb : 8 * ps;
      int* rh = rh_all + (part ? 0 : cur * kSortWarps * kRadixBins);
      int* rn = rh_all + (cur ^ 1) * kSortWarps * kRadixBins;
      int* myh = rh + warp * nbins;
      const bool more = !part && shift + 8 < a.id_bits;
      // digit d: exclusive offset over digits, then over warps within the
      // digit; thread t owns digits [t*dper, (t+1)*dper)
      const int dper = (nbins + kQueryThreads - 1) / kQueryThreads;
      const int d0 = threadIdx.x * dper;
      int tot = 0;
      for (int j = 0; j < dper; ++j)
        if (d0 + j < nbins)
          for (int w = 0; w < kSortWarps; ++w) tot += rh[w * nbins + d0 + j];
      int inc = tot;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
      }
      if (lane == 31) wsum[warp] = inc;
      __syncthreads();
      {
        int off = inc - tot;
        for (int w = 0; w < warp; ++w) off += wsum[w];
        for (int j = 0; j < dper; ++j) {
          const int d = d0 + j;
          if (d >= nbins) break;
          if (part) pstart[d] = off;
          for (int w = 0; w < kSortWarps; ++w) {
            const int c = rh[w * nbins + d];
            rh[w * nbins + d] = off;
            off += c;
          }
        }
        if (part && threadIdx.x == 0) pstart[nbins] = E;
      }
      __syncthreads();
      // one 32-pair step: lanes with a pair are ranked among the lanes of equal
      // digit (lanes without one get a key no digit has), in lane order
      // Columns of a CEOs / coCEOs index hold distinct ids, and one 32-pair
      // step reads one column, so lanes of equal digit hold different ids: their
      // order within the partition cannot change a sum, and a shared-memory
      // atomic places them. Stream columns (repeats) are ranked in lane order.
      const bool atom_scatter = part && a.distinct_ids;
      auto place = [&](const int2 v, const bool has) {
        const int dg = has ? ((v.x >> shift) & (nbins - 1)) : 0;
        if (atom_scatter) {
          if (has) {
            int b;
            asm volatile("atom.shared.add.u32 %0, [%1], 1;" : "=r"(b) : "r"(smem_u32(myh + dg)) : "memory");
            dst[b] = v;
          }
          return;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, has ? dg : nbins + lane);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        const int b = has ? myh[dg] : 0;
        __syncwarp();
        if (has) {
          dst[b + rank] = v;
          if (rank == 0) myh[dg] = b + __popc(peers);
          // the next pass's digit counts, by destination segment
          if (more) atomicAdd(&rn[((b + rank) / seg) * kRadixBins + ((v.x >> (shift + 8)) & 255)], 1);
        }
        __syncwarp();
      };
      if (ps == 0) {
        // the warp's run of probed columns, straight from the bucket table
        for (int j = jw0; j < jw1; ++j) {
          const int* bid;
          const float* bval;
          column(j, bid, bval);
          for (int e0 = 0; e0 < a.p; e0 += 32 * kU) {
            int2 v[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
              const int e = e0 + 32 * u + lane;
              v[u] = make_int2(0, 0);
              if (e < a.p) {
                const int id = __ldg(bid + e);
                v[u] = make_int2((unsigned)id >= (unsigned)npts ? npts : id, __float_as_int(__ldg(bval + e)));
              }
            }
#pragma unroll
            for (int u = 0; u < kU; ++u) {
              if (e0 + 32 * u >= a.p) break;
              place(v[u], e0 + 32 * u + lane < a.p);
            }
          }
        }
      } else {
        for (int c0 = w0; c0 < w1; c0 += 32 * kU) {
          int2 v[kU];
#pragma unroll
          for (int u = 0; u < kU; ++u) {
            const int i = c0 + 32 * u + lane;
            v[u] = i < w1 ? src[i] : make_int2(0, 0);
          }
#pragma unroll
          for (int u = 0; u < kU; ++u) place(v[u], c0 + 32 * u + lane < w1);
        }
      }
      __syncthreads();
      if (!part)
        for (int i = threadIdx.x; i < kSortWarps * kRadixBins; i += blockDim.x) rh[i] = 0;  // next-next pass
      int2* t = src;
      src = dst;
      dst = t;
    }
    // ---- 4. sums in probe order -> compact (value, id) list in dst ----
    if (threadIdx.x == 0) {
      scratch[8] = 0u;
      scratch[9] = 0xffffffffu;  // min key of the sums
      scratch[10] = 0u;          // max key
    }
    __syncthreads();
    uint32_t klo = 0xffffffffu, khi = 0u;
    if (part) {
      // each warp: the partitions [Pa, Pb), a contiguous run [e0, e1) of src;
      // its sums overwrite the front of the run
      const int TR = 1 << tb;
      float* tab = reinterpret_cast<float*>(sm + Lq.rhist) + (size_t)warp * kPartTable;
      uint8_t* tag = reinterpret_cast<uint8_t*>(sm + Lq.rhist + kPartTagOff) + (size_t)warp * kPartTable;
      float* stv = reinterpret_cast<float*>(sm + Lq.rhist + kPartStageOff) + warp * 64;
      int* stt = reinterpret_cast<int*>(stv + 32);
      for (int i = lane; i < kPartTable / 4; i += 32) reinterpret_cast<uint32_t*>(tag)[i] = 0u;
      if (lane == 0) wcnt[warp] = 0;
      __syncwarp();
      const int Pa = (int)((long)warp * nbins / kSortWarps);
      const int Pb = (int)((long)(warp + 1) * nbins / kSortWarps);
      const int e0 = pstart[Pa], e1 = pstart[Pb];
      // the sums are written in place over the partitioned pairs: a sum is
      // emitted after at least one pair of its id was read, so its position
      // (the warp's emit count) stays below every pair still to be read
      int2* wout = src + e0;
      int wbase = 0;
      for (int c0 = e0; c0 < e1; c0 += 32 * kU) {
        int2 v[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int i = c0 + 32 * u + lane;
          v[u] = i < e1 ? src[i] : make_int2(npts, 0);
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          if (c0 + 32 * u >= e1) break;
          const int id = v[u].x;
          const bool act = id < npts;  // past e1 or a stale row: nothing to add
          const int loc = id & (TR - 1);
          stv[lane] = __int_as_float(v[u].y);
          stt[lane] = (id >> tb) - Pa + 1;
          // lanes on the same slot: the lowest applies them all, in lane
          // (= partition, then probe) order
          const unsigned peers = __match_any_sync(0xffffffffu, act ? loc : TR + lane);
          __syncwarp();
          const bool lead = act && __ffs(peers) - 1 == lane;
          int ct = 0;
          float t = 0.f;
          unsigned rest = lead ? peers : 0u;
          if (lead) {
            ct = tag[loc];
            t = tab[loc];
          }
          // every lane takes part in each round, so the finished sums of a
          // round get consecutive positions from one ballot
          while (__any_sync(0xffffffffu, rest != 0u)) {
            bool em = false;
            int et = 0;
            float ev = 0.f;
            if (rest) {
              const int l = __ffs(rest) - 1;
              rest &= rest - 1u;
              const int tm = stt[l];
              const float vm = stv[l];
              if (tm == ct) {
                t = t + vm;
              } else {
                em = ct != 0;  // the slot's previous id is finished
                et = ct;
                ev = t;
                ct = tm;
                t = vm;  // first value of the id as is
              }
            }
            const unsigned m = __ballot_sync(0xffffffffu, em);
            if (em) {
              wout[wbase + __popc(m & ((1u << lane) - 1u))] =
                  make_int2(((Pa + et - 1) << tb) | loc, __float_as_int(ev));
              klo = min(klo, fkey(ev));
              khi = max(khi, fkey(ev));
            }
            wbase += __popc(m);
          }
          if (lead) {
            tag[loc] = (uint8_t)ct;
            tab[loc] = t;
          }
          __syncwarp();
        }
      }
      // the slots still held
      for (int loc = lane; loc < TR; loc += 32) {
        const int ct = tag[loc];
        const unsigned m = __ballot_sync(0xffffffffu, ct != 0);
        if (ct != 0) {
          const float sv = tab[loc];
          wout[wbase + __popc(m & ((1u << lane) - 1u))] = make_int2(((Pa + ct - 1) << tb) | loc, __float_as_int(sv));
          klo = min(klo, fkey(sv));
          khi = max(khi, fkey(sv));
        }
        wbase += __popc(m);
      }
      if (lane == 0) wcnt[warp] = wbase;
      __syncwarp();
      // the warp's sums fill src[e0, e0 + cnt); the rest of its run is marked
      // empty, and the top-c reads all of src[0, E) (no packing copy)
      for (int i = e0 + wcnt[warp] + lane; i < e1; i += 32) src[i] = make_int2(-1, 0);
      __syncthreads();
      if (threadIdx.x == 0) {
        int tot = 0;
        for (int w = 0; w < kSortWarps; ++w) tot += wcnt[w];
        scratch[8] = (uint32_t)tot;
      }
    } else {
      // each warp takes 32 consecutive elements per step; the previous id
      // comes from the neighbour lane, so a step needs one load per lane (and
      // a run that continues past the step is walked by its head lane)
      for (int c0 = warp * 32 * kU; c0 < E; c0 += kSortWarps * 32 * kU) {
        int2 v[kU];
        int prev0 = -1;
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int i = c0 + 32 * u + lane;
          v[u] = i < E ? src[i] : make_int2(-1, 0);
        }
        if (lane == 0 && c0 > 0) prev0 = src[c0 - 1].x;
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int i = c0 + 32 * u + lane;
          int prev = __shfl_up_sync(0xffffffffu, v[u].x, 1);
          const int last = __shfl_sync(0xffffffffu, v[u > 0 ? u - 1 : 0].x, 31);
          if (lane == 0) prev = u == 0 ? prev0 : last;
          const int id = v[u].x;
          const bool head = i < E && id < npts && id != prev;
          float sum = head ? __int_as_float(v[u].y) : 0.0f;
          if (head) {
            // the run's following values, in order; four pairs per round trip
            int j = i + 1;
            bool go = true;
            while (go && j < E) {
              int2 w[4];
#pragma unroll
              for (int t = 0; t < 4; ++t) w[t] = j + t < E ? src[j + t] : make_int2(-1, 0);
#pragma unroll
              for (int t = 0; t < 4; ++t) {
                if (go && w[t].x == id) {
                  sum = sum + __int_as_float(w[t].y);
                } else {
                  go = false;
                }
              }
              j += 4;
            }
          }
          const uint32_t pos = warp_reserve(head, &scratch[8]);
          if (head) {
            dst[pos] = make_int2(id, __float_as_int(sum));
            klo = min(klo, fkey(sum));
            khi = max(khi, fkey(sum));
          }
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      klo = min(klo, __shfl_xor_sync(0xffffffffu, klo, o));
      khi = max(khi, __shfl_xor_sync(0xffffffffu, khi, o));
    }
    if (lane == 0) {
      atomicMin(&scratch[9], klo);
      atomicMax(&scratch[10], khi);
    }
    __syncthreads();
    const int U = (int)scratch[8];
    const uint32_t pre[3] = {scratch[9], scratch[10], (uint32_t)U};
    __syncthreads();
    // ---- 5. top-c by estimate, rerank, top-k ----
    // the sums: dst[0, U) compact (radix path), or dst[0, E) with empty
    // entries (id -1) between the warps' runs (partitioned path)
    const int2* sums = part ? src : dst;
    auto sget = [&](long i, float& v, int& id) {
      const int2 w = sums[i];
      id = w.x;
      v = __int_as_float(w.y);
      return w.x >= 0;
    };
    // eight items in flight per thread, and the next round prefetched: the
    // sums come from L2 or HBM
    const int nc = block_topk_hist<false, 8>(sget, (long)(part ? E : U), a.c, cand, hist, maybe, kMaybe, scratch,
                                             pre, sums);
    const int ns2 = score_candidates(a, rq, cand, nc, qv, resc, hist, maybe, kMaybe, scratch);
    const int nres = block_topk_hist_sorted(
        [&](long i, float& v, int& id) {
          const uint64_t k = cand[i];
          v = key_val(k);
          id = key_id(k);
          return true;
        },
        (long)ns2, kq, topk, k_cap, hist, maybe, kMaybe, scratch);
    for (int i = threadIdx.x; i < kq; i += blockDim.x) {
      a.out_ids[oq + i] = i < nres ? key_id(topk[i]) : 0;
      a.out_d[oq + i] = i < nres ? key_val(topk[i]) : 0.0f;
    }
    __syncthreads();
  }
}


cudaError_t launch_query_sorted(const QueryArgs& a, int grid, size_t smem, cudaStream_t st) {
  if (a.nq <= 0) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_query_sorted<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  k_query_sorted<2><<<grid, kQueryThreads, smem, st>>>(a);
  return cudaGetLastError();
}

bool query_table_preferred(const QueryArgs& a) {
  // the shared-memory table wins while two 512-thread CTAs fit per SM
  QueryArgs t = a;
  t.table_in_smem = 1;
  return two_per_sm(q_layout(t, Q_ESTIMATE).total);
}

int query_sorted_blocks_per_sm(size_t smem) {
  int n = 0;
  cudaError_t e = cudaFuncSetAttribute(k_query_sorted<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_query_sorted<2>, kQueryThreads, smem);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n;
}

// ---------------------------------------------------------------------------
// Dense CEOs-Est.

__global__ void __launch_bounds__(256) k_probe_select(QueryArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ uint32_t scratch[16];
  const int s_cap = np2(a.s > 0 ? a.s : 1);
  uint64_t* pk = reinterpret_cast<uint64_t*>(sm);
  uint32_t* hist = reinterpret_cast<uint32_t*>(sm + (size_t)s_cap * 8);
  uint64_t* maybe = reinterpret_cast<uint64_t*>(sm + (size_t)s_cap * 8 + (size_t)kHistBins * 4);
  const int q = blockIdx.x;
  const float* qp = a.qproj + (long)q * a.C;
  const int ns = block_topk_hist_sorted(
      [&](long i, float& v, int& id) {
        v = abs_ref(qp[i]);
        id = (int)i;
        return true;
      },
      (long)a.C, a.s, pk, s_cap, hist, maybe, kMaybe, scratch);
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
  const size_t smem = (size_t)np2(a.s) * 8 + (size_t)kHistBins * 4 + (size_t)kMaybe * 8;
  cudaError_t e =
      cudaFuncSetAttribute(k_probe_select, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
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
  __shared__ uint32_t scratch[16];
  const int qi = blockIdx.x;
  const int q = q0 + qi;
  const int k_cap = np2(a.k > 0 ? a.k : 1);
  float* qv = reinterpret_cast<float*>(sm);
  uint64_t* topk = reinterpret_cast<uint64_t*>(sm + al16((size_t)a.ldx * 4));
  uint64_t* resc = topk + k_cap;
  uint64_t* cand = resc + (a.rescore > 0 ? a.rescore : 0);
  uint32_t* hist = reinterpret_cast<uint32_t*>(cand + (a.c > 0 ? a.c : 1));
  uint64_t* maybe = reinterpret_cast<uint64_t*>(hist + kHistBins);
  for (int j = threadIdx.x; j < a.ldx; j += blockDim.x) qv[j] = a.Q[(long)q * a.ldx + j];
  const float* est = a.est + (long)qi * a.n_points;
  const int nc = block_topk_hist(
      [&](long i, float& v, int& id) {
        v = est[i];
        id = (int)i;
        return true;
      },
      a.n_points, a.c, cand, hist, maybe, kMaybe, scratch);
  const int ns2 = score_candidates(a, a.rescore, cand, nc, qv, resc, hist, maybe, kMaybe, scratch);
  const int nres = block_topk_hist_sorted(
      [&](long i, float& v, int& id) {
        v = key_val(cand[i]);
        id = key_id(cand[i]);
        return true;
      },
      (long)ns2, a.k, topk, k_cap, hist, maybe, kMaybe, scratch);
  for (int i = threadIdx.x; i < a.k; i += blockDim.x) {
    a.out_ids[(long)q * a.k + i] = i < nres ? key_id(topk[i]) : 0;
    a.out_d[(long)q * a.k + i] = i < nres ? key_val(topk[i]) : 0.0f;
  }
}

cudaError_t launch_dense_select_rerank(const QueryArgs& a, int q0, int nq_chunk, cudaStream_t st) {
  if (nq_chunk <= 0) return cudaSuccess;
  const int k_cap = np2(a.k > 0 ? a.k : 1);
  const size_t smem = al16((size_t)a.ldx * 4) + (size_t)k_cap * 8 +
                      (size_t)(a.rescore > 0 ? a.rescore : 0) * 8 + (size_t)(a.c > 0 ? a.c : 1) * 8 +
                      (size_t)kHistBins * 4 + (size_t)kMaybe * 8;
  cudaError_t e = cudaFuncSetAttribute(k_dense_select_rerank,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_dense_select_rerank<<<nq_chunk, kQueryThreads, smem, st>>>(a, q0);
  return cudaGetLastError();
}

}  // namespace ceos
