// CPU oracle for the CEOs / coCEOs / streamCEOs index path.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker for the GPU library: the
// parity tests, the smoke check and the CPU-baseline leg of the benchmark load
// it. Nothing in the shipped library (ceos_gb300/) links, calls or falls back
// to it.
//
// It restates, loop for loop, the reference's CPU algorithms (NinhPham/CEOs):
//   src/Utilities.cpp:21-41    bitHD3Generator (seeded +-1 sign bits)
//   src/fht_avx.c / fht.h:11   fht_float (in-place unnormalised Walsh-Hadamard)
//   src/CEOs.cpp:18-98         build_CEOs          (dense projections)
//   src/CEOs.cpp:107-297       search_CEOs         (dense estimate, top-c, rerank)
//   src/CEOs.cpp:311-441       build_coCEOs_Est    (two-ended top-m per column)
//   src/CEOs.cpp:450-694       search_coCEOs_Est   (bucket estimate, top-c, rerank)
//   src/CEOs.cpp:708-840       build_CEOs_Hash     (ids-only buckets)
//   src/CEOs.cpp:850-1066      search_CEOs_Hash    (candidate union, rerank)
//   src/streamCEOs.cpp:9-161   streamCEOs::build
//   src/streamCEOs.cpp:174-369 streamCEOs::update  (FIFO delete, merge)
//   src/streamCEOs.cpp:378-612 streamCEOs::estimate_search
//   src/streamCEOs.cpp:621-877 streamCEOs::hash_search
//   src/CEOs.h:63-81, src/streamCEOs.h:53-70  parameter setters
//
// Deliberate, documented differences from the reference (each one only
// matters at exact ties or on inputs where the reference has undefined
// behaviour):
//  * Every bounded min-heap orders its items by a TOTAL order: value first,
//    compared through the order-preserving uint32 image of the float (so -0 <
//    +0), then smaller id wins. The reference (src/Header.h:53-80) compares
//    the value only, so which of several exactly tied items it keeps depends
//    on heap layout / robin_map iteration order.
//  * The rerank inner product uses one fixed association (8 strided fused
//    multiply-add chains over float4 chunks, then a butterfly; see dot_fma),
//    the one the GPU kernels compute. The reference uses Eigen's vectorised
//    dot, whose association differs at the ulp level.
//  * Per-query estimates are kept in an open-addressing table of this file
//    (EstTable) instead of tsl::robin_map; the accumulation order per point
//    (probe pop order) is the reference's, and the total order above makes
//    the candidate selection independent of the table's iteration order.
//  * Parameter errors return a negative status instead of exit(1); asking for
//    more candidates than exist uses all of them instead of popping an empty
//    heap (src/CEOs.cpp:634-647 is undefined behaviour there).
//  * Ids are int32 (the reference stores them as float inside matrix_P,
//    exact only below 2^24 points).
//  * streamCEOs searches skip bucket entries whose id is not a live point
//    (stale rows left by update can hold such ids; the reference indexes
//    deque_X out of range there).
//
// Pins: the FWHT is checked bit for bit against the reference's own FFHT
// sources compiled by oracle/Makefile (target `ref`), and the sign generator
// against std::default_random_engine and a known-answer vector. The whole
// index path is checked against the reference's own CEOs / streamCEOs classes,
// compiled unchanged by the same Makefile against stand-ins for the Eigen and
// Boost headers (oracle/refshim): bucket values bit-identical, bucket ids
// equal up to the order of exact ties, search ids equal and scores within
// 1e-5 relative (tests/test_reference_pins.py, golden fixtures made by
// tests/golden/make_reference_golden.py).

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <queue>
#include <random>
#include <vector>
#include <deque>
#include <omp.h>

namespace {

// ----------------------------------------------------------------------------
// Status codes (same values as the GPU library's C ABI).
enum {
  ST_OK = 0,
  ST_BAD_ARG = -1,
  ST_NOT_BUILT = -2,
  ST_PROBED_POINTS = -3,   // n_probed_points > top_m
  ST_PROBED_VECTORS = -4,  // n_probed_vectors > n_proj * n_repeats (stream: > n_proj)
  ST_UPDATE_DEL = -5,      // n_del > current size
  ST_UPDATE_TOPM = -6,     // top_m > size after update
};

// ----------------------------------------------------------------------------
// Total order used by every selection.
static inline uint32_t fkey(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

struct Item {
  int id;
  float val;
};

// a ranks strictly before b: larger value, then smaller id.
static inline bool better(const Item& a, const Item& b) {
  uint32_t ka = fkey(a.val), kb = fkey(b.val);
  if (ka != kb) return ka > kb;
  return a.id < b.id;
}

// priority_queue comparator: top() is the WORST item (the next one to evict),
// mirroring priority_queue<IFPair, vector<IFPair>, greater<>> of the reference.
struct WorstOnTop {
  bool operator()(const Item& a, const Item& b) const { return better(a, b); }
};
using MinQue = std::priority_queue<Item, std::vector<Item>, WorstOnTop>;

// Per-query estimate accumulator: open addressing with linear probing over a
// power-of-two table sized for the number of probed pairs. add() keeps the
// first value of an id as is and adds later ones in call order, which is the
// reference's per-point accumulation (src/CEOs.cpp:562-610).
struct EstTable {
  std::vector<int> keys;
  std::vector<float> vals;
  std::vector<int> used;  // occupied slots, in first-insertion order
  unsigned mask = 0;
  void reset(size_t expected) {
    size_t cap = 16;
    while (cap < 2 * expected + 16) cap <<= 1;
    if (keys.size() != cap) {
      keys.assign(cap, -1);
      vals.assign(cap, 0.0f);
    } else {
      for (int sl : used) keys[sl] = -1;
    }
    used.clear();
    mask = (unsigned)cap - 1;
  }
  void add(int id, float v) {
    unsigned h = ((unsigned)id * 2654435761u) & mask;
    while (true) {
      if (keys[h] == id) {
        vals[h] += v;
        return;
      }
      if (keys[h] == -1) {
        keys[h] = id;
        vals[h] = v;
        used.push_back((int)h);
        return;
      }
      h = (h + 1) & mask;
    }
  }
  template <typename F>
  void for_each(F f) const {
    for (int sl : used) f(keys[sl], vals[sl]);
  }
};

// Bounded insertion used by every top-K loop of the reference
// (e.g. src/CEOs.cpp:393-399): push while not full, else replace the worst if
// the newcomer ranks above it.
static inline void offer(MinQue& q, int K, int id, float v) {
  if ((int)q.size() < K) {
    q.push(Item{id, v});
  } else if (K > 0 && better(Item{id, v}, q.top())) {
    q.pop();
    q.push(Item{id, v});
  }
}

// ----------------------------------------------------------------------------
// Seeded sign bits, restating src/Utilities.cpp:21-41.
//
// std::default_random_engine in libstdc++ is the Park-Miller "minimal
// standard" generator minstd_rand0: x <- 16807 * x mod (2^31 - 1), seeded with
// s mod (2^31 - 1) (a zero remainder becomes 1). uniform_int_distribution<
// uint32_t>(0, 1) draws from it by rejection: the generator's range
// [1, 2^31 - 2] has 2^31 - 2 values; values are shifted to start at 0, the
// top two (which would bias the split) are rejected, and the rest are divided
// by (2^31 - 2) / 2 so that the lower half gives 0 and the upper half 1.
struct ParkMiller {
  uint64_t x;
  explicit ParkMiller(uint64_t seed) {
    uint64_t s = seed % 2147483647ull;
    x = (s == 0) ? 1 : s;
  }
  uint32_t next() {
    x = (x * 16807ull) % 2147483647ull;
    return (uint32_t)x;
  }
};

static inline uint32_t draw_bit(ParkMiller& g) {
  const uint64_t span = 2147483645ull;          // max - min of the generator
  const uint64_t buckets = 2;                   // values of the distribution
  const uint64_t scale = span / buckets;        // 1073741822
  const uint64_t limit = buckets * scale;       // 2147483644
  uint64_t r;
  do {
    r = (uint64_t)g.next() - 1ull;
  } while (r >= limit);
  return (uint32_t)(r / scale);
}

static void sign_bits(int n_bits, int seed, std::vector<uint8_t>& bits) {
  // A negative seed means "seed from the wall clock" (src/Utilities.cpp:23-25);
  // the count is truncated to `unsigned` as in the reference.
  unsigned s = (unsigned)std::chrono::system_clock::now().time_since_epoch().count();
  if (seed >= 0) s = (unsigned)seed;
  ParkMiller g(s);
  bits.assign(n_bits, 0);
  for (int i = 0; i < n_bits; ++i) bits[i] = (uint8_t)(draw_bit(g) & 1u);
}

// ----------------------------------------------------------------------------
// In-place unnormalised Walsh-Hadamard transform. Stage s (s = 0, 1, ...)
// combines the elements whose indices differ in bit s: (a, b) -> (a+b, a-b).
// This ascending stage order reproduces the reference's FFHT fht_float
// (src/fht_avx.c:10081) bit for bit.
static void fwht(float* v, int log_n) {
  const int n = 1 << log_n;
  for (int s = 0; s < log_n; ++s) {
    const int h = 1 << s;
    for (int base = 0; base < n; base += 2 * h) {
      for (int j = base; j < base + h; ++j) {
        float a = v[j], b = v[j + h];
        v[j] = a + b;
        v[j + h] = a - b;
      }
    }
  }
}

static int log2_int(int F) {
  int l = 0;
  while ((1 << l) < F) ++l;
  return l;
}

// fhtDim rule of src/CEOs.h:76-79 and src/streamCEOs.h:64-67.
static int fht_dim(int n_proj, int n_features) {
  if (n_proj < n_features) return 1 << (int)std::ceil(std::log2((double)n_features));
  return 1 << (int)std::ceil(std::log2((double)n_proj));
}

// One row through R x (3 x (sign flip, FWHT)), keeping the first D outputs of
// each repeat (src/CEOs.cpp:61-87). out has R*D floats.
static void project_row(const float* x, int d, int F, int D, int R,
                        const uint8_t* bits, float* out, std::vector<float>& tmp,
                        std::vector<float>& rot) {
  const int L = log2_int(F);
  tmp.assign(F, 0.0f);
  for (int j = 0; j < d; ++j) tmp[j] = x[j];
  rot.resize(F);
  for (int r = 0; r < R; ++r) {
    std::copy(tmp.begin(), tmp.end(), rot.begin());
    const int base = F * 3 * r;
    for (int i = 0; i < 3; ++i) {
      const uint8_t* b = bits + base + i * F;
      for (int j = 0; j < F; ++j) rot[j] *= (2.0f * (float)b[j] - 1.0f);
      fwht(rot.data(), L);
    }
    std::copy(rot.begin(), rot.begin() + D, out + (size_t)r * D);
  }
}

// Projections of n rows, row-major n x (R*D).
static void project_rows(const float* X, long n, int d, int F, int D, int R,
                         const uint8_t* bits, float* P) {
  const int C = D * R;
#pragma omp parallel
  {
    std::vector<float> tmp, rot;
#pragma omp for schedule(static)
    for (long i = 0; i < n; ++i)
      project_row(X + (size_t)i * d, d, F, D, R, bits, P + (size_t)i * C, tmp, rot);
  }
}

// Rerank score in the GPU library's canonical order: the row is split into
// float4 chunks; partial sum g (g = 0..7) is a sequential fused multiply-add
// chain over chunks g, g+8, g+16, ... (4 elements each, elements past d
// count as zero), and the 8 partial sums are combined as a butterfly (pairs
// g, g^4; then g, g^2; then g, g^1), the value lane 0 of an 8-lane group ends
// with.
static inline float dot_fma(const float* a, const float* b, int d) {
  const int n4 = (d + 3) / 4;
  float p[8];
  for (int g = 0; g < 8; ++g) {
    float s = 0.0f;
    for (int c = g; c < n4; c += 8)
      for (int e = 0; e < 4; ++e) {
        const int j = 4 * c + e;
        if (j < d) s = std::fma(a[j], b[j], s);
      }
    p[g] = s;
  }
  float t[8];
  for (int g = 0; g < 8; ++g) t[g] = p[g] + p[g ^ 4];
  for (int g = 0; g < 8; ++g) p[g] = t[g] + t[g ^ 2];
  for (int g = 0; g < 8; ++g) t[g] = p[g] + p[g ^ 1];
  return t[0];
}

// Two-ended top-m of one projection column, written as the reference lays
// out matrix_P (src/CEOs.cpp:385-428): close ids/values sorted best first,
// far ids and negated values sorted best first.
static void select_column(const float* col_vals, long n, long stride, int m,
                          int* ids_close, float* vals_close, int* ids_far,
                          float* vals_far) {
  MinQue close, far;
  for (long i = 0; i < n; ++i) {
    float v = col_vals[i * stride];
    offer(close, m, (int)i, v);
    offer(far, m, (int)i, -v);
  }
  for (int r = m - 1; r >= 0; --r) {
    ids_close[r] = close.top().id;
    vals_close[r] = close.top().val;
    close.pop();
    ids_far[r] = far.top().id;
    vals_far[r] = far.top().val;
    far.pop();
  }
}

// Two-ended top-m of every projection column of n rows, laid out as
// select_column writes them ([C][2][m] ids and values). The rows are
// projected in chunks, so only chunk x C projections exist at a time (the
// reference holds the whole n x C matrix, src/CEOs.cpp:335); each column's
// heaps take the rows in ascending order, as select_column's do, so the
// buckets are the same.
static void select_all_columns(const float* X, long n, int d, int F, int D, int R,
                               const uint8_t* bits, int m, int* B_ids, float* B_vals) {
  const int C = D * R;
  const long chunk = 2048;
  const int cb = 16;  // columns per task: one 64-byte line of a projected row
  std::vector<MinQue> close(C), far(C);
  std::vector<float> P((size_t)std::min<long>(chunk, std::max<long>(n, 1)) * C);
  for (long r0 = 0; r0 < n; r0 += chunk) {
    const long nr = std::min(chunk, n - r0);
    project_rows(X + (size_t)r0 * d, nr, d, F, D, R, bits, P.data());
#pragma omp parallel for schedule(dynamic, 1)
    for (int c0 = 0; c0 < C; c0 += cb) {
      const int c1 = std::min(C, c0 + cb);
      for (long i = 0; i < nr; ++i) {
        const float* row = P.data() + (size_t)i * C;
        for (int c = c0; c < c1; ++c) {
          offer(close[c], m, (int)(r0 + i), row[c]);
          offer(far[c], m, (int)(r0 + i), -row[c]);
        }
      }
    }
  }
#pragma omp parallel for schedule(dynamic, 16)
  for (int c = 0; c < C; ++c) {
    const size_t o = (size_t)c * 2 * m;
    for (int r = m - 1; r >= 0; --r) {
      B_ids[o + r] = close[c].top().id;
      B_vals[o + r] = close[c].top().val;
      close[c].pop();
      B_ids[o + m + r] = far[c].top().id;
      B_vals[o + m + r] = far[c].top().val;
      far[c].pop();
    }
  }
}

// Probe selection of the search functions (e.g. src/CEOs.cpp:526-548):
// returns the s probed columns as signed tags +-(col+1) in POP order
// (worst first), which is the order the estimate loops consume them in.
static void probe_columns(const float* proj, int C, int s, std::vector<int>& pop_order) {
  MinQue q;
  for (int c = 0; c < C; ++c) {
    float v = proj[c];
    // abs as the reference computes it: -0.0 stays -0.0 with a positive tag.
    float a = v;
    if (v < 0) a = -v;
    offer(q, s, c, a);
  }
  // Remember the sign of each kept column.
  pop_order.clear();
  while (!q.empty()) {
    int c = q.top().id;
    q.pop();
    pop_order.push_back(proj[c] < 0 ? -(c + 1) : (c + 1));
  }
}

// Final top-k, written best first; slots beyond the number of results stay 0
// (src/CEOs.cpp:263-270).
static void write_topk(MinQue& q, int k, int* ids, float* dists) {
  for (int j = 0; j < k; ++j) {
    ids[j] = 0;
    dists[j] = 0.0f;
  }
  for (int j = (int)q.size() - 1; j >= 0; --j) {
    ids[j] = q.top().id;
    dists[j] = q.top().val;
    q.pop();
  }
}

// ----------------------------------------------------------------------------
// Split precision (no reference counterpart): rows rounded to bfloat16
// (round to nearest, ties to even) for an approximate scan; the best
// `rescore` candidates of the scan are rescored exactly with dot_fma.
static inline float bf16_round(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) {  // inf / nan: truncate (keep nan quiet)
    u &= 0xffff0000u;
    if ((x != x)) u |= 0x00400000u;
  } else {
    u += 0x7fffu + ((u >> 16) & 1u);
    u &= 0xffff0000u;
  }
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}

// Approximate score: 8 partial sums over 8-element chunks (chunk c goes to
// partial c mod 8), each a sequential fused multiply-add chain of q_j and the
// bfloat16-rounded x_j, combined by the same butterfly as dot_fma.
static inline float dot_bf16(const float* q, const float* x, int d) {
  const int n8 = (d + 7) / 8;
  float p[8];
  for (int g = 0; g < 8; ++g) {
    float s = 0.0f;
    for (int c = g; c < n8; c += 8)
      for (int e = 0; e < 8; ++e) {
        const int j = 8 * c + e;
        if (j < d) s = std::fma(q[j], bf16_round(x[j]), s);
      }
    p[g] = s;
  }
  float t[8];
  for (int g = 0; g < 8; ++g) t[g] = p[g] + p[g ^ 4];
  for (int g = 0; g < 8; ++g) p[g] = t[g] + t[g ^ 2];
  for (int g = 0; g < 8; ++g) t[g] = p[g] + p[g ^ 1];
  return t[0];
}

// Rerank a candidate set: plain (exact scores for all), or split (bfloat16
// scan of all, exact rescore of the best `rescore`). Returns the top-k heap.
template <typename RowFn>
static void rerank(const std::vector<int>& cand, const float* qv, int d, int k, int split,
                   int rescore, RowFn row, MinQue& topk) {
  if (!split) {
    for (int id : cand) offer(topk, k, id, dot_fma(qv, row(id), d));
    return;
  }
  MinQue approx;
  for (int id : cand) offer(approx, rescore, id, dot_bf16(qv, row(id), d));
  while (!approx.empty()) {
    const int id = approx.top().id;
    approx.pop();
    offer(topk, k, id, dot_fma(qv, row(id), d));
  }
}

// ----------------------------------------------------------------------------
// CEOs index (src/CEOs.h:18-114).
struct OracleCEOs {
  int n_points, n_features;
  int n_proj = 256, n_rotate = 3, top_m = 100, n_repeats = 1, seed = -1;
  int n_threads = -1;
  int n_probed_vectors = 10, n_probed_points = 10, n_cand = 10;
  bool centering = false;
  int split = 0, rescore_mult = 4;  // split precision: rescore rescore_mult * k
  int fhtDim = 0;
  std::vector<float> X;        // n x d
  std::vector<float> P;        // dense: n x C row-major
  std::vector<int> B_ids;      // coCEOs / hash: [C][2][m]
  std::vector<float> B_vals;   // coCEOs: [C][2][m]
  std::vector<uint8_t> bits;
  int built = 0;               // 1 dense, 2 coCEOs, 3 hash

  OracleCEOs(int n, int d) : n_points(n), n_features(d) {}

  void set_param(int D, int R, int m, int t, int s) {
    n_proj = D;
    n_repeats = R;
    top_m = m;
    n_probed_points = top_m;
    n_threads = t <= 0 ? omp_get_max_threads() : t;
    seed = s;
    fhtDim = fht_dim(n_proj, n_features);
  }

  int C() const { return n_proj * n_repeats; }

  void common_build(const float* Xin) {
    X.assign(Xin, Xin + (size_t)n_points * n_features);
    sign_bits(fhtDim * n_rotate * n_repeats, seed, bits);
  }

  void project_query(const float* q, std::vector<float>& proj, std::vector<float>& tmp,
                     std::vector<float>& rot) const {
    proj.resize(C());
    project_row(q, n_features, fhtDim, n_proj, n_repeats, bits.data(), proj.data(), tmp, rot);
  }

  // src/CEOs.cpp:18-98
  int build_dense(const float* Xin) {
    omp_set_num_threads(n_threads);
    common_build(Xin);
    P.assign((size_t)n_points * C(), 0.0f);
    project_rows(X.data(), n_points, n_features, fhtDim, n_proj, n_repeats, bits.data(), P.data());
    built = 1;
    return ST_OK;
  }

  // CEOs-Hash centering as the GPU library defines it (the reference's
  // src/CEOs.cpp:721-728 subtracts the n-vector of row means from every row,
  // which is not a column centering): column means as double sums over
  // chunks of 4096 rows, chunks added in order, rounded to float; each row
  // minus the means. The stored rows, used by the rerank, are the centered ones.
  void center_rows() {
    const long n = n_points, chunk = 4096, chunks = (n + chunk - 1) / chunk;
    std::vector<float> mu(n_features);
    for (int j = 0; j < n_features; ++j) {
      double total = 0.0;
      for (long b = 0; b < chunks; ++b) {
        double sb = 0.0;
        for (long r = b * chunk; r < std::min(n, (b + 1) * chunk); ++r) sb += (double)X[(size_t)r * n_features + j];
        total += sb;
      }
      mu[j] = (float)(total / (double)n);
    }
    for (long r = 0; r < n; ++r)
      for (int j = 0; j < n_features; ++j) X[(size_t)r * n_features + j] -= mu[j];
  }

  // src/CEOs.cpp:311-441 (with_vals) and :708-840 (ids only)
  int build_buckets(const float* Xin, bool with_vals) {
    omp_set_num_threads(n_threads);
    if (top_m < 1 || top_m > n_points) return ST_BAD_ARG;
    common_build(Xin);
    if (!with_vals && centering) center_rows();
    const int Cc = C();
    B_ids.assign((size_t)Cc * 2 * top_m, 0);
    B_vals.assign((size_t)Cc * 2 * top_m, 0.0f);
    select_all_columns(X.data(), n_points, n_features, fhtDim, n_proj, n_repeats, bits.data(), top_m,
                       B_ids.data(), B_vals.data());
    if (!with_vals) B_vals.assign(B_vals.size(), 0.0f);
    built = with_vals ? 2 : 3;
    return ST_OK;
  }

  // src/CEOs.cpp:107-297
  int search_dense(const float* Q, int nq, int k, int* ids, float* dists) {
    if (built != 1) return ST_NOT_BUILT;
    if (n_probed_vectors > C() || n_probed_vectors < 0 || k < 0 || n_cand < 0) return ST_PROBED_VECTORS;
    omp_set_num_threads(n_threads);
    const int d = n_features;
    const int Cc = C();
#pragma omp parallel
    {
      std::vector<float> proj, tmp, rot, est(n_points);
      std::vector<int> probes;
#pragma omp for schedule(dynamic, 1)
      for (int q = 0; q < nq; ++q) {
        const float* qv = Q + (size_t)q * d;
        project_query(qv, proj, tmp, rot);
        probe_columns(proj.data(), Cc, n_probed_vectors, probes);
        std::fill(est.begin(), est.end(), 0.0f);
        for (int tag : probes) {
          if (tag < 0) {
            int c = -tag - 1;
            for (int i = 0; i < n_points; ++i) est[i] -= P[(size_t)i * Cc + c];
          } else {
            int c = tag - 1;
            for (int i = 0; i < n_points; ++i) est[i] += P[(size_t)i * Cc + c];
          }
        }
        MinQue cand;
        for (int i = 0; i < n_points; ++i) offer(cand, n_cand, i, est[i]);
        std::vector<int> cids;
        while (!cand.empty()) {
          cids.push_back(cand.top().id);
          cand.pop();
        }
        MinQue topk;
        rerank(cids, qv, d, k, split, rescore_mult * k,
               [&](int id) { return &X[(size_t)id * d]; }, topk);
        write_topk(topk, k, ids + (size_t)q * k, dists + (size_t)q * k);
      }
    }
    return ST_OK;
  }

  // src/CEOs.cpp:450-694
  int search_coceos(const float* Q, int nq, int k, int* ids, float* dists) {
    if (built != 2) return ST_NOT_BUILT;
    if (n_probed_points > top_m || n_probed_points < 0) return ST_PROBED_POINTS;
    if (n_probed_vectors > C() || n_probed_vectors < 0 || k < 0 || n_cand < 0) return ST_PROBED_VECTORS;
    omp_set_num_threads(n_threads);
    const int d = n_features, m = top_m, p = n_probed_points;
    const int Cc = C();
#pragma omp parallel
    {
      std::vector<float> proj, tmp, rot;
      std::vector<int> probes;
      EstTable est;
#pragma omp for schedule(dynamic, 1)
      for (int q = 0; q < nq; ++q) {
        const float* qv = Q + (size_t)q * d;
        project_query(qv, proj, tmp, rot);
        probe_columns(proj.data(), Cc, n_probed_vectors, probes);
        est.reset(probes.size() * (size_t)std::max(p, 0));
        for (int tag : probes) {
          int c = tag < 0 ? -tag - 1 : tag - 1;
          size_t o = (size_t)c * 2 * m + (tag < 0 ? m : 0);
          for (int j = 0; j < p; ++j) est.add(B_ids[o + j], B_vals[o + j]);
        }
        MinQue cand;
        est.for_each([&](int id, float v) { offer(cand, n_cand, id, v); });
        std::vector<int> cids;
        while (!cand.empty()) {
          cids.push_back(cand.top().id);
          cand.pop();
        }
        MinQue topk;
        rerank(cids, qv, d, k, split, rescore_mult * k,
               [&](int id) { return &X[(size_t)id * d]; }, topk);
        write_topk(topk, k, ids + (size_t)q * k, dists + (size_t)q * k);
      }
    }
    return ST_OK;
  }

  // src/CEOs.cpp:850-1066
  int search_hash(const float* Q, int nq, int k, int* ids, float* dists) {
    if (built != 3) return ST_NOT_BUILT;
    if (n_probed_points > top_m || n_probed_points < 0) return ST_PROBED_POINTS;
    if (n_probed_vectors > C() || n_probed_vectors < 0 || k < 0) return ST_PROBED_VECTORS;
    omp_set_num_threads(n_threads);
    const int d = n_features, m = top_m, p = n_probed_points;
    const int Cc = C();
#pragma omp parallel
    {
      std::vector<float> proj, tmp, rot;
      std::vector<int> probes;
      std::vector<uint8_t> seen(n_points);
#pragma omp for schedule(dynamic, 1)
      for (int q = 0; q < nq; ++q) {
        const float* qv = Q + (size_t)q * d;
        project_query(qv, proj, tmp, rot);
        probe_columns(proj.data(), Cc, n_probed_vectors, probes);
        std::fill(seen.begin(), seen.end(), 0);
        for (int tag : probes) {
          int c = tag < 0 ? -tag - 1 : tag - 1;
          size_t o = (size_t)c * 2 * m + (tag < 0 ? m : 0);
          for (int j = 0; j < p; ++j) seen[B_ids[o + j]] = 1;
        }
        std::vector<int> cids;
        for (int i = 0; i < n_points; ++i)
          if (seen[i]) cids.push_back(i);
        MinQue topk;
        rerank(cids, qv, d, k, split, rescore_mult * k,
               [&](int id) { return &X[(size_t)id * d]; }, topk);
        write_topk(topk, k, ids + (size_t)q * k, dists + (size_t)q * k);
      }
    }
    return ST_OK;
  }
};

// ----------------------------------------------------------------------------
// streamCEOs (src/streamCEOs.h:12-107).
struct OracleStream {
  int n_points = 0, n_features;
  int n_proj = 256, n_rotate = 3, top_m = 100, n_repeats = 1, seed = -1;
  int n_threads = -1;
  int n_probed_vectors = 10, n_probed_points = 10, n_cand = 10;
  int split = 0, rescore_mult = 4;
  int fhtDim = 0;
  std::deque<std::vector<float>> X;
  std::vector<int> B_ids;      // [C][2][m]
  std::vector<float> B_vals;   // [C][2][m]
  std::vector<uint8_t> bits;
  bool built = false;
  // Exact maintenance (the GPU library's random-delete extension): after every
  // update or delete the buckets are the exact two-ended top-m over the live
  // rows, recomputed here from scratch.
  bool exact = false;

  explicit OracleStream(int d) : n_features(d) {}

  void rebuild_exact() {
    const int n = (int)X.size(), Cc = C();
    std::vector<float> flat((size_t)n * n_features);
    for (int i = 0; i < n; ++i) std::memcpy(&flat[(size_t)i * n_features], X[i].data(), n_features * sizeof(float));
    B_ids.assign((size_t)Cc * 2 * top_m, 0);
    B_vals.assign((size_t)Cc * 2 * top_m, 0.0f);
    select_all_columns(flat.data(), n, n_features, fhtDim, n_proj, n_repeats, bits.data(), top_m,
                       B_ids.data(), B_vals.data());
    n_points = n;
  }

  // Delete the rows with the given current ids (positions); later rows move
  // down, as erasing from a deque would.
  int delete_ids(const int* ids, int nd) {
    if (!built) return ST_NOT_BUILT;
    if (!exact) return ST_BAD_ARG;
    std::vector<int> v(ids, ids + nd);
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    for (int id : v)
      if (id < 0 || id >= (int)X.size()) return ST_BAD_ARG;
    if (top_m > (int)X.size() - (int)v.size()) return ST_UPDATE_TOPM;
    for (int i = (int)v.size() - 1; i >= 0; --i) X.erase(X.begin() + v[i]);
    omp_set_num_threads(n_threads);
    rebuild_exact();
    return ST_OK;
  }

  // src/streamCEOs.h:53-70: note n_probed_vectors (not n_probed_points) is
  // reset to top_m here.
  void set_param(int D, int R, int m, int t, int s) {
    n_proj = D;
    n_repeats = R;
    top_m = m;
    n_probed_vectors = top_m;
    n_threads = t <= 0 ? omp_get_max_threads() : t;
    seed = s;
    fhtDim = fht_dim(n_proj, n_features);
  }

  int C() const { return n_proj * n_repeats; }

  // src/streamCEOs.cpp:9-161
  int build(const float* Xin, int n) {
    if (top_m < 1 || top_m > n) return ST_BAD_ARG;
    omp_set_num_threads(n_threads);
    n_points = n;
    X.clear();
    for (int i = 0; i < n; ++i)
      X.emplace_back(Xin + (size_t)i * n_features, Xin + (size_t)(i + 1) * n_features);
    sign_bits(fhtDim * n_rotate * n_repeats, seed, bits);
    const int Cc = C();
    std::vector<float> flat((size_t)n * n_features);
    std::memcpy(flat.data(), Xin, flat.size() * sizeof(float));
    B_ids.assign((size_t)Cc * 2 * top_m, 0);
    B_vals.assign((size_t)Cc * 2 * top_m, 0.0f);
    select_all_columns(flat.data(), n, n_features, fhtDim, n_proj, n_repeats, bits.data(), top_m,
                       B_ids.data(), B_vals.data());
    built = true;
    return ST_OK;
  }

  // src/streamCEOs.cpp:174-369
  int update(const float* newX, int b, int n_del) {
    if (!built) return ST_NOT_BUILT;
    const int cur = (int)X.size();
    if (n_del < 0 || b < 0) return ST_BAD_ARG;
    if (n_del > cur) return ST_UPDATE_DEL;
    if (top_m > cur + b - n_del) return ST_UPDATE_TOPM;
    omp_set_num_threads(n_threads);
    for (int i = 0; i < b; ++i)
      X.emplace_back(newX + (size_t)i * n_features, newX + (size_t)(i + 1) * n_features);
    for (int i = 0; i < n_del; ++i) X.pop_front();
    n_points = (int)X.size();
    if (exact) {
      rebuild_exact();
      return ST_OK;
    }
    const int Cc = C(), m = top_m;
    std::vector<float> Pn((size_t)b * Cc);
    project_rows(newX, b, n_features, fhtDim, n_proj, n_repeats, bits.data(), Pn.data());
#pragma omp parallel for schedule(dynamic, 4)
    for (int c = 0; c < Cc; ++c) {
      size_t o = (size_t)c * 2 * m;
      MinQue close, far;
      // Survivors: every stored row, stale rows included (:271-287).
      for (int j = 0; j < m; ++j) {
        if (B_ids[o + j] >= n_del) close.push(Item{B_ids[o + j], B_vals[o + j]});
        if (B_ids[o + m + j] >= n_del) far.push(Item{B_ids[o + m + j], B_vals[o + m + j]});
      }
      // New points, ids continuing after the old size (:292-325).
      for (int i = 0; i < b; ++i) {
        float v = Pn[(size_t)i * Cc + c];
        offer(close, m, i + cur, v);
        offer(far, m, i + cur, -v);
      }
      // Write back rebased ids; rows past the heap size keep their old
      // contents (:331-352).
      for (int r = (int)close.size() - 1; r >= 0; --r) {
        B_ids[o + r] = close.top().id - n_del;
        B_vals[o + r] = close.top().val;
        close.pop();
      }
      for (int r = (int)far.size() - 1; r >= 0; --r) {
        B_ids[o + m + r] = far.top().id - n_del;
        B_vals[o + m + r] = far.top().val;
        far.pop();
      }
    }
    return ST_OK;
  }

  void project_query(const float* q, std::vector<float>& proj, std::vector<float>& tmp,
                     std::vector<float>& rot) const {
    proj.resize(C());
    project_row(q, n_features, fhtDim, n_proj, n_repeats, bits.data(), proj.data(), tmp, rot);
  }

  int check_query(int k) const {
    if (!built) return ST_NOT_BUILT;
    if (n_probed_points > top_m || n_probed_points < 0) return ST_PROBED_POINTS;
    if (n_probed_vectors > n_proj || n_probed_vectors < 0 || k < 0 || n_cand < 0) return ST_PROBED_VECTORS;
    return ST_OK;
  }

  // src/streamCEOs.cpp:378-612
  int estimate_search(const float* Q, int nq, int k, int* ids, float* dists) {
    int st = check_query(k);
    if (st) return st;
    omp_set_num_threads(n_threads);
    const int d = n_features, m = top_m, p = n_probed_points;
#pragma omp parallel
    {
      std::vector<float> proj, tmp, rot;
      std::vector<int> probes;
      EstTable est;
#pragma omp for schedule(dynamic, 1)
      for (int q = 0; q < nq; ++q) {
        const float* qv = Q + (size_t)q * d;
        project_query(qv, proj, tmp, rot);
        probe_columns(proj.data(), C(), n_probed_vectors, probes);
        est.reset(probes.size() * (size_t)std::max(p, 0));
        for (int tag : probes) {
          int c = tag < 0 ? -tag - 1 : tag - 1;
          size_t o = (size_t)c * 2 * m + (tag < 0 ? m : 0);
          for (int j = 0; j < p; ++j) {
            int id = B_ids[o + j];
            // A stale row (see update) can hold an id past the current size;
            // the reference then reads deque_X out of range (undefined
            // behaviour). Such entries are skipped.
            if (id < 0 || id >= n_points) continue;
            est.add(id, B_vals[o + j]);
          }
        }
        MinQue cand;
        est.for_each([&](int id, float v) { offer(cand, n_cand, id, v); });
        std::vector<int> cids;
        while (!cand.empty()) {
          cids.push_back(cand.top().id);
          cand.pop();
        }
        MinQue topk;
        rerank(cids, qv, d, k, split, rescore_mult * k, [&](int id) { return X[id].data(); }, topk);
        write_topk(topk, k, ids + (size_t)q * k, dists + (size_t)q * k);
      }
    }
    return ST_OK;
  }

  // src/streamCEOs.cpp:621-877
  int hash_search(const float* Q, int nq, int k, int* ids, float* dists) {
    int st = check_query(k);
    if (st) return st;
    omp_set_num_threads(n_threads);
    const int d = n_features, m = top_m, p = n_probed_points;
#pragma omp parallel
    {
      std::vector<float> proj, tmp, rot;
      std::vector<int> probes;
      std::vector<uint8_t> seen(n_points);
#pragma omp for schedule(dynamic, 1)
      for (int q = 0; q < nq; ++q) {
        const float* qv = Q + (size_t)q * d;
        project_query(qv, proj, tmp, rot);
        probe_columns(proj.data(), C(), n_probed_vectors, probes);
        std::fill(seen.begin(), seen.end(), 0);
        for (int tag : probes) {
          int c = tag < 0 ? -tag - 1 : tag - 1;
          size_t o = (size_t)c * 2 * m + (tag < 0 ? m : 0);
          for (int j = 0; j < p; ++j) {
            const int id = B_ids[o + j];
            if (id >= 0 && id < n_points) seen[id] = 1;  // stale ids skipped, as above
          }
        }
        std::vector<int> cids;
        for (int i = 0; i < n_points; ++i)
          if (seen[i]) cids.push_back(i);
        MinQue topk;
        rerank(cids, qv, d, k, split, rescore_mult * k, [&](int id) { return X[id].data(); }, topk);
        write_topk(topk, k, ids + (size_t)q * k, dists + (size_t)q * k);
      }
    }
    return ST_OK;
  }
};

}  // namespace

// ----------------------------------------------------------------------------
// C interface for the test harness (oracle/oracle.py).
extern "C" {

int orc_sign_bits(int n_bits, int seed, uint8_t* out) {
  if (n_bits < 0) return ST_BAD_ARG;
  std::vector<uint8_t> b;
  sign_bits(n_bits, seed, b);
  std::memcpy(out, b.data(), b.size());
  return ST_OK;
}

// The same bits drawn through the C++ standard library, to cross-check the
// restatement above.
int orc_sign_bits_std(int n_bits, int seed, uint8_t* out) {
  std::default_random_engine g((unsigned)seed);
  std::uniform_int_distribution<uint32_t> u(0, 1);
  for (int i = 0; i < n_bits; ++i) out[i] = (uint8_t)(u(g) & 1u);
  return ST_OK;
}

void orc_fwht(float* v, int log_n) { fwht(v, log_n); }

int orc_fht_dim(int n_proj, int n_features) { return fht_dim(n_proj, n_features); }

// Projections of n rows into row-major n x (R*D).
int orc_project(const float* X, long n, int d, int F, int D, int R, const uint8_t* bits,
                float* P, int n_threads) {
  if (n_threads > 0) omp_set_num_threads(n_threads);
  project_rows(X, n, d, F, D, R, bits, P);
  return ST_OK;
}

int orc_bruteforce(const float* X, long n, int d, const float* Q, int nq, int k, int* ids,
                   double* scores, int n_threads) {
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 1)
  for (int q = 0; q < nq; ++q) {
    std::vector<std::pair<double, int>> h;  // min-heap of (score, -id)
    auto worse = [](const std::pair<double, int>& a, const std::pair<double, int>& b) {
      if (a.first != b.first) return a.first > b.first;
      return a.second < b.second;
    };
    for (long i = 0; i < n; ++i) {
      double s = 0.0;
      const float* x = X + (size_t)i * d;
      const float* qq = Q + (size_t)q * d;
      for (int j = 0; j < d; ++j) s += (double)qq[j] * (double)x[j];
      std::pair<double, int> it(s, (int)i);
      if ((int)h.size() < k) {
        h.push_back(it);
        std::push_heap(h.begin(), h.end(), worse);
      } else if (k > 0 && (s > h.front().first || (s == h.front().first && (int)i < h.front().second))) {
        std::pop_heap(h.begin(), h.end(), worse);
        h.back() = it;
        std::push_heap(h.begin(), h.end(), worse);
      }
    }
    std::sort(h.begin(), h.end(), [](const std::pair<double, int>& a, const std::pair<double, int>& b) {
      if (a.first != b.first) return a.first > b.first;
      return a.second < b.second;
    });
    for (int j = 0; j < k; ++j) {
      ids[(size_t)q * k + j] = j < (int)h.size() ? h[j].second : 0;
      scores[(size_t)q * k + j] = j < (int)h.size() ? h[j].first : 0.0;
    }
  }
  return ST_OK;
}

void* orc_ceos_create(int n, int d) { return new OracleCEOs(n, d); }
void orc_ceos_destroy(void* h) { delete (OracleCEOs*)h; }
void orc_ceos_set_param(void* h, int D, int R, int m, int t, int s) {
  ((OracleCEOs*)h)->set_param(D, R, m, t, s);
}
void orc_ceos_set_query(void* h, int s, int p, int c) {
  auto* o = (OracleCEOs*)h;
  o->n_probed_vectors = s;
  o->n_probed_points = p;
  o->n_cand = c;
}
void orc_ceos_get_query(void* h, int* s, int* p, int* c) {
  auto* o = (OracleCEOs*)h;
  *s = o->n_probed_vectors;
  *p = o->n_probed_points;
  *c = o->n_cand;
}
int orc_ceos_fht_dim(void* h) { return ((OracleCEOs*)h)->fhtDim; }
void orc_ceos_set_split(void* h, int split, int mult) {
  ((OracleCEOs*)h)->split = split;
  ((OracleCEOs*)h)->rescore_mult = mult;
}
void orc_stream_set_split(void* h, int split, int mult) {
  ((OracleStream*)h)->split = split;
  ((OracleStream*)h)->rescore_mult = mult;
}
float orc_bf16_round(float x) { return bf16_round(x); }
float orc_dot_bf16(const float* q, const float* x, int d) { return dot_bf16(q, x, d); }
float orc_dot(const float* q, const float* x, int d) { return dot_fma(q, x, d); }
int orc_ceos_build_dense(void* h, const float* X) { return ((OracleCEOs*)h)->build_dense(X); }
int orc_ceos_build_coceos(void* h, const float* X) { return ((OracleCEOs*)h)->build_buckets(X, true); }
int orc_ceos_build_hash(void* h, const float* X) { return ((OracleCEOs*)h)->build_buckets(X, false); }
void orc_ceos_set_centering(void* h, int c) { ((OracleCEOs*)h)->centering = c != 0; }
int orc_ceos_search_dense(void* h, const float* Q, int nq, int k, int* ids, float* d) {
  return ((OracleCEOs*)h)->search_dense(Q, nq, k, ids, d);
}
int orc_ceos_search_coceos(void* h, const float* Q, int nq, int k, int* ids, float* d) {
  return ((OracleCEOs*)h)->search_coceos(Q, nq, k, ids, d);
}
int orc_ceos_search_hash(void* h, const float* Q, int nq, int k, int* ids, float* d) {
  return ((OracleCEOs*)h)->search_hash(Q, nq, k, ids, d);
}
// Buckets as [C][2][m] ids and values.
int orc_ceos_get_buckets(void* h, int* ids, float* vals) {
  auto* o = (OracleCEOs*)h;
  if (o->built < 2) return ST_NOT_BUILT;
  std::memcpy(ids, o->B_ids.data(), o->B_ids.size() * sizeof(int));
  std::memcpy(vals, o->B_vals.data(), o->B_vals.size() * sizeof(float));
  return ST_OK;
}
// Dense projections, row-major n x C.
int orc_ceos_get_projections(void* h, float* P) {
  auto* o = (OracleCEOs*)h;
  if (o->built != 1) return ST_NOT_BUILT;
  std::memcpy(P, o->P.data(), o->P.size() * sizeof(float));
  return ST_OK;
}

void* orc_stream_create(int d) { return new OracleStream(d); }
void orc_stream_destroy(void* h) { delete (OracleStream*)h; }
void orc_stream_set_param(void* h, int D, int R, int m, int t, int s) {
  ((OracleStream*)h)->set_param(D, R, m, t, s);
}
void orc_stream_set_query(void* h, int s, int p, int c) {
  auto* o = (OracleStream*)h;
  o->n_probed_vectors = s;
  o->n_probed_points = p;
  o->n_cand = c;
}
void orc_stream_get_query(void* h, int* s, int* p, int* c) {
  auto* o = (OracleStream*)h;
  *s = o->n_probed_vectors;
  *p = o->n_probed_points;
  *c = o->n_cand;
}
int orc_stream_size(void* h) { return (int)((OracleStream*)h)->X.size(); }
int orc_stream_build(void* h, const float* X, int n) { return ((OracleStream*)h)->build(X, n); }
int orc_stream_update(void* h, const float* X, int b, int n_del) {
  return ((OracleStream*)h)->update(X, b, n_del);
}
void orc_stream_set_exact(void* h, int exact) { ((OracleStream*)h)->exact = exact != 0; }
int orc_stream_delete(void* h, const int* ids, int n) { return ((OracleStream*)h)->delete_ids(ids, n); }
int orc_stream_estimate_search(void* h, const float* Q, int nq, int k, int* ids, float* d) {
  return ((OracleStream*)h)->estimate_search(Q, nq, k, ids, d);
}
int orc_stream_hash_search(void* h, const float* Q, int nq, int k, int* ids, float* d) {
  return ((OracleStream*)h)->hash_search(Q, nq, k, ids, d);
}
int orc_stream_get_buckets(void* h, int* ids, float* vals) {
  auto* o = (OracleStream*)h;
  if (!o->built) return ST_NOT_BUILT;
  std::memcpy(ids, o->B_ids.data(), o->B_ids.size() * sizeof(int));
  std::memcpy(vals, o->B_vals.data(), o->B_vals.size() * sizeof(float));
  return ST_OK;
}

}  // extern "C"
