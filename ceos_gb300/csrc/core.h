// Host-side index state shared by the C ABI (capi.cu) and the serving loop
// (serve.cu): device buffers, parameters with the reference's semantics
// (src/CEOs.h:52-81, src/streamCEOs.h:40-70) and the kernel orchestration of
// build and search on one CUDA stream per index. Internal to the library.
#pragma once
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <random>
#include <string>
#include <vector>

#include "../../include/ceos_gb300.h"
#include "kernels.h"

namespace ceos_host {

using namespace ceos;

inline thread_local std::string g_err;
inline int g_log = -1;

inline int log_level() {
  if (g_log < 0) {
    const char* e = std::getenv("CEOS_GB300_LOG");
    g_log = e ? std::atoi(e) : 1;
  }
  return g_log;
}

inline int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CUDA_TRY(expr)                                                                   \
  do {                                                                                   \
    cudaError_t _e = (expr);                                                             \
    if (_e != cudaSuccess)                                                               \
      return fail(CEOS_ERR_CUDA, "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                  __FILE__, __LINE__);                                                   \
  } while (0)

#define ST_TRY(expr)          \
  do {                        \
    int _s = (expr);          \
    if (_s != CEOS_OK) return _s; \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void swap(DevBuf& o) {
    std::swap(p, o.p);
    std::swap(bytes, o.bytes);
  }
  cudaError_t ensure(size_t b) {
    if (b <= bytes && p) return cudaSuccess;
    release();
    if (b == 0) b = 16;
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) {
      p = nullptr;
      bytes = 0;
      return e;
    }
    bytes = b;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <typename T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

inline int np2(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

// Hash-table capacity for a query probing s columns of p entries: the
// smallest prime >= max(64, 1.2 * s * p) (prime for double hashing), or -1
// when it would not fit an int.
inline long table_capacity(int s, int p) {
  const long pairs = (long)std::max(s, 0) * std::max(p, 0);
  long c = std::max(64L, pairs + pairs / 5 + 1);
  if (c > INT_MAX / 4) return -1;
  auto is_prime = [](long x) {
    if (x < 2) return false;
    for (long d = 2; d * d <= x; ++d)
      if (x % d == 0) return false;
    return true;
  };
  while (!is_prime(c)) ++c;
  return c;
}

inline int ilog2(int F) {
  int l = 0;
  while ((1 << l) < F) ++l;
  return l;
}

// fhtDim rule of src/CEOs.h:76-79 / src/streamCEOs.h:64-67.
inline int fht_dim(int n_proj, int n_features) {
  if (n_proj < n_features) return 1 << (int)std::ceil(std::log2((double)n_features));
  return 1 << (int)std::ceil(std::log2((double)n_proj));
}

// bitHD3Generator (src/Utilities.cpp:21-41): F*3*R bits from
// std::default_random_engine + uniform_int_distribution<uint32_t>(0, 1); a
// negative seed seeds from the wall clock.
inline void sign_bits(int n_bits, int random_seed, std::vector<uint8_t>& bits) {
  unsigned seed = (unsigned)std::chrono::system_clock::now().time_since_epoch().count();
  if (random_seed >= 0) seed = (unsigned)random_seed;
  std::default_random_engine generator(seed);
  std::uniform_int_distribution<uint32_t> unif(0, 1);
  bits.assign(n_bits, 0);
  for (int i = 0; i < n_bits; ++i) bits[i] = (uint8_t)(unif(generator) & 1u);
}

struct Timer {
  cudaStream_t st = nullptr;
  std::vector<std::string> names;
  std::vector<cudaEvent_t> ev;
  std::vector<float> ms;
  void begin(cudaStream_t s) {
    clear();
    st = s;
    mark("start");
  }
  void mark(const char* name) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    cudaEventRecord(e, st);
    ev.push_back(e);
    names.push_back(name);
  }
  void finish() {
    ms.clear();
    if (ev.empty()) return;
    cudaEventSynchronize(ev.back());
    for (size_t i = 1; i < ev.size(); ++i) {
      float t = 0;
      cudaEventElapsedTime(&t, ev[i - 1], ev[i]);
      ms.push_back(t);
    }
    for (auto e : ev) cudaEventDestroy(e);
    ev.clear();
    names.erase(names.begin());
  }
  void clear() {
    for (auto e : ev) cudaEventDestroy(e);
    ev.clear();
    names.clear();
    ms.clear();
  }
};

enum Built { B_NONE = 0, B_DENSE = 1, B_COCEOS = 2, B_HASH = 3, B_STREAM = 4 };

struct Core {
  int n_features = 0;
  int n_proj = 256, n_repeats = 1, top_m = 100, n_threads = -1, seed = -1;
  int s = 10, p = 10, c = 10;
  int centering = 0, precision = CEOS_PRECISION_FP32;
  int fht = 0, L = 0, ldx = 0;
  int device = -1, sms = 0;
  size_t smem_optin = 0;
  cudaStream_t stream = nullptr;
  std::vector<uint8_t> bits;
  int built = B_NONE;
  long n_rows = 0, head = 0, cap_rows = 0;
  DevBuf dX, dSigns, dP, dBids, dBvals;
  DevBuf dXb;  // bfloat16 copy of the rows (split precision), same ring layout
  bool xb_valid = false;
  DevBuf wStage, wQ, wQproj, wIds, wD, wTable, wProbes, wEst, wNewP, wNewX, wSort;
  Timer timer;
  int attached = 0;  // a serving loop owns the index (serve.cu)
  // streamCEOs maintenance: -1 = the reference's (FIFO update refilled from
  // new points only); >= 0 = exact, each column end keeping its best
  // top_m + reserve live points (cnt valid in dCnt) so that random deletes can
  // be absorbed, refilled from all live points when a list drops below top_m.
  int reserve = -1;
  DevBuf dCnt, dTau;
  // transform of the built index: 1 = split-precision tensor-core FWHT, taken
  // from the precision at build time and used for every later projection of
  // index rows (updates, refills), so that all bucket values come from one
  // transform; query projections use the FP32 kernel (query_proj_base)
  int proj_tensor = 0;

  int C() const { return n_proj * n_repeats; }
  // entries stored per column end (the bucket list stride)
  int stride() const { return top_m + (reserve > 0 ? reserve : 0); }

  void set_param(int D, int R, int m, int t, int sd) {
    n_proj = D;
    n_repeats = R;
    top_m = m;
    n_threads = t;
    seed = sd;
    fht = (D >= 1 && n_features >= 1) ? fht_dim(D, n_features) : 0;
    L = fht > 0 ? ilog2(fht) : 0;
    // rows padded to a multiple of 8 floats: 16-byte aligned float4 chunks of
    // the FP32 rows and 16-byte chunks of the bfloat16 copy
    ldx = (n_features + 7) & ~7;
  }

  int ensure_device() {
    if (device >= 0) {
      CUDA_TRY(cudaSetDevice(device));
      return CEOS_OK;
    }
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count < 1)
      return fail(CEOS_ERR_NO_DEVICE, "no CUDA device is visible; the CEOs GPU library has no CPU path");
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaSetDevice(dev));
    cudaDeviceProp prop;
    CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
    if (prop.major < 10)
      return fail(CEOS_ERR_NO_DEVICE, "device %s (sm_%d%d) is not a Blackwell GPU", prop.name,
                  prop.major, prop.minor);
    device = dev;
    sms = prop.multiProcessorCount;
    smem_optin = prop.sharedMemPerBlockOptin;
    CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    return CEOS_OK;
  }

  void release_all() {
    DevBuf* bufs[] = {&dX, &dSigns, &dP, &dBids, &dBvals, &dXb, &wStage, &wQ, &wQproj, &wIds,
                      &wD, &wTable, &wProbes, &wEst, &wNewP, &wNewX, &wSort, &dCnt, &dTau};
    xb_valid = false;
    for (DevBuf* b : bufs) b->release();
    built = B_NONE;
    n_rows = head = cap_rows = 0;
  }

  ~Core() {
    if (device >= 0) cudaSetDevice(device);
    release_all();
    timer.clear();
    if (stream) cudaStreamDestroy(stream);
  }

  int check_param() const {
    if (n_features < 1) return fail(CEOS_ERR_ARG, "n_features must be >= 1");
    if (n_proj < 1 || n_repeats < 1) return fail(CEOS_ERR_ARG, "n_proj and n_repeats must be >= 1");
    if (fht < 2 || fht > 4096)
      return fail(CEOS_ERR_UNSUPPORTED, "fhtDim %d outside the supported range [2, 4096]", fht);
    return CEOS_OK;
  }

  // Upload sign words: [R][3][max(F/32,1)], bit j set => multiply by +1.
  int upload_signs() {
    sign_bits(fht * 3 * n_repeats, seed, bits);
    const int words = fht >= 32 ? fht / 32 : 1;
    std::vector<uint32_t> w((size_t)n_repeats * 3 * words, 0u);
    for (int r = 0; r < n_repeats; ++r)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < fht; ++j)
          if (bits[(size_t)r * 3 * fht + (size_t)i * fht + j])
            w[((size_t)r * 3 + i) * words + (j >> 5)] |= 1u << (j & 31);
    CUDA_TRY(dSigns.ensure(w.size() * 4));
    CUDA_TRY(cudaMemcpyAsync(dSigns.p, w.data(), w.size() * 4, cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    return CEOS_OK;
  }

  // Copy n host rows (n x n_features) into dst (n x ldx, zero padded).
  int upload_rows(const float* hX, long n, float* dst) {
    if (n <= 0) return CEOS_OK;
    const size_t raw = (size_t)n * n_features * 4;
    if (ldx == n_features) {
      CUDA_TRY(cudaMemcpyAsync(dst, hX, raw, cudaMemcpyHostToDevice, stream));
      return CEOS_OK;
    }
    CUDA_TRY(wStage.ensure(raw));
    CUDA_TRY(cudaMemcpyAsync(wStage.p, hX, raw, cudaMemcpyHostToDevice, stream));
    CUDA_TRY(launch_pad_rows(wStage.as<float>(), n, n_features, dst, ldx, stream));
    return CEOS_OK;
  }

  // Rows n x n_features from a raw row-major float32 file (the reference's
  // loadbinData format, src/Utilities.cpp:142-214) into dst (n x ldx), streamed
  // through mmap and two pinned chunks, so the file never has to fit in host
  // memory at once. Defined in ingest.cu.
  int upload_rows_from_file(const char* path, long n, float* dst);

  ProjArgs proj_base() const {
    ProjArgs a;
    a.X = dX.as<float>();
    a.ldx = ldx;
    a.head = head;
    a.cap_rows = cap_rows;
    a.d = n_features;
    a.D = n_proj;
    a.R = n_repeats;
    a.signs = dSigns.as<uint32_t>();
    a.tensor = proj_tensor;
    return a;
  }

  // Query projections run on the FP32 kernel in either precision: a batch of
  // queries is too few rows for the tensor-core tiles (16 rows each, two per
  // SM) to fill the GPU, so the FP32 butterflies are faster there, and every
  // query's projection is the same whatever its batch. Only the probe choice
  // reads them; the buckets keep the index's precision.
  ProjArgs query_proj_base() const {
    ProjArgs a = proj_base();
    a.tensor = 0;
    return a;
  }

  // Two-ended top-m buckets of the n_rows rows held in dX (see select.cu);
  // m = stride() entries per column end.
  int build_buckets() {
    const long n = n_rows;
    const int m = stride(), Cc = C();
    if (m < 1 || m > n)
      return fail(CEOS_ERR_ARG, "top_m (+ reserve) (%d) must be in [1, n_points=%ld]", m, n);
    if (m > 8192) return fail(CEOS_ERR_UNSUPPORTED, "top_m (+ reserve) > 8192 is not supported");
    // ---- sample thresholds ----
    // A strided sample of S rows; the rank-r key of each column end in it is
    // that end's emission threshold. The sample holds Binomial(S, m/n) of the
    // end's true top m (mean mu = S m / n); the list comes out short only if
    // more than r of them fall in the sample, which for r = mu + 5 sqrt(mu) + 8
    // has a Poisson tail probability below 1e-8 per column end (a short list
    // is then selected exactly, never wrong).
    long S = n <= 65536 ? n : std::max(8192L, std::min(n / 8, 16L * m));
    if (S > n) S = n;
    const bool exact = (S == n);
    int rank;
    long cap;
    if (exact) {
      rank = m;
      cap = std::max(128, np2(2 * m));
    } else {
      const double mu = (double)S * m / (double)n;
      rank = (int)std::min((double)S, std::ceil(mu + 5.0 * std::sqrt(mu) + 8.0));
      const double expected = (double)rank * (double)n / (double)S;
      cap = np2((int)std::min(1e9, std::max((double)m + 64.0, 2.0 * expected)));
      cap = std::min(cap, 16384L);
      if (cap < m + 1) cap = np2(m + 1);
    }
    DevBuf samp, rowmap, th, thf, cnt, cand, failb;
    CUDA_TRY(samp.ensure((size_t)Cc * S * 4));
    if (!exact) {
      std::vector<long> rm(S);
      for (long i = 0; i < S; ++i) rm[i] = (long)((__int128)i * n / S);
      CUDA_TRY(rowmap.ensure((size_t)S * sizeof(long)));
      CUDA_TRY(cudaMemcpyAsync(rowmap.p, rm.data(), S * sizeof(long), cudaMemcpyHostToDevice, stream));
      CUDA_TRY(cudaStreamSynchronize(stream));
    }
    ProjArgs a = proj_base();
    a.row_map = exact ? nullptr : rowmap.as<long>();
    a.n_rows = S;
    a.out = samp.as<float>();  // row-major [S][C]
    // A sample of a split-precision index is projected by the FP32 kernel,
    // which splits few rows finer over the SMs than the tensor-core tiles: its
    // thresholds only filter the candidates (the float tests below compare
    // split-precision values with them), and a column end that comes up short
    // is selected exactly from the split-precision projection. An exact
    // sample (S == n) keeps the index's own precision.
    if (!exact) a.tensor = 0;
    CUDA_TRY(launch_project(a, PROJ_ROWS, L, sms, stream));
    CUDA_TRY(th.ensure((size_t)Cc * 2 * 4));
    CUDA_TRY(thf.ensure((size_t)Cc * sizeof(float2)));
    CUDA_TRY(launch_sample_thresholds(samp.as<float>(), S, Cc, rank, th.as<uint32_t>(),
                                      thf.as<float2>(), stream));
    timer.mark("sample+thresholds");
    // ---- fused projection + candidate emission ----
    CUDA_TRY(cnt.ensure((size_t)Cc * 2 * 4));
    CUDA_TRY(cudaMemsetAsync(cnt.p, 0, (size_t)Cc * 2 * 4, stream));
    CUDA_TRY(cand.ensure((size_t)Cc * 2 * cap * 8));
    CUDA_TRY(failb.ensure((size_t)Cc * 2 * 4));
    CUDA_TRY(cudaMemsetAsync(failb.p, 0, (size_t)Cc * 2 * 4, stream));
    ProjArgs e = proj_base();
    e.n_rows = n;
    e.th = th.as<uint32_t>();
    e.thf = thf.as<float2>();
    e.cnt = cnt.as<unsigned>();
    e.cand = cand.as<uint64_t>();
    e.cap = (int)cap;
    CUDA_TRY(launch_project(e, PROJ_EMIT, L, sms, stream));
    timer.mark("project+emit");
    CUDA_TRY(dBids.ensure((size_t)Cc * 2 * m * 4));
    CUDA_TRY(dBvals.ensure((size_t)Cc * 2 * m * 4));
    CUDA_TRY(launch_finish_buckets(cand.as<uint64_t>(), cnt.as<unsigned>(), (int)cap, Cc, m,
                                   dBids.as<int>(), dBvals.as<float>(), failb.as<unsigned>(), stream));
    timer.mark("select");
    if (e.tensor && L == 10) {
      // The tensor-core projection ends a CTA whose bounded wait gave up. The
      // count is read after the selection is queued (the selection only reads
      // the candidate lists within their counts and capacity), so the device
      // runs on without a host round trip; on a fault the index is released.
      const int faults = project_t5_take_faults(stream);
      if (faults != 0)
        return fail(CEOS_ERR_CUDA, "tensor-core projection: %d blocks stopped at a wait that did not complete", faults);
    }
    samp.release();
    cand.release();
    // ---- exact fallback for flagged column ends ----
    ST_TRY(exact_refill(failb.as<unsigned>(), m, m, nullptr, nullptr, &fallback_columns));
    if (fallback_columns) timer.mark("exact-fallback");
    return CEOS_OK;
  }

  // Exact top-msel over all n_rows rows for the column ends flagged in
  // d_flags ([C][2]): the flagged columns are projected for every row
  // (column-major dump, at most 2 GB at a time) and selected exactly, written
  // at stride lds; d_cnt[end] = msel when given. Synchronizes the stream.
  int exact_refill(const unsigned* d_flags, int msel, int lds, int* d_cnt, uint2* d_tau,
                   int* n_cols_out) {
    const long n = n_rows;
    const int Cc = C();
    std::vector<unsigned> hf((size_t)Cc * 2);
    CUDA_TRY(cudaMemcpyAsync(hf.data(), d_flags, hf.size() * 4, cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    std::vector<int> failed_cols;
    for (int col = 0; col < Cc; ++col)
      if (hf[2 * col] || hf[2 * col + 1]) failed_cols.push_back(col);
    if (n_cols_out) *n_cols_out = (int)failed_cols.size();
    if (failed_cols.empty()) return CEOS_OK;
    const size_t budget = (size_t)2 << 30;
    long per = std::max(1L, (long)(budget / ((size_t)n * 4)));
    DevBuf dump, colslot, colofslot;
    CUDA_TRY(colslot.ensure((size_t)Cc * 4));
    for (size_t b0 = 0; b0 < failed_cols.size(); b0 += per) {
      const int cnt_cols = (int)std::min((long)failed_cols.size() - (long)b0, per);
      std::vector<int> cs(Cc, -1), cos(cnt_cols);
      for (int i = 0; i < cnt_cols; ++i) {
        cs[failed_cols[b0 + i]] = i;
        cos[i] = failed_cols[b0 + i];
      }
      CUDA_TRY(dump.ensure((size_t)cnt_cols * n * 4));
      CUDA_TRY(colofslot.ensure((size_t)cnt_cols * 4));
      CUDA_TRY(cudaMemcpyAsync(colslot.p, cs.data(), Cc * 4, cudaMemcpyHostToDevice, stream));
      CUDA_TRY(cudaMemcpyAsync(colofslot.p, cos.data(), cnt_cols * 4, cudaMemcpyHostToDevice, stream));
      ProjArgs f = proj_base();
      f.n_rows = n;
      f.out = dump.as<float>();
      f.ld_out = n;
      f.col_slot = colslot.as<int>();
      CUDA_TRY(launch_project(f, PROJ_COLS, L, sms, stream));
      CUDA_TRY(launch_exact_buckets(dump.as<float>(), n, n, cnt_cols, colofslot.as<int>(), d_flags,
                                    msel, lds, dBids.as<int>(), dBvals.as<float>(), d_cnt, d_tau,
                                    stream));
      CUDA_TRY(cudaStreamSynchronize(stream));
    }
    return CEOS_OK;
  }

  int fallback_columns = 0;
  int refilled_columns = 0;  // column ends refilled by the last exact update / delete

  // Bfloat16 copy of the whole row ring for the split-precision scan, made
  // on the first split search after a build and kept current by updates.
  int ensure_bf16() {
    if (precision != CEOS_PRECISION_SPLIT_BF16 || xb_valid) return CEOS_OK;
    CUDA_TRY(dXb.ensure((size_t)cap_rows * ldx * 2));
    CUDA_TRY(launch_to_bf16(dX.as<float>(), cap_rows * (long)ldx, dXb.as<uint16_t>(), stream));
    xb_valid = true;
    return CEOS_OK;
  }

  // Stage queries (host or device, n x n_features) into wQ (n x ldx) and
  // project them into wQproj (n x C).
  int stage_queries(const float* Q, long nq, bool on_device) {
    CUDA_TRY(wQ.ensure((size_t)nq * ldx * 4));
    if (on_device) {
      CUDA_TRY(launch_pad_rows(Q, nq, n_features, wQ.as<float>(), ldx, stream));
    } else {
      const size_t raw = (size_t)nq * n_features * 4;
      if (ldx == n_features) {
        CUDA_TRY(cudaMemcpyAsync(wQ.p, Q, raw, cudaMemcpyHostToDevice, stream));
      } else {
        CUDA_TRY(wStage.ensure(raw));
        CUDA_TRY(cudaMemcpyAsync(wStage.p, Q, raw, cudaMemcpyHostToDevice, stream));
        CUDA_TRY(launch_pad_rows(wStage.as<float>(), nq, n_features, wQ.as<float>(), ldx, stream));
      }
    }
    timer.mark("h2d+stage");
    CUDA_TRY(wQproj.ensure((size_t)nq * C() * 4));
    ProjArgs a = query_proj_base();
    a.X = wQ.as<float>();
    a.head = 0;
    a.cap_rows = LONG_MAX;
    a.n_rows = nq;
    a.out = wQproj.as<float>();
    CUDA_TRY(launch_project(a, PROJ_ROWS, L, sms, stream));
    timer.mark("project");
    return CEOS_OK;
  }

  QueryArgs query_base(long nq, int k) const {
    QueryArgs q;
    q.Q = wQ.as<float>();
    q.qproj = wQproj.as<float>();
    q.nq = (int)nq;
    q.d = n_features;
    q.ldx = ldx;
    q.C = C();
    q.s = s;
    q.p = p;
    q.m = stride();
    q.c = c;
    q.k = k;
    q.X = dX.as<float>();
    q.head = head;
    q.cap_rows = cap_rows;
    q.n_points = n_rows;
    q.bids = dBids.as<int>();
    q.bvals = dBvals.as<float>();
    q.P = dP.as<float>();
    q.distinct_ids = (built != B_STREAM || reserve >= 0) ? 1 : 0;
    if (precision == CEOS_PRECISION_SPLIT_BF16) {
      q.Xb = dXb.as<uint16_t>();
      q.rescore = 4 * k;
    }
    return q;
  }

  // coCEOs-Est / CEOs-Hash / stream searches over the buckets.
  int search_buckets(int mode, const float* Q, long nq, int k, int32_t* ids, float* dists,
                     bool on_device, cudaStream_t user_stream) {
    (void)user_stream;
    ST_TRY(ensure_bf16());
    timer.begin(stream);
    ST_TRY(stage_queries(Q, nq, on_device));
    QueryArgs q = query_base(nq, k);
    int32_t* out_ids = ids;
    float* out_d = dists;
    if (!on_device) {
      CUDA_TRY(wIds.ensure((size_t)nq * k * 4));
      CUDA_TRY(wD.ensure((size_t)nq * k * 4));
      out_ids = wIds.as<int32_t>();
      out_d = wD.as<float>();
    }
    q.out_ids = out_ids;
    q.out_d = out_d;
    if (mode == Q_ESTIMATE && use_sorted(q)) {
      ST_TRY(sorted_args(q, nq));
      const size_t ssm = query_sorted_smem(q);
      const int grid = (int)std::min<long>(nq, (long)sms * std::max(query_sorted_blocks_per_sm(ssm), 1));
      CUDA_TRY(wSort.ensure((size_t)std::max(grid, 1) * 2 * q.sort_cap * 8));
      q.sort_scratch = wSort.as<int2>();
      // the probes of every query, chosen by a kernel of their own (many small
      // blocks hide the selection's latency better than the query CTAs)
      CUDA_TRY(wProbes.ensure((size_t)nq * std::max(s, 1) * 4));
      q.probes_out = wProbes.as<int>();
      CUDA_TRY(launch_probe_select(q, stream));
      q.probes = wProbes.as<int>();
      CUDA_TRY(launch_query_sorted(q, std::max(grid, 1), ssm, stream));
      return finish_search(mode, nq, k, ids, dists, out_ids, out_d, on_device);
    }
    const long tc = table_capacity(s, p);
    if (tc < 0) return fail(CEOS_ERR_UNSUPPORTED, "n_probed_vectors * n_probed_points too large");
    q.table_cap = (int)tc;
    q.table_in_smem = 1;
    size_t smem = query_buckets_smem(q, mode);
    int grid;
    if (smem <= smem_optin) {
      int per_sm = query_blocks_per_sm(mode, smem, true);
      grid = (int)std::min<long>(nq, (long)sms * std::max(per_sm, 1));
    } else {
      q.table_in_smem = 0;
      smem = query_buckets_smem(q, mode);
      if (smem > smem_optin)
        return fail(CEOS_ERR_UNSUPPORTED, "query working set (n_cand=%d, n_neighbors=%d) exceeds shared memory", c, k);
      int per_sm = query_blocks_per_sm(mode, smem, false);
      grid = (int)std::min<long>(nq, (long)sms * std::max(per_sm, 1));
      CUDA_TRY(wTable.ensure((size_t)grid * tc * 8));
      q.gtable = wTable.as<uint64_t>();
    }
    CUDA_TRY(launch_query_buckets(q, mode, std::max(grid, 1), smem, stream));
    return finish_search(mode, nq, k, ids, dists, out_ids, out_d, on_device);
  }

  // Estimate searches run sorted (k_query_sorted) unless the hash table fits
  // in shared memory with two CTAs per SM; CEOS_GB300_QUERY=table|sorted
  // forces one form for indexes whose columns hold distinct ids.
  bool use_sorted(const QueryArgs& q) const {
    // A FIFO stream's stale bucket rows can repeat an id within one column.
    // Only the sorted kernel adds such repeats in entry order (the table's
    // shared adds would apply them in hardware order), so it always runs.
    if (!q.distinct_ids) return true;
    const char* e = std::getenv("CEOS_GB300_QUERY");
    if (e && std::strcmp(e, "table") == 0) return false;
    if (e && std::strcmp(e, "sorted") == 0) return true;
    const long tc = table_capacity(q.s, q.p);
    if (tc < 0) return true;
    QueryArgs t = q;
    t.table_cap = (int)tc;
    return !query_table_preferred(t);
  }

  int sorted_args(QueryArgs& q, long nq) const {
    (void)nq;
    const long pairs = (long)std::max(s, 0) * std::max(p, 0);
    if (pairs > INT_MAX / 2) return fail(CEOS_ERR_UNSUPPORTED, "n_probed_vectors * n_probed_points too large");
    q.sort_cap = std::max(pairs, 1L);
    int bits = 1;
    while (bits < 31 && (1L << bits) <= n_rows) ++bits;
    q.id_bits = bits;  // ids 0 .. n_rows (n_rows marks dropped entries)
    if (query_sorted_smem(q) > smem_optin)
      return fail(CEOS_ERR_UNSUPPORTED, "query working set (n_cand=%d, n_neighbors=%d) exceeds shared memory", c, q.k);
    return CEOS_OK;
  }

  int finish_search(int mode, long nq, int k, int32_t* ids, float* dists, int32_t* out_ids,
                    float* out_d, bool on_device) {
    timer.mark(mode == Q_ESTIMATE ? "estimate+rerank" : "union+rerank");
    if (!on_device) {
      CUDA_TRY(cudaMemcpyAsync(ids, out_ids, (size_t)nq * k * 4, cudaMemcpyDeviceToHost, stream));
      CUDA_TRY(cudaMemcpyAsync(dists, out_d, (size_t)nq * k * 4, cudaMemcpyDeviceToHost, stream));
      timer.mark("d2h");
    }
    CUDA_TRY(cudaStreamSynchronize(stream));
    timer.finish();
    return CEOS_OK;
  }

  int search_dense(const float* Q, long nq, int k, int32_t* ids, float* dists, bool on_device) {
    ST_TRY(ensure_bf16());
    timer.begin(stream);
    ST_TRY(stage_queries(Q, nq, on_device));
    QueryArgs q = query_base(nq, k);
    int32_t* out_ids = ids;
    float* out_d = dists;
    if (!on_device) {
      CUDA_TRY(wIds.ensure((size_t)nq * k * 4));
      CUDA_TRY(wD.ensure((size_t)nq * k * 4));
      out_ids = wIds.as<int32_t>();
      out_d = wD.as<float>();
    }
    q.out_ids = out_ids;
    q.out_d = out_d;
    CUDA_TRY(wProbes.ensure((size_t)nq * std::max(s, 1) * 4));
    q.probes_out = wProbes.as<int>();
    q.probes = wProbes.as<int>();
    CUDA_TRY(launch_probe_select(q, stream));
    const size_t budget = (size_t)1 << 30;
    long chunk = std::max(1L, (long)(budget / ((size_t)n_rows * 4)));
    chunk = std::min(chunk, nq);
    CUDA_TRY(wEst.ensure((size_t)chunk * n_rows * 4));
    q.est = wEst.as<float>();
    for (long q0 = 0; q0 < nq; q0 += chunk) {
      const int nc = (int)std::min(chunk, nq - q0);
      CUDA_TRY(launch_dense_estimate(q, (int)q0, nc, stream));
      CUDA_TRY(launch_dense_select_rerank(q, (int)q0, nc, stream));
    }
    timer.mark("estimate+rerank");
    if (!on_device) {
      CUDA_TRY(cudaMemcpyAsync(ids, out_ids, (size_t)nq * k * 4, cudaMemcpyDeviceToHost, stream));
      CUDA_TRY(cudaMemcpyAsync(dists, out_d, (size_t)nq * k * 4, cudaMemcpyDeviceToHost, stream));
      timer.mark("d2h");
    }
    CUDA_TRY(cudaStreamSynchronize(stream));
    timer.finish();
    return CEOS_OK;
  }

  int query_blocks_per_sm(int mode, size_t smem, bool table_in_smem);
};

inline int Core::query_blocks_per_sm(int mode, size_t smem, bool table_in_smem) {
  return query_buckets_blocks_per_sm(mode, smem, table_in_smem);
}

inline void print_timings(const char* what, const Timer& t) {
  if (log_level() < 1) return;
  float total = 0;
  for (size_t i = 0; i < t.ms.size(); ++i) {
    std::printf("%s %s time: %.3f ms\n", what, t.names[i].c_str(), t.ms[i]);
    total += t.ms[i];
  }
  std::printf("%s total device time: %.3f ms\n", what, total);
  std::fflush(stdout);
}

}  // namespace ceos_host

// ===========================================================================
struct ceos_index {
  ceos_host::Core core;
  int n_points = 0;
};

struct ceos_stream {
  ceos_host::Core core;
};

namespace ceos_host {
// streamCEOs::update (src/streamCEOs.cpp:174-369) on a built stream index;
// defined in capi.cu, shared by ceos_stream_update and the serving loop.
int stream_update(ceos_stream* h, const float* Xn, int b, int n_del);
// Random-id deletes under exact maintenance; defined in capi.cu.
int stream_delete(ceos_stream* h, const int32_t* ids, int n_ids);
}  // namespace ceos_host
