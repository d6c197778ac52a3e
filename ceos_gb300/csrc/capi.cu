// Host layer and C ABI (include/ceos_gb300.h).
//
// Owns the device state of each index (rows, sign words, buckets or dense
// projections, workspaces), validates parameters with the reference's rules
// and orchestrates the kernels on one CUDA stream per index. Parameter
// semantics follow src/CEOs.h:52-81 and src/streamCEOs.h:40-70.
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

namespace {

using namespace ceos;

thread_local std::string g_err;
int g_log = -1;

int log_level() {
  if (g_log < 0) {
    const char* e = std::getenv("CEOS_GB300_LOG");
    g_log = e ? std::atoi(e) : 1;
  }
  return g_log;
}

int fail(int code, const char* fmt, ...) {
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

int np2(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

// Hash-table capacity for a query probing s columns of p entries: the
// smallest prime >= max(64, 1.2 * s * p) (prime for double hashing), or -1
// when it would not fit an int.
long table_capacity(int s, int p) {
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

int ilog2(int F) {
  int l = 0;
  while ((1 << l) < F) ++l;
  return l;
}

// fhtDim rule of src/CEOs.h:76-79 / src/streamCEOs.h:64-67.
int fht_dim(int n_proj, int n_features) {
  if (n_proj < n_features) return 1 << (int)std::ceil(std::log2((double)n_features));
  return 1 << (int)std::ceil(std::log2((double)n_proj));
}

// bitHD3Generator (src/Utilities.cpp:21-41): F*3*R bits from
// std::default_random_engine + uniform_int_distribution<uint32_t>(0, 1); a
// negative seed seeds from the wall clock.
void sign_bits(int n_bits, int random_seed, std::vector<uint8_t>& bits) {
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
  DevBuf wStage, wQ, wQproj, wIds, wD, wTable, wProbes, wEst, wNewP, wNewX;
  Timer timer;

  int C() const { return n_proj * n_repeats; }

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
                      &wD, &wTable, &wProbes, &wEst, &wNewP, &wNewX};
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
    return a;
  }

  // Two-ended top-m buckets of the n_rows rows held in dX (see select.cu).
  int build_buckets() {
    const long n = n_rows;
    const int m = top_m, Cc = C();
    if (m < 1 || m > n) return fail(CEOS_ERR_ARG, "top_m (%d) must be in [1, n_points=%ld]", m, n);
    if (m > 8192) return fail(CEOS_ERR_UNSUPPORTED, "top_m > 8192 is not supported");
    // ---- sample thresholds ----
    long S = n <= 65536 ? n : std::max(8192L, std::min(n / 8, 32L * m));
    if (S > n) S = n;
    const bool exact = (S == n);
    int rank;
    long cap;
    if (exact) {
      rank = m;
      cap = std::max(128, np2(2 * m));
    } else {
      const double mu = (double)S * m / (double)n;
      rank = (int)std::min((double)S, std::ceil(2.0 * mu + 4.0 * std::sqrt(mu) + 8.0));
      const double expected = (double)rank * (double)n / (double)S;
      cap = np2((int)std::min(1e9, std::max((double)m + 64.0, 2.0 * expected)));
      cap = std::min(cap, 16384L);
      if (cap < m + 1) cap = np2(m + 1);
    }
    DevBuf samp, rowmap, th, cnt, cand, failb;
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
    a.out = samp.as<float>();
    a.ld_out = S;
    CUDA_TRY(launch_project(a, PROJ_COLS, L, sms, stream));
    CUDA_TRY(th.ensure((size_t)Cc * 2 * 4));
    CUDA_TRY(launch_sample_thresholds(samp.as<float>(), S, Cc, rank, th.as<uint32_t>(), stream));
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
    samp.release();
    cand.release();
    // ---- exact fallback for flagged column ends ----
    std::vector<unsigned> hf((size_t)Cc * 2);
    CUDA_TRY(cudaMemcpyAsync(hf.data(), failb.p, hf.size() * 4, cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    std::vector<int> failed_cols;
    for (int col = 0; col < Cc; ++col)
      if (hf[2 * col] || hf[2 * col + 1]) failed_cols.push_back(col);
    fallback_columns = (int)failed_cols.size();
    if (!failed_cols.empty()) {
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
        CUDA_TRY(launch_exact_buckets(dump.as<float>(), n, n, cnt_cols, colofslot.as<int>(),
                                      failb.as<unsigned>(), m, dBids.as<int>(), dBvals.as<float>(),
                                      stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
      }
      timer.mark("exact-fallback");
    }
    return CEOS_OK;
  }

  int fallback_columns = 0;

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
    ProjArgs a = proj_base();
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
    q.m = top_m;
    q.c = c;
    q.k = k;
    q.X = dX.as<float>();
    q.head = head;
    q.cap_rows = cap_rows;
    q.n_points = n_rows;
    q.bids = dBids.as<int>();
    q.bvals = dBvals.as<float>();
    q.P = dP.as<float>();
    q.distinct_ids = built == B_STREAM ? 0 : 1;
    if (precision == CEOS_PRECISION_SPLIT_BF16) {
      q.Xb = dXb.as<uint16_t>();
      q.rescore = 4 * k;
    }
    return q;
  }

  // coCEOs-Est / CEOs-Hash / stream searches over the buckets.
  int search_buckets(int mode, const float* Q, long nq, int k, int32_t* ids, float* dists,
                     bool on_device, cudaStream_t user_stream) {
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
    timer.mark(mode == Q_ESTIMATE ? "estimate+rerank" : "union+rerank");
    if (!on_device) {
      CUDA_TRY(cudaMemcpyAsync(ids, out_ids, (size_t)nq * k * 4, cudaMemcpyDeviceToHost, stream));
      CUDA_TRY(cudaMemcpyAsync(dists, out_d, (size_t)nq * k * 4, cudaMemcpyDeviceToHost, stream));
      timer.mark("d2h");
    }
    CUDA_TRY(cudaStreamSynchronize(stream));
    timer.finish();
    (void)user_stream;
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

int Core::query_blocks_per_sm(int mode, size_t smem, bool table_in_smem) {
  return query_buckets_blocks_per_sm(mode, smem, table_in_smem);
}

void print_timings(const char* what, const Timer& t) {
  if (log_level() < 1) return;
  float total = 0;
  for (size_t i = 0; i < t.ms.size(); ++i) {
    std::printf("%s %s time: %.3f ms\n", what, t.names[i].c_str(), t.ms[i]);
    total += t.ms[i];
  }
  std::printf("%s total device time: %.3f ms\n", what, total);
  std::fflush(stdout);
}

}  // namespace

// ===========================================================================
struct ceos_index {
  Core core;
  int n_points = 0;
};

struct ceos_stream {
  Core core;
};

extern "C" {

int ceos_abi_version(void) { return CEOS_ABI_VERSION; }
const char* ceos_last_error(void) { return g_err.c_str(); }
int ceos_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}
void ceos_set_log_level(int level) { g_log = level < 0 ? 0 : level; }

int ceos_flush_l2(long bytes) {
  static DevBuf* flush = nullptr;
  if (bytes <= 0) return fail(CEOS_ERR_ARG, "bytes must be > 0");
  if (!flush) flush = new DevBuf();
  CUDA_TRY(flush->ensure((size_t)bytes));
  CUDA_TRY(cudaMemsetAsync(flush->p, 0x5a, (size_t)bytes, 0));
  CUDA_TRY(cudaDeviceSynchronize());
  return CEOS_OK;
}

// ---------------------------------------------------------------------------
int ceos_create(int n_points, int n_features, ceos_index** out) {
  if (!out) return fail(CEOS_ERR_ARG, "null output handle");
  *out = nullptr;
  if (n_points < 1 || n_features < 1)
    return fail(CEOS_ERR_ARG, "n_points (%d) and n_features (%d) must be >= 1", n_points, n_features);
  ceos_index* h = new ceos_index();
  h->n_points = n_points;
  h->core.n_features = n_features;
  h->core.set_param(256, 1, 100, -1, -1);  // class defaults, src/CEOs.h:24-29
  *out = h;
  return CEOS_OK;
}

void ceos_destroy(ceos_index* h) { delete h; }

int ceos_set_index_param(ceos_index* h, int n_proj, int n_repeats, int top_m, int n_threads,
                         int random_seed) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (n_proj < 1 || n_repeats < 1) return fail(CEOS_ERR_ARG, "n_proj and n_repeats must be >= 1");
  h->core.set_param(n_proj, n_repeats, top_m, n_threads, random_seed);
  h->core.p = top_m;  // n_probed_points = top_m (src/CEOs.h:69)
  return CEOS_OK;
}

int ceos_get_index_param(const ceos_index* h, int* n_proj, int* n_repeats, int* top_m,
                         int* n_threads, int* random_seed, int* fht_dim_out) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  const Core& c = h->core;
  if (n_proj) *n_proj = c.n_proj;
  if (n_repeats) *n_repeats = c.n_repeats;
  if (top_m) *top_m = c.top_m;
  if (n_threads) *n_threads = c.n_threads;
  if (random_seed) *random_seed = c.seed;
  if (fht_dim_out) *fht_dim_out = c.fht;
  return CEOS_OK;
}

int ceos_set_threads(ceos_index* h, int n_threads) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  h->core.n_threads = n_threads;
  return CEOS_OK;
}

int ceos_clear(ceos_index* h) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.device >= 0) cudaSetDevice(h->core.device);
  h->core.release_all();
  return CEOS_OK;
}

int ceos_set_query_param(ceos_index* h, int s, int p, int c) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  h->core.s = s;
  h->core.p = p;
  h->core.c = c;
  return CEOS_OK;
}

int ceos_get_query_param(const ceos_index* h, int* s, int* p, int* c) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (s) *s = h->core.s;
  if (p) *p = h->core.p;
  if (c) *c = h->core.c;
  return CEOS_OK;
}

int ceos_set_centering(ceos_index* h, int centering) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  h->core.centering = centering ? 1 : 0;
  return CEOS_OK;
}

int ceos_get_centering(const ceos_index* h, int* centering) {
  if (!h || !centering) return fail(CEOS_ERR_ARG, "null argument");
  *centering = h->core.centering;
  return CEOS_OK;
}

int ceos_set_precision(ceos_index* h, int precision) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (precision != CEOS_PRECISION_FP32 && precision != CEOS_PRECISION_SPLIT_BF16)
    return fail(CEOS_ERR_ARG, "unknown precision %d", precision);
  h->core.precision = precision;
  return CEOS_OK;
}

static int index_build_common(ceos_index* h, const float* X, const char* what) {
  if (!h || !X) return fail(CEOS_ERR_ARG, "null argument");
  Core& c = h->core;
  ST_TRY(c.check_param());
  ST_TRY(c.ensure_device());
  c.release_all();
  c.timer.begin(c.stream);
  c.n_rows = h->n_points;
  c.head = 0;
  c.cap_rows = h->n_points;
  CUDA_TRY(c.dX.ensure((size_t)c.n_rows * c.ldx * 4));
  ST_TRY(c.upload_rows(X, c.n_rows, c.dX.as<float>()));
  ST_TRY(c.upload_signs());
  c.timer.mark("h2d");
  if (log_level() >= 1) {
    std::printf("%s\nn_points: %ld\nn_features: %d\nn_repeats: %d\nn_proj: %d\ntop_m: %d\nfhtDim: %d\n",
                what, c.n_rows, c.n_features, c.n_repeats, c.n_proj, c.top_m, c.fht);
  }
  return CEOS_OK;
}

int ceos_build(ceos_index* h, const float* X) {
  ST_TRY(index_build_common(h, X, "Building CEOs index..."));
  Core& c = h->core;
  const int Cc = c.C();
  CUDA_TRY(c.dP.ensure((size_t)Cc * c.n_rows * 4));
  ProjArgs a = c.proj_base();
  a.n_rows = c.n_rows;
  a.out = c.dP.as<float>();
  a.ld_out = c.n_rows;
  CUDA_TRY(launch_project(a, PROJ_COLS, c.L, c.sms, c.stream));
  c.timer.mark("project");
  CUDA_TRY(cudaStreamSynchronize(c.stream));
  c.timer.finish();
  c.built = B_DENSE;
  print_timings("CEOs build", c.timer);
  return CEOS_OK;
}

static int build_buckets_api(ceos_index* h, const float* X, int kind, const char* what) {
  ST_TRY(index_build_common(h, X, what));
  Core& c = h->core;
  const int st = c.build_buckets();
  if (st != CEOS_OK) {
    c.timer.clear();
    c.release_all();
    return st;
  }
  CUDA_TRY(cudaStreamSynchronize(c.stream));
  c.timer.finish();
  c.built = kind;
  print_timings(kind == B_COCEOS ? "coCEOs-Est build" : "CEOs-Hash build", c.timer);
  return CEOS_OK;
}

int ceos_build_coceos_est(ceos_index* h, const float* X) {
  return build_buckets_api(h, X, B_COCEOS, "Building coCEOs-Estimate index...");
}

int ceos_build_ceos_hash(ceos_index* h, const float* X) {
  return build_buckets_api(h, X, B_HASH, "Building CEOs-Hash index...");
}

// Reference validation order: n_probed_points first, then n_probed_vectors
// (src/CEOs.cpp:452-461).
static int check_query(const Core& c, int built_kind, int algo_needs_points, long nq, int k,
                       int s_limit) {
  if (c.built != built_kind) return fail(CEOS_ERR_NOT_BUILT, "index is not built for this search");
  if (nq < 0 || k < 0) return fail(CEOS_ERR_ARG, "n_queries and n_neighbors must be >= 0");
  if (algo_needs_points && (c.p > c.top_m))
    return fail(CEOS_ERR_PROBED_POINTS,
                "Number of probed points must be smaller than number of indexed top-m points");
  if (c.p < 0 && algo_needs_points) return fail(CEOS_ERR_ARG, "n_probed_points must be >= 0");
  if (c.s > s_limit)
    return fail(CEOS_ERR_PROBED_VECTORS,
                "Number of probed vectors must be smaller than n_proj * n_repeats");
  if (c.s < 0 || c.c < 0) return fail(CEOS_ERR_ARG, "n_probed_vectors and n_cand must be >= 0");
  if (k > 8192 || c.c > 65536)
    return fail(CEOS_ERR_UNSUPPORTED, "n_neighbors > 8192 or n_cand > 65536 is not supported");
  return CEOS_OK;
}


int ceos_search(ceos_index* h, const float* Q, int nq, int k, int verbose, int32_t* ids,
                float* dists) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  Core& c = h->core;
  ST_TRY(check_query(c, B_DENSE, 0, nq, k, c.C()));
  if (nq == 0 || k == 0) return CEOS_OK;
  if (!Q || !ids || !dists) return fail(CEOS_ERR_ARG, "null buffer");
  ST_TRY(c.ensure_device());
  ST_TRY(c.search_dense(Q, nq, k, ids, dists, false));
  if (verbose) print_timings("CEOs search", c.timer);
  return CEOS_OK;
}

int ceos_search_coceos_est(ceos_index* h, const float* Q, int nq, int k, int verbose,
                           int32_t* ids, float* dists) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  Core& c = h->core;
  ST_TRY(check_query(c, B_COCEOS, 1, nq, k, c.C()));
  if (nq == 0 || k == 0) return CEOS_OK;
  if (!Q || !ids || !dists) return fail(CEOS_ERR_ARG, "null buffer");
  ST_TRY(c.ensure_device());
  ST_TRY(c.search_buckets(Q_ESTIMATE, Q, nq, k, ids, dists, false, nullptr));
  if (verbose) print_timings("coCEOs-Est search", c.timer);
  return CEOS_OK;
}

int ceos_search_ceos_hash(ceos_index* h, const float* Q, int nq, int k, int verbose,
                          int32_t* ids, float* dists) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  Core& c = h->core;
  ST_TRY(check_query(c, B_HASH, 1, nq, k, c.C()));
  if (nq == 0 || k == 0) return CEOS_OK;
  if (!Q || !ids || !dists) return fail(CEOS_ERR_ARG, "null buffer");
  ST_TRY(c.ensure_device());
  ST_TRY(c.search_buckets(Q_UNION, Q, nq, k, ids, dists, false, nullptr));
  if (verbose) print_timings("CEOs-Hash search", c.timer);
  return CEOS_OK;
}

int ceos_search_device(ceos_index* h, int algo, const float* dQ, int nq, int k, int32_t* d_ids,
                       float* d_dists, void* cuda_stream) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  Core& c = h->core;
  const int kind = algo == CEOS_ALGO_DENSE ? B_DENSE : algo == CEOS_ALGO_COCEOS ? B_COCEOS
                   : algo == CEOS_ALGO_HASH ? B_HASH : -1;
  if (kind < 0) return fail(CEOS_ERR_ARG, "unknown algorithm %d", algo);
  ST_TRY(check_query(c, kind, kind != B_DENSE, nq, k, c.C()));
  if (nq == 0 || k == 0) return CEOS_OK;
  if (!dQ || !d_ids || !d_dists) return fail(CEOS_ERR_ARG, "null buffer");
  ST_TRY(c.ensure_device());
  cudaStream_t user = reinterpret_cast<cudaStream_t>(cuda_stream);
  if (user) {
    // order the index stream after the caller's prior work
    cudaEvent_t ev;
    CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CUDA_TRY(cudaEventRecord(ev, user));
    CUDA_TRY(cudaStreamWaitEvent(c.stream, ev, 0));
    cudaEventDestroy(ev);
  }
  if (kind == B_DENSE) {
    ST_TRY(c.search_dense(dQ, nq, k, d_ids, d_dists, true));
  } else {
    ST_TRY(c.search_buckets(kind == B_COCEOS ? Q_ESTIMATE : Q_UNION, dQ, nq, k, d_ids, d_dists,
                            true, user));
  }
  return CEOS_OK;
}

int ceos_get_buckets(const ceos_index* h, int32_t* ids, float* vals) {
  if (!h || !ids || !vals) return fail(CEOS_ERR_ARG, "null argument");
  const Core& c = h->core;
  if (c.built != B_COCEOS && c.built != B_HASH) return fail(CEOS_ERR_NOT_BUILT, "no buckets built");
  const size_t cnt = (size_t)c.C() * 2 * c.top_m;
  CUDA_TRY(cudaSetDevice(c.device));
  CUDA_TRY(cudaMemcpy(ids, c.dBids.p, cnt * 4, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(vals, c.dBvals.p, cnt * 4, cudaMemcpyDeviceToHost));
  if (c.built == B_HASH) std::memset(vals, 0, cnt * 4);
  return CEOS_OK;
}

int ceos_get_projections(const ceos_index* h, float* P) {
  if (!h || !P) return fail(CEOS_ERR_ARG, "null argument");
  const Core& c = h->core;
  if (c.built != B_DENSE) return fail(CEOS_ERR_NOT_BUILT, "dense index not built");
  const int Cc = c.C();
  std::vector<float> colmajor((size_t)Cc * c.n_rows);
  CUDA_TRY(cudaSetDevice(c.device));
  CUDA_TRY(cudaMemcpy(colmajor.data(), c.dP.p, colmajor.size() * 4, cudaMemcpyDeviceToHost));
  for (long i = 0; i < c.n_rows; ++i)
    for (int col = 0; col < Cc; ++col) P[i * Cc + col] = colmajor[(size_t)col * c.n_rows + i];
  return CEOS_OK;
}

int ceos_get_sign_bits(const ceos_index* h, uint8_t* bits) {
  if (!h || !bits) return fail(CEOS_ERR_ARG, "null argument");
  if (h->core.bits.empty()) return fail(CEOS_ERR_NOT_BUILT, "signs are generated at build");
  std::memcpy(bits, h->core.bits.data(), h->core.bits.size());
  return CEOS_OK;
}

int ceos_last_timings(const ceos_index* h, float* ms, int max_phases) {
  if (!h) return 0;
  const Timer& t = h->core.timer;
  int n = std::min((int)t.ms.size(), max_phases);
  for (int i = 0; i < n; ++i) ms[i] = t.ms[i];
  return n;
}

const char* ceos_timing_name(const ceos_index* h, int phase) {
  if (!h || phase < 0 || phase >= (int)h->core.timer.names.size()) return "";
  return h->core.timer.names[phase].c_str();
}

// ---------------------------------------------------------------------------
// streamCEOs

int ceos_stream_create(int n_features, ceos_stream** out) {
  if (!out) return fail(CEOS_ERR_ARG, "null output handle");
  *out = nullptr;
  if (n_features < 1) return fail(CEOS_ERR_ARG, "n_features must be >= 1");
  ceos_stream* h = new ceos_stream();
  h->core.n_features = n_features;
  h->core.set_param(256, 1, 100, -1, -1);  // class defaults, src/streamCEOs.h:19-24
  *out = h;
  return CEOS_OK;
}

void ceos_stream_destroy(ceos_stream* h) { delete h; }

int ceos_stream_set_index_param(ceos_stream* h, int n_proj, int n_repeats, int top_points,
                                int n_threads, int random_seed) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (n_proj < 1 || n_repeats < 1) return fail(CEOS_ERR_ARG, "n_proj and n_repeats must be >= 1");
  h->core.set_param(n_proj, n_repeats, top_points, n_threads, random_seed);
  h->core.s = top_points;  // n_probed_vectors = top_m (src/streamCEOs.h:58)
  return CEOS_OK;
}

int ceos_stream_set_precision(ceos_stream* h, int precision) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (precision != CEOS_PRECISION_FP32 && precision != CEOS_PRECISION_SPLIT_BF16)
    return fail(CEOS_ERR_ARG, "unknown precision %d", precision);
  h->core.precision = precision;
  return CEOS_OK;
}

int ceos_stream_set_threads(ceos_stream* h, int n_threads) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  h->core.n_threads = n_threads;
  return CEOS_OK;
}

int ceos_stream_clear(ceos_stream* h) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (h->core.device >= 0) cudaSetDevice(h->core.device);
  h->core.release_all();
  return CEOS_OK;
}

int ceos_stream_set_query_param(ceos_stream* h, int s, int p, int c) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  h->core.s = s;
  h->core.p = p;
  h->core.c = c;
  return CEOS_OK;
}

int ceos_stream_get_query_param(const ceos_stream* h, int* s, int* p, int* c) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (s) *s = h->core.s;
  if (p) *p = h->core.p;
  if (c) *c = h->core.c;
  return CEOS_OK;
}

int ceos_stream_build(ceos_stream* h, const float* X, int n_points) {
  if (!h || !X) return fail(CEOS_ERR_ARG, "null argument");
  if (n_points < 1) return fail(CEOS_ERR_ARG, "n_points must be >= 1");
  Core& c = h->core;
  ST_TRY(c.check_param());
  ST_TRY(c.ensure_device());
  c.release_all();
  c.timer.begin(c.stream);
  c.n_rows = n_points;
  c.head = 0;
  c.cap_rows = n_points;
  CUDA_TRY(c.dX.ensure((size_t)c.cap_rows * c.ldx * 4));
  ST_TRY(c.upload_rows(X, c.n_rows, c.dX.as<float>()));
  ST_TRY(c.upload_signs());
  c.timer.mark("h2d");
  if (log_level() >= 1)
    std::printf("n_features: %d\nn_proj: %d\ntop_m: %d\nfhtDim: %d\nn_points: %ld\n", c.n_features,
                c.n_proj, c.top_m, c.fht, c.n_rows);
  const int st = c.build_buckets();
  if (st != CEOS_OK) {
    c.timer.clear();
    c.release_all();
    return st;
  }
  CUDA_TRY(cudaStreamSynchronize(c.stream));
  c.timer.finish();
  c.built = B_STREAM;
  print_timings("streamCEOs build", c.timer);
  return CEOS_OK;
}

int ceos_stream_update(ceos_stream* h, const float* Xn, int b, int n_del) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  Core& c = h->core;
  if (c.built != B_STREAM) return fail(CEOS_ERR_NOT_BUILT, "streamCEOs is not built");
  if (b < 0 || n_del < 0) return fail(CEOS_ERR_ARG, "n_new and n_delPoints must be >= 0");
  if (b > 0 && !Xn) return fail(CEOS_ERR_ARG, "null new rows");
  const long cur = c.n_rows;
  if (n_del > cur)
    return fail(CEOS_ERR_UPDATE_DEL,
                "Number of removed points must be smaller than the current number of points");
  if ((long)c.top_m > cur + b - n_del)
    return fail(CEOS_ERR_UPDATE_TOPM, "There is not enough indexed top-points for coCEOs after update");
  ST_TRY(c.ensure_device());
  c.timer.begin(c.stream);
  const int Cc = c.C();
  // new rows, padded, and their projections [C][b]
  CUDA_TRY(c.wNewX.ensure((size_t)std::max(b, 1) * c.ldx * 4));
  ST_TRY(c.upload_rows(Xn, b, c.wNewX.as<float>()));
  c.timer.mark("h2d");
  if (b > 0) {
    CUDA_TRY(c.wNewP.ensure((size_t)Cc * b * 4));
    ProjArgs a = c.proj_base();
    a.X = c.wNewX.as<float>();
    a.head = 0;
    a.cap_rows = LONG_MAX;
    a.n_rows = b;
    a.out = c.wNewP.as<float>();
    a.ld_out = b;
    CUDA_TRY(launch_project(a, PROJ_COLS, c.L, c.sms, c.stream));
  }
  c.timer.mark("project");
  CUDA_TRY(launch_stream_merge(Cc, c.top_m, c.wNewP.as<float>(), b, cur, n_del, c.dBids.as<int>(),
                               c.dBvals.as<float>(), c.stream));
  c.timer.mark("merge");
  // append the rows to the ring, growing it when full
  if (cur + b > c.cap_rows) {
    const long ncap = std::max(2 * c.cap_rows, cur + b);
    DevBuf nx;
    CUDA_TRY(nx.ensure((size_t)ncap * c.ldx * 4));
    const size_t rowb = (size_t)c.ldx * 4;
    const long first = std::min(cur, c.cap_rows - c.head);
    CUDA_TRY(cudaMemcpyAsync(nx.p, c.dX.as<float>() + c.head * c.ldx, first * rowb,
                             cudaMemcpyDeviceToDevice, c.stream));
    if (cur > first)
      CUDA_TRY(cudaMemcpyAsync(nx.as<float>() + first * c.ldx, c.dX.p, (cur - first) * rowb,
                               cudaMemcpyDeviceToDevice, c.stream));
    CUDA_TRY(cudaStreamSynchronize(c.stream));
    c.dX.swap(nx);
    nx.release();
    c.cap_rows = ncap;
    c.head = 0;
    c.dXb.release();
    c.xb_valid = false;
  }
  if (b > 0) {
    const size_t rowb = (size_t)c.ldx * 4;
    long pos = (c.head + cur) % c.cap_rows;
    const long first = std::min((long)b, c.cap_rows - pos);
    CUDA_TRY(cudaMemcpyAsync(c.dX.as<float>() + pos * c.ldx, c.wNewX.p, first * rowb,
                             cudaMemcpyDeviceToDevice, c.stream));
    if (b > first)
      CUDA_TRY(cudaMemcpyAsync(c.dX.p, c.wNewX.as<float>() + first * c.ldx, (b - first) * rowb,
                               cudaMemcpyDeviceToDevice, c.stream));
    if (c.xb_valid) {  // keep the bfloat16 copy of the ring current
      CUDA_TRY(launch_to_bf16(c.dX.as<float>() + pos * c.ldx, first * (long)c.ldx,
                              c.dXb.as<uint16_t>() + pos * c.ldx, c.stream));
      if (b > first)
        CUDA_TRY(launch_to_bf16(c.dX.as<float>(), (b - first) * (long)c.ldx, c.dXb.as<uint16_t>(),
                                c.stream));
    }
  }
  c.head = (c.head + n_del) % c.cap_rows;
  c.n_rows = cur + b - n_del;
  c.timer.mark("append");
  CUDA_TRY(cudaStreamSynchronize(c.stream));
  c.timer.finish();
  if (log_level() >= 1) {
    std::printf("n_points (after update): %ld\n", c.n_rows);
    print_timings("streamCEOs update", c.timer);
  }
  return CEOS_OK;
}

static int stream_search(ceos_stream* h, int mode, const float* Q, int nq, int k, int verbose,
                         int32_t* ids, float* dists) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  Core& c = h->core;
  // streamCEOs limits n_probed_vectors by n_proj (src/streamCEOs.cpp:386-390)
  ST_TRY(check_query(c, B_STREAM, 1, nq, k, c.n_proj));
  if (nq == 0 || k == 0) return CEOS_OK;
  if (!Q || !ids || !dists) return fail(CEOS_ERR_ARG, "null buffer");
  ST_TRY(c.ensure_device());
  ST_TRY(c.search_buckets(mode, Q, nq, k, ids, dists, false, nullptr));
  if (verbose) print_timings(mode == Q_ESTIMATE ? "streamCEOs-est search" : "streamCEOs-hash search", c.timer);
  return CEOS_OK;
}

int ceos_stream_estimate_search(ceos_stream* h, const float* Q, int nq, int k, int verbose,
                                int32_t* ids, float* dists) {
  return stream_search(h, Q_ESTIMATE, Q, nq, k, verbose, ids, dists);
}

int ceos_stream_hash_search(ceos_stream* h, const float* Q, int nq, int k, int verbose,
                            int32_t* ids, float* dists) {
  return stream_search(h, Q_UNION, Q, nq, k, verbose, ids, dists);
}

int ceos_stream_size(const ceos_stream* h, int* n_points) {
  if (!h || !n_points) return fail(CEOS_ERR_ARG, "null argument");
  *n_points = (int)h->core.n_rows;
  return CEOS_OK;
}

int ceos_stream_get_buckets(const ceos_stream* h, int32_t* ids, float* vals) {
  if (!h || !ids || !vals) return fail(CEOS_ERR_ARG, "null argument");
  const Core& c = h->core;
  if (c.built != B_STREAM) return fail(CEOS_ERR_NOT_BUILT, "streamCEOs is not built");
  const size_t cnt = (size_t)c.C() * 2 * c.top_m;
  CUDA_TRY(cudaSetDevice(c.device));
  CUDA_TRY(cudaMemcpy(ids, c.dBids.p, cnt * 4, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(vals, c.dBvals.p, cnt * 4, cudaMemcpyDeviceToHost));
  return CEOS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free search.
//
// Some callers cannot let this library call cudaMalloc: a host process that
// owns every byte of device memory through its own arena (a database or
// search-engine plugin host), or a latency-critical serving loop in which an
// allocation could stall the device or fail in the middle of a request. For
// them, ceos_search_coceos_est_device_noalloc takes its scratch (the padded
// queries, their projections and, when a query's hash table does not fit in
// shared memory, the per-CTA tables) from the fixed array below instead of
// allocating. The array is a file-scope __device__ object, so every GPU that
// loads this library holds it until the process exits.
constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;  // 64 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[128] = {};

// Device address of g_noalloc_scratch on `dev` (which must be current). In
// host code the symbol itself is only a host-side stand-in, so the address is
// looked up once per device with cudaGetSymbolAddress and cached.
int noalloc_scratch(int dev, void** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (dev < 0 || dev >= 128) return fail(CEOS_ERR_ARG, "device ordinal %d out of range", dev);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(CEOS_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return CEOS_OK;
}

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }
}  // namespace

extern "C" int ceos_search_coceos_est_device_noalloc(ceos_index* h, const float* d_Q, int nq,
                                                     int k, int32_t* d_ids, float* d_dists,
                                                     void* cuda_stream) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  Core& c = h->core;
  ST_TRY(check_query(c, B_COCEOS, 1, nq, k, c.C()));
  if (nq == 0 || k == 0) return CEOS_OK;
  if (!d_Q || !d_ids || !d_dists) return fail(CEOS_ERR_ARG, "null buffer");
  CUDA_TRY(cudaSetDevice(c.device));
  cudaStream_t st = cuda_stream ? reinterpret_cast<cudaStream_t>(cuda_stream) : c.stream;
  // Scratch layout: padded queries | query projections | per-CTA hash tables.
  QueryArgs q;
  q.nq = nq;
  q.d = c.n_features;
  q.ldx = c.ldx;
  q.C = c.C();
  q.s = c.s;
  q.p = c.p;
  q.m = c.top_m;
  q.c = c.c;
  q.k = k;
  q.X = c.dX.as<float>();
  q.head = c.head;
  q.cap_rows = c.cap_rows;
  q.n_points = c.n_rows;
  q.bids = c.dBids.as<int>();
  q.bvals = c.dBvals.as<float>();
  q.distinct_ids = 1;
  q.out_ids = d_ids;
  q.out_d = d_dists;
  const long tc = table_capacity(c.s, c.p);
  if (tc < 0) return fail(CEOS_ERR_UNSUPPORTED, "n_probed_vectors * n_probed_points too large");
  q.table_cap = (int)tc;
  q.table_in_smem = 1;
  size_t smem = query_buckets_smem(q, Q_ESTIMATE);
  int per_sm;
  if (smem > c.smem_optin) {
    q.table_in_smem = 0;
    smem = query_buckets_smem(q, Q_ESTIMATE);
    if (smem > c.smem_optin)
      return fail(CEOS_ERR_UNSUPPORTED, "query working set exceeds shared memory");
  }
  per_sm = c.query_blocks_per_sm(Q_ESTIMATE, smem, q.table_in_smem != 0);
  const int grid = (int)std::max<long>(1, std::min<long>(nq, (long)c.sms * std::max(per_sm, 1)));
  const size_t qbytes = al256((size_t)nq * c.ldx * 4);
  const size_t pbytes = al256((size_t)nq * c.C() * 4);
  const size_t tbytes = q.table_in_smem ? 0 : (size_t)grid * tc * 8;
  const size_t need = qbytes + pbytes + tbytes;
  if (need > kNoAllocScratchBytes)
    return fail(CEOS_ERR_UNSUPPORTED,
                "this batch needs %zu bytes of scratch; the allocation-free search is limited to %zu "
                "bytes (n_queries * (n_features + n_proj * n_repeats) * 4 plus hash tables): split "
                "the batch",
                need, kNoAllocScratchBytes);
  void* base = nullptr;
  ST_TRY(noalloc_scratch(c.device, &base));
  unsigned char* sc = static_cast<unsigned char*>(base);
  float* qpad = reinterpret_cast<float*>(sc);
  float* qproj = reinterpret_cast<float*>(sc + qbytes);
  q.gtable = q.table_in_smem ? nullptr : reinterpret_cast<uint64_t*>(sc + qbytes + pbytes);
  q.Q = qpad;
  q.qproj = qproj;
  // Every buffer above is fully written before it is read (the hash tables
  // are reset per query inside the kernel), so no clearing is needed.
  CUDA_TRY(launch_pad_rows(d_Q, nq, c.n_features, qpad, c.ldx, st));
  ProjArgs a = c.proj_base();
  a.X = qpad;
  a.head = 0;
  a.cap_rows = LONG_MAX;
  a.n_rows = nq;
  a.out = qproj;
  CUDA_TRY(launch_project(a, PROJ_ROWS, c.L, c.sms, st));
  CUDA_TRY(launch_query_buckets(q, Q_ESTIMATE, grid, smem, st));
  return CEOS_OK;
}
