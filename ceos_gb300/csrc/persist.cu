// Index save / load (no reference counterpart: the reference rebuilds every
// index from its rows). A versioned binary file holds the parameters, the
// rows in logical order, the sign words, and the built structures (buckets,
// or the dense CEOs-Est projections; for streams also the exact-maintenance
// counts and thresholds), followed by an FNV-1a checksum of everything
// before it. Loading restores a device-resident index that searches and
// updates exactly like the saved one, without rebuilding.
//
// Layout (little-endian):
//   "CEOSGB3\0" | u32 version | u32 kind (1 = CEOs, 2 = streamCEOs)
//   | i64 n_rows | i32 x 16 parameters | sign words | rows (n_rows x d f32)
//   | payload of the built kind | u64 checksum
#include <cstdio>
#include <memory>

#include "core.h"

using namespace ceos_host;

namespace {

constexpr char kMagic[8] = {'C', 'E', 'O', 'S', 'G', 'B', '3', '\0'};
constexpr uint32_t kVersion = 1;
constexpr size_t kChunk = (size_t)64 << 20;  // host staging per copy

struct Writer {
  FILE* f = nullptr;
  uint64_t h = 1469598103934665603ull;
  bool ok = true;
  void put(const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    if (n && std::fwrite(p, 1, n, f) != n) ok = false;
  }
  template <typename T>
  void val(T v) { put(&v, sizeof(T)); }
};

struct Reader {
  FILE* f = nullptr;
  uint64_t h = 1469598103934665603ull;
  bool ok = true;
  void get(void* p, size_t n) {
    if (n && std::fread(p, 1, n, f) != n) {
      ok = false;
      return;
    }
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
  }
  template <typename T>
  T val() {
    T v{};
    get(&v, sizeof(T));
    return v;
  }
};

struct FileCloser {
  void operator()(FILE* f) const { if (f) std::fclose(f); }
};

// device buffer -> file, through a host staging block
int put_device(Writer& w, const void* d, size_t bytes) {
  std::vector<unsigned char> buf(std::min(bytes, kChunk));
  for (size_t o = 0; o < bytes; o += kChunk) {
    const size_t n = std::min(kChunk, bytes - o);
    CUDA_TRY(cudaMemcpy(buf.data(), static_cast<const unsigned char*>(d) + o, n, cudaMemcpyDeviceToHost));
    w.put(buf.data(), n);
  }
  return CEOS_OK;
}

int get_device(Reader& r, void* d, size_t bytes) {
  std::vector<unsigned char> buf(std::min(bytes, kChunk));
  for (size_t o = 0; o < bytes; o += kChunk) {
    const size_t n = std::min(kChunk, bytes - o);
    r.get(buf.data(), n);
    if (!r.ok) return fail(CEOS_ERR_ARG, "truncated index file");
    CUDA_TRY(cudaMemcpy(static_cast<unsigned char*>(d) + o, buf.data(), n, cudaMemcpyHostToDevice));
  }
  return CEOS_OK;
}

// Rows in logical order, unpadded (n x d), from the ring (head, cap, ldx).
int put_rows(Writer& w, const Core& c) {
  const long rows_per = std::max(1L, (long)(kChunk / ((size_t)c.n_features * 4)));
  std::vector<float> buf((size_t)std::min(rows_per, std::max(c.n_rows, 1L)) * c.n_features);
  for (long r0 = 0; r0 < c.n_rows; r0 += rows_per) {
    const long nr = std::min(rows_per, c.n_rows - r0);
    long done = 0;
    while (done < nr) {  // contiguous segments of the ring
      const long phys = (c.head + r0 + done) % c.cap_rows;
      const long seg = std::min(nr - done, c.cap_rows - phys);
      CUDA_TRY(cudaMemcpy2D(buf.data() + (size_t)done * c.n_features, (size_t)c.n_features * 4,
                            c.dX.as<float>() + phys * c.ldx, (size_t)c.ldx * 4,
                            (size_t)c.n_features * 4, (size_t)seg, cudaMemcpyDeviceToHost));
      done += seg;
    }
    w.put(buf.data(), (size_t)nr * c.n_features * 4);
  }
  return CEOS_OK;
}

int get_rows(Reader& r, Core& c) {
  CUDA_TRY(c.dX.ensure((size_t)std::max(c.cap_rows, 1L) * c.ldx * 4));
  CUDA_TRY(cudaMemset(c.dX.p, 0, (size_t)std::max(c.cap_rows, 1L) * c.ldx * 4));
  const long rows_per = std::max(1L, (long)(kChunk / ((size_t)c.n_features * 4)));
  std::vector<float> buf((size_t)std::min(rows_per, std::max(c.n_rows, 1L)) * c.n_features);
  for (long r0 = 0; r0 < c.n_rows; r0 += rows_per) {
    const long nr = std::min(rows_per, c.n_rows - r0);
    r.get(buf.data(), (size_t)nr * c.n_features * 4);
    if (!r.ok) return fail(CEOS_ERR_ARG, "truncated index file");
    CUDA_TRY(cudaMemcpy2D(c.dX.as<float>() + r0 * c.ldx, (size_t)c.ldx * 4, buf.data(),
                          (size_t)c.n_features * 4, (size_t)c.n_features * 4, (size_t)nr,
                          cudaMemcpyHostToDevice));
  }
  return CEOS_OK;
}

int save_core(const Core& c, uint32_t kind, long n_points, const char* path) {
  if (!path) return fail(CEOS_ERR_ARG, "null path");
  if (c.built == B_NONE) return fail(CEOS_ERR_NOT_BUILT, "nothing to save: the index is not built");
  CUDA_TRY(cudaSetDevice(c.device));
  CUDA_TRY(cudaStreamSynchronize(c.stream));
  std::unique_ptr<FILE, FileCloser> f(std::fopen(path, "wb"));
  if (!f) return fail(CEOS_ERR_ARG, "cannot open %s for writing", path);
  Writer w;
  w.f = f.get();
  w.put(kMagic, 8);
  w.val<uint32_t>(kVersion);
  w.val<uint32_t>(kind);
  w.val<int64_t>(c.n_rows);
  const int32_t params[16] = {(int32_t)n_points, c.n_features, c.n_proj, c.n_repeats, c.top_m,
                              c.n_threads, c.seed, c.s, c.p, c.c, c.centering, c.precision,
                              c.reserve, c.built, c.proj_tensor, 0};
  w.put(params, sizeof(params));
  const int words = c.fht >= 32 ? c.fht / 32 : 1;
  ST_TRY(put_device(w, c.dSigns.p, (size_t)c.n_repeats * 3 * words * 4));
  ST_TRY(put_rows(w, c));
  const size_t ends = (size_t)c.C() * 2;
  if (c.built == B_DENSE) {
    ST_TRY(put_device(w, c.dP.p, (size_t)c.C() * c.n_rows * 4));
  } else {
    ST_TRY(put_device(w, c.dBids.p, ends * c.stride() * 4));
    ST_TRY(put_device(w, c.dBvals.p, ends * c.stride() * 4));
    if (c.built == B_STREAM && c.reserve >= 0) {
      ST_TRY(put_device(w, c.dCnt.p, ends * 4));
      ST_TRY(put_device(w, c.dTau.p, ends * 8));
    }
  }
  const uint64_t sum = w.h;
  w.put(&sum, 8);
  if (!w.ok) return fail(CEOS_ERR_ARG, "write to %s failed", path);
  return CEOS_OK;
}

int load_core(Core& c, uint32_t kind, long* n_points, const char* path) {
  if (!path) return fail(CEOS_ERR_ARG, "null path");
  std::unique_ptr<FILE, FileCloser> f(std::fopen(path, "rb"));
  if (!f) return fail(CEOS_ERR_ARG, "cannot open %s", path);
  Reader r;
  r.f = f.get();
  char magic[8];
  r.get(magic, 8);
  if (!r.ok || std::memcmp(magic, kMagic, 8) != 0) return fail(CEOS_ERR_ARG, "%s is not a CEOs GB300 index file", path);
  const uint32_t ver = r.val<uint32_t>();
  if (ver != kVersion) return fail(CEOS_ERR_ARG, "index file version %u is not supported (expected %u)", ver, kVersion);
  if (r.val<uint32_t>() != kind)
    return fail(CEOS_ERR_ARG, "%s holds a %s index", path, kind == 1 ? "streamCEOs" : "CEOs");
  const int64_t n_rows = r.val<int64_t>();
  int32_t prm[16];
  r.get(prm, sizeof(prm));
  if (!r.ok || n_rows < 1 || prm[1] < 1) return fail(CEOS_ERR_ARG, "corrupt index header");
  // The header must describe an index of this handle's kind before anything
  // is allocated: CEOs files hold a dense, coCEOs-Est or CEOs-Hash build with
  // n_points == the stored row count, streamCEOs files a stream build.
  {
    const int b = prm[13];
    const bool kind_ok = kind == 1u ? (b == B_DENSE || b == B_COCEOS || b == B_HASH) : (b == B_STREAM);
    if (!kind_ok) return fail(CEOS_ERR_ARG, "corrupt index header (build kind %d)", b);
    if (prm[14] != 0 && prm[14] != 1) return fail(CEOS_ERR_ARG, "corrupt index header (projection form %d)", prm[14]);
    if (kind == 1u && (int64_t)prm[0] != n_rows)
      return fail(CEOS_ERR_ARG, "corrupt index header (n_points %d, %lld rows)", prm[0], (long long)n_rows);
  }
  *n_points = prm[0];
  c.n_features = prm[1];
  c.set_param(prm[2], prm[3], prm[4], prm[5], prm[6]);
  c.s = prm[7];
  c.p = prm[8];
  c.c = prm[9];
  c.centering = prm[10];
  c.precision = prm[11];
  c.reserve = prm[12];
  const int built = prm[13];
  ST_TRY(c.check_param());
  ST_TRY(c.ensure_device());
  c.release_all();
  c.proj_tensor = prm[14];
  c.n_rows = n_rows;
  c.head = 0;
  c.cap_rows = n_rows;
  sign_bits(c.fht * 3 * c.n_repeats, c.seed, c.bits);  // host copy, as after a build
  const int words = c.fht >= 32 ? c.fht / 32 : 1;
  CUDA_TRY(c.dSigns.ensure((size_t)c.n_repeats * 3 * words * 4));
  ST_TRY(get_device(r, c.dSigns.p, (size_t)c.n_repeats * 3 * words * 4));
  ST_TRY(get_rows(r, c));
  const size_t ends = (size_t)c.C() * 2;
  if (built == B_DENSE) {
    CUDA_TRY(c.dP.ensure((size_t)c.C() * c.n_rows * 4));
    ST_TRY(get_device(r, c.dP.p, (size_t)c.C() * c.n_rows * 4));
  } else {
    CUDA_TRY(c.dBids.ensure(ends * c.stride() * 4));
    CUDA_TRY(c.dBvals.ensure(ends * c.stride() * 4));
    ST_TRY(get_device(r, c.dBids.p, ends * c.stride() * 4));
    ST_TRY(get_device(r, c.dBvals.p, ends * c.stride() * 4));
    if (built == B_STREAM && c.reserve >= 0) {
      CUDA_TRY(c.dCnt.ensure(ends * 4));
      CUDA_TRY(c.dTau.ensure(ends * 8));
      ST_TRY(get_device(r, c.dCnt.p, ends * 4));
      ST_TRY(get_device(r, c.dTau.p, ends * 8));
    }
  }
  const uint64_t want = r.h;
  uint64_t sum = 0;
  r.get(&sum, 8);
  if (!r.ok || sum != want) {
    c.release_all();
    return fail(CEOS_ERR_ARG, "index file %s is corrupt (checksum mismatch)", path);
  }
  c.built = built;
  return CEOS_OK;
}

}  // namespace

extern "C" {

int ceos_get_shape(const ceos_index* h, int* n_points, int* n_features) {
  if (!h || !n_points || !n_features) return fail(CEOS_ERR_ARG, "null argument");
  *n_points = h->n_points;
  *n_features = h->core.n_features;
  return CEOS_OK;
}

int ceos_get_precision(const ceos_index* h, int* precision) {
  if (!h || !precision) return fail(CEOS_ERR_ARG, "null argument");
  *precision = h->core.precision;
  return CEOS_OK;
}

int ceos_stream_get_index_param(const ceos_stream* h, int* n_proj, int* n_repeats, int* top_points,
                                int* seed, int* n_features) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  if (n_proj) *n_proj = h->core.n_proj;
  if (n_repeats) *n_repeats = h->core.n_repeats;
  if (top_points) *top_points = h->core.top_m;
  if (seed) *seed = h->core.seed;
  if (n_features) *n_features = h->core.n_features;
  return CEOS_OK;
}

int ceos_stream_get_precision(const ceos_stream* h, int* precision) {
  if (!h || !precision) return fail(CEOS_ERR_ARG, "null argument");
  *precision = h->core.precision;
  return CEOS_OK;
}

int ceos_save(const ceos_index* h, const char* path) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  return save_core(h->core, 1u, h->n_points, path);
}

int ceos_load(const char* path, ceos_index** out) {
  if (!out) return fail(CEOS_ERR_ARG, "null output handle");
  *out = nullptr;
  auto h = std::make_unique<ceos_index>();
  long n_points = 0;
  ST_TRY(load_core(h->core, 1u, &n_points, path));
  h->n_points = (int)n_points;
  *out = h.release();
  return CEOS_OK;
}

int ceos_stream_save(const ceos_stream* h, const char* path) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  return save_core(h->core, 2u, h->core.n_rows, path);
}

int ceos_stream_load(const char* path, ceos_stream** out) {
  if (!out) return fail(CEOS_ERR_ARG, "null output handle");
  *out = nullptr;
  auto h = std::make_unique<ceos_stream>();
  long n_points = 0;
  ST_TRY(load_core(h->core, 2u, &n_points, path));
  *out = h.release();
  return CEOS_OK;
}

}  // extern "C"
