// C entry points over the reference's own CEOs and streamCEOs classes
// (src/CEOs.h:18-114, src/streamCEOs.h:12-107), compiled unchanged from the
// reference sources against the Eigen / boost::dynamic_bitset stand-ins in
// oracle/refshim. Test infrastructure: it pins the oracle restatement
// (oracle/ceos_oracle.cpp) to the reference and generates golden fixtures;
// nothing in the product loads it.
#include <cstdint>
#include <cstring>
#include <iostream>
#include <tuple>

#include "CEOs.h"
#include "streamCEOs.h"

namespace {

// Subclasses that expose the protected bucket matrices for comparison.
struct RefCEOs : CEOs {
  RefCEOs(int n, int d) : CEOs(n, d) {}
  const MatrixXf& P() const { return matrix_P; }
  const MatrixXi& H() const { return matrix_H; }
};
struct RefStream : streamCEOs {
  explicit RefStream(int d) : streamCEOs(d) {}
  const MatrixXf& P() const { return matrix_P; }
  int size() const { return (int)deque_X.size(); }
};

// The reference reports progress and timings on std::cout; silence it.
struct Quiet {
  std::streambuf* old;
  Quiet() : old(std::cout.rdbuf(nullptr)) {}
  ~Quiet() {
    std::cout.rdbuf(old);
    std::cout.clear();
  }
};

Ref<const RowMajorMatrixXf> rows(const float* X, int n, int d) {
  return Ref<const RowMajorMatrixXf>(View<const float>(X, n, d, d, 1));
}

void copy_out(const std::tuple<RowMajorMatrixXi, RowMajorMatrixXf>& r, int32_t* ids, float* dists) {
  const RowMajorMatrixXi& I = std::get<0>(r);
  const RowMajorMatrixXf& D = std::get<1>(r);
  std::memcpy(ids, I.data(), sizeof(int32_t) * (size_t)I.size());
  std::memcpy(dists, D.data(), sizeof(float) * (size_t)D.size());
}

}  // namespace

extern "C" {

void* ref_ceos_new(int n, int d) { return new RefCEOs(n, d); }
void ref_ceos_free(void* h) { delete static_cast<RefCEOs*>(h); }
void ref_ceos_set_param(void* h, int D, int R, int m, int threads, int seed) {
  static_cast<RefCEOs*>(h)->set_CEOsParam(D, R, m, threads, seed);
}
void ref_ceos_set_query(void* h, int s, int p, int c) {
  RefCEOs* x = static_cast<RefCEOs*>(h);
  x->n_probed_vectors = s;
  x->n_probed_points = p;
  x->n_cand = c;
}
// kind: 0 = CEOs-Est (build_CEOs / search_CEOs), 1 = coCEOs-Est, 2 = CEOs-Hash
void ref_ceos_build(void* h, int kind, const float* X, int n, int d) {
  Quiet q;
  RefCEOs* x = static_cast<RefCEOs*>(h);
  if (kind == 0) x->build_CEOs(rows(X, n, d));
  else if (kind == 1) x->build_coCEOs_Est(rows(X, n, d));
  else x->build_CEOs_Hash(rows(X, n, d));
}
void ref_ceos_search(void* h, int kind, const float* Q, int nq, int d, int k, int32_t* ids, float* dists) {
  Quiet q;
  RefCEOs* x = static_cast<RefCEOs*>(h);
  if (kind == 0) copy_out(x->search_CEOs(rows(Q, nq, d), k), ids, dists);
  else if (kind == 1) copy_out(x->search_coCEOs_Est(rows(Q, nq, d), k), ids, dists);
  else copy_out(x->search_CEOs_Hash(rows(Q, nq, d), k), ids, dists);
}
// matrix_P (coCEOs: 4m x C, ids stored as float) or matrix_H (CEOs-Hash: 2m x C),
// column-major as the reference holds them; returns the number of rows.
int ref_ceos_buckets(void* h, int kind, float* out) {
  RefCEOs* x = static_cast<RefCEOs*>(h);
  if (kind == 1) {
    std::memcpy(out, x->P().data(), sizeof(float) * (size_t)x->P().size());
    return (int)x->P().rows();
  }
  const MatrixXi& H = x->H();
  for (Index i = 0; i < H.size(); ++i) out[i] = (float)H.data()[i];
  return (int)H.rows();
}

void* ref_stream_new(int d) { return new RefStream(d); }
void ref_stream_free(void* h) { delete static_cast<RefStream*>(h); }
void ref_stream_set_param(void* h, int D, int R, int m, int threads, int seed) {
  static_cast<RefStream*>(h)->set_streamCEOsParam(D, R, m, threads, seed);
}
void ref_stream_set_query(void* h, int s, int p, int c) {
  RefStream* x = static_cast<RefStream*>(h);
  x->n_probed_vectors = s;
  x->n_probed_points = p;
  x->n_cand = c;
}
void ref_stream_build(void* h, const float* X, int n, int d) {
  Quiet q;
  static_cast<RefStream*>(h)->build(rows(X, n, d));
}
void ref_stream_update(void* h, const float* X, int n, int d, int n_del) {
  Quiet q;
  static_cast<RefStream*>(h)->update(rows(X, n, d), n_del);
}
int ref_stream_size(void* h) { return static_cast<RefStream*>(h)->size(); }
// kind: 1 = estimate_search, 2 = hash_search
void ref_stream_search(void* h, int kind, const float* Q, int nq, int d, int k, int32_t* ids, float* dists) {
  Quiet q;
  RefStream* x = static_cast<RefStream*>(h);
  if (kind == 1) copy_out(x->estimate_search(rows(Q, nq, d), k), ids, dists);
  else copy_out(x->hash_search(rows(Q, nq, d), k), ids, dists);
}
int ref_stream_buckets(void* h, float* out) {
  RefStream* x = static_cast<RefStream*>(h);
  std::memcpy(out, x->P().data(), sizeof(float) * (size_t)x->P().size());
  return (int)x->P().rows();
}

}  // extern "C"
