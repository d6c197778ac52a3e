// pybind11 module `CEOs`: the drop-in for the reference's Python module
// (python/python_wrapper.cpp:13-74), backed by the GB300 library through the
// C ABI of include/ceos_gb300.h.
//
// Same module name, class names, constructor arguments, setIndexParam
// keywords and defaults, read/write attributes and methods as the reference's
// binding, so `import CEOs` scripts run unchanged. Inputs are n x d float32
// arrays; pybind11 converts other dtypes or strides to a C-contiguous float32
// copy, as the reference's Eigen::Ref binding does. Searches return
// (ids int32, distances float32) arrays of n_queries x n_neighbors, best
// first, zero-filled past the number of results (src/CEOs.cpp:659-666).
//
// Differences, all deliberate: the GIL is released while the GPU works (the
// reference holds it); invalid parameters raise ValueError with the
// reference's message instead of printing it and calling exit(1)
// (src/CEOs.cpp:452-461, src/streamCEOs.cpp:179-189, :380-390); the
// reference's precision / device extensions are reachable through the
// `precision` attribute only (the rest of this library's API is in the
// ceos_gb300 Python package).
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>

#include <string>
#include <tuple>

#include "ceos_gb300.h"

namespace py = pybind11;

namespace {

using FloatRows = py::array_t<float, py::array::c_style | py::array::forcecast>;
using Result = std::tuple<py::array_t<int32_t>, py::array_t<float>>;

// A C ABI status as the Python exception of the reference's error path.
void check(int st) {
  if (st == CEOS_OK) return;
  const std::string msg = ceos_last_error();
  switch (st) {
    case CEOS_ERR_ARG:
    case CEOS_ERR_PROBED_POINTS:
    case CEOS_ERR_PROBED_VECTORS:
    case CEOS_ERR_UPDATE_DEL:
    case CEOS_ERR_UPDATE_TOPM:
    case CEOS_ERR_UNSUPPORTED:
      throw py::value_error(msg);
    default:
      throw std::runtime_error("[" + std::to_string(st) + "] " + msg);
  }
}

void check_rows(const FloatRows& a, int n_features, const char* what) {
  if (a.ndim() != 2 || a.shape(1) != n_features)
    throw py::value_error(std::string(what) + " must be a 2-D array with " + std::to_string(n_features) +
                          " columns");
}

Result empty_result(long nq, int k) {
  py::array_t<int32_t> ids({nq, (long)k});
  py::array_t<float> dists({nq, (long)k});
  return Result(std::move(ids), std::move(dists));
}

int precision_code(const std::string& p) {
  if (p == "fp32") return CEOS_PRECISION_FP32;
  if (p == "split_bf16") return CEOS_PRECISION_SPLIT_BF16;
  throw py::value_error("precision must be 'fp32' or 'split_bf16'");
}

// CEOs (src/CEOs.h:18-114)
class PyCEOs {
 public:
  PyCEOs(int n_points, int n_features) : n_(n_points), d_(n_features) {
    check(ceos_create(n_points, n_features, &h_));
  }
  ~PyCEOs() { ceos_destroy(h_); }
  PyCEOs(const PyCEOs&) = delete;
  PyCEOs& operator=(const PyCEOs&) = delete;

  void set_index_param(int n_proj, int n_repeats, int top_m, int n_threads, int random_seed) {
    check(ceos_set_index_param(h_, n_proj, n_repeats, top_m, n_threads, random_seed));
  }
  int get_q(int which) const {
    int s, p, c;
    check(ceos_get_query_param(h_, &s, &p, &c));
    return which == 0 ? s : which == 1 ? p : c;
  }
  void set_q(int which, int v) {
    int s, p, c;
    check(ceos_get_query_param(h_, &s, &p, &c));
    if (which == 0) s = v;
    else if (which == 1) p = v;
    else c = v;
    check(ceos_set_query_param(h_, s, p, c));
  }
  bool centering() const {
    int c;
    check(ceos_get_centering(h_, &c));
    return c != 0;
  }
  void set_centering(bool c) { check(ceos_set_centering(h_, c ? 1 : 0)); }
  std::string precision() const {
    int p;
    check(ceos_get_precision(h_, &p));
    return p == CEOS_PRECISION_SPLIT_BF16 ? "split_bf16" : "fp32";
  }
  void set_precision(const std::string& p) { check(ceos_set_precision(h_, precision_code(p))); }
  void set_threads(int t) { check(ceos_set_threads(h_, t)); }
  void clear() { check(ceos_clear(h_)); }

  template <int (*BUILD)(ceos_index*, const float*)>
  void build(const FloatRows& X) {
    check_rows(X, d_, "dataset");
    if (X.shape(0) != n_) throw py::value_error("dataset must have n_points = " + std::to_string(n_) + " rows");
    const float* p = X.data();
    int st;
    {
      py::gil_scoped_release nogil;
      st = BUILD(h_, p);
    }
    check(st);
  }

  template <int (*SEARCH)(ceos_index*, const float*, int, int, int, int32_t*, float*)>
  Result search(const FloatRows& Q, int k, bool verbose) {
    check_rows(Q, d_, "queries");
    if (k < 0) throw py::value_error("n_neighbors must be >= 0");
    const long nq = (long)Q.shape(0);
    Result r = empty_result(nq, k);
    int32_t* ids = std::get<0>(r).mutable_data();
    float* dists = std::get<1>(r).mutable_data();
    const float* q = Q.data();
    int st;
    {
      py::gil_scoped_release nogil;
      st = SEARCH(h_, q, (int)nq, k, verbose ? 1 : 0, ids, dists);
    }
    check(st);
    return r;
  }

 private:
  ceos_index* h_ = nullptr;
  int n_, d_;
};

// streamCEOs (src/streamCEOs.h:12-107)
class PyStream {
 public:
  explicit PyStream(int n_features) : d_(n_features) { check(ceos_stream_create(n_features, &h_)); }
  ~PyStream() { ceos_stream_destroy(h_); }
  PyStream(const PyStream&) = delete;
  PyStream& operator=(const PyStream&) = delete;

  void set_index_param(int n_proj, int n_repeats, int top_points, int n_threads, int random_seed) {
    check(ceos_stream_set_index_param(h_, n_proj, n_repeats, top_points, n_threads, random_seed));
  }
  int get_q(int which) const {
    int s, p, c;
    check(ceos_stream_get_query_param(h_, &s, &p, &c));
    return which == 0 ? s : which == 1 ? p : c;
  }
  void set_q(int which, int v) {
    int s, p, c;
    check(ceos_stream_get_query_param(h_, &s, &p, &c));
    if (which == 0) s = v;
    else if (which == 1) p = v;
    else c = v;
    check(ceos_stream_set_query_param(h_, s, p, c));
  }
  std::string precision() const {
    int p;
    check(ceos_stream_get_precision(h_, &p));
    return p == CEOS_PRECISION_SPLIT_BF16 ? "split_bf16" : "fp32";
  }
  void set_precision(const std::string& p) { check(ceos_stream_set_precision(h_, precision_code(p))); }
  void set_threads(int t) { check(ceos_stream_set_threads(h_, t)); }
  void clear() { check(ceos_stream_clear(h_)); }

  void build(const FloatRows& X) {
    check_rows(X, d_, "dataset");
    const float* p = X.data();
    const int n = (int)X.shape(0);
    int st;
    {
      py::gil_scoped_release nogil;
      st = ceos_stream_build(h_, p, n);
    }
    check(st);
  }
  void update(const FloatRows& X, int n_del) {
    check_rows(X, d_, "new_dataset");
    const float* p = X.data();
    const int n = (int)X.shape(0);
    int st;
    {
      py::gil_scoped_release nogil;
      st = ceos_stream_update(h_, p, n, n_del);
    }
    check(st);
  }
  template <int (*SEARCH)(ceos_stream*, const float*, int, int, int, int32_t*, float*)>
  Result search(const FloatRows& Q, int k, bool verbose) {
    check_rows(Q, d_, "queries");
    if (k < 0) throw py::value_error("n_neighbors must be >= 0");
    const long nq = (long)Q.shape(0);
    Result r = empty_result(nq, k);
    int32_t* ids = std::get<0>(r).mutable_data();
    float* dists = std::get<1>(r).mutable_data();
    const float* q = Q.data();
    int st;
    {
      py::gil_scoped_release nogil;
      st = SEARCH(h_, q, (int)nq, k, verbose ? 1 : 0, ids, dists);
    }
    check(st);
    return r;
  }

 private:
  ceos_stream* h_ = nullptr;
  int d_;
};

}  // namespace

PYBIND11_MODULE(CEOs, m) {
  m.doc() = "CEOs / coCEOs / streamCEOs maximum inner product search on one GB300 GPU";

  py::class_<PyCEOs>(m, "CEOs")
      .def(py::init<int, int>(), py::arg("n_points"), py::arg("n_features"),
           "Constructor for CEOs.\nn_points: number of points.\nn_features: number of dimensions.")
      .def("setIndexParam", &PyCEOs::set_index_param, py::arg("n_proj"), py::arg("n_repeats") = 1,
           py::arg("top_m") = 10, py::arg("n_threads") = -1, py::arg("random_seed") = -1,
           "n_proj: projections per repeat; n_repeats: repeats (n_proj * n_repeats projections in "
           "all); top_m: points kept at each end of every projection; n_threads: kept for "
           "compatibility; random_seed: seed of the sign tables (< 0: wall clock).")
      .def_property("n_probed_vectors", [](const PyCEOs& s) { return s.get_q(0); },
                    [](PyCEOs& s, int v) { s.set_q(0, v); },
                    "Number of probed vectors among n_repeats * n_proj random vectors.")
      .def_property("n_probed_points", [](const PyCEOs& s) { return s.get_q(1); },
                    [](PyCEOs& s, int v) { s.set_q(1, v); },
                    "Number of probed points for each random vector; at most top_m.")
      .def_property("n_cand", [](const PyCEOs& s) { return s.get_q(2); },
                    [](PyCEOs& s, int v) { s.set_q(2, v); },
                    "Number of candidates whose dot product is computed for each query.")
      .def_property("centering", &PyCEOs::centering, &PyCEOs::set_centering,
                    "Center the rows by their column means in build_CEOs_Hash (default False).")
      .def_property("precision", &PyCEOs::precision, &PyCEOs::set_precision,
                    "'fp32' (default) or 'split_bf16' (bfloat16 rerank scan, FP32 rescore).")
      .def("set_threads", &PyCEOs::set_threads, py::arg("n_threads"))
      .def("clear", &PyCEOs::clear)
      .def("build", &PyCEOs::build<ceos_build>, py::arg("dataset"))
      .def("search", &PyCEOs::search<ceos_search>, py::arg("queries"), py::arg("n_neighbors"),
           py::arg("verbose") = false)
      .def("build_coCEOs_Est", &PyCEOs::build<ceos_build_coceos_est>, py::arg("dataset"))
      .def("search_coCEOs_Est", &PyCEOs::search<ceos_search_coceos_est>, py::arg("queries"),
           py::arg("n_neighbors"), py::arg("verbose") = false)
      .def("build_CEOs_Hash", &PyCEOs::build<ceos_build_ceos_hash>, py::arg("dataset"))
      .def("search_CEOs_Hash", &PyCEOs::search<ceos_search_ceos_hash>, py::arg("queries"),
           py::arg("n_neighbors"), py::arg("verbose") = false);

  py::class_<PyStream>(m, "streamCEOs")
      .def(py::init<int>(), py::arg("n_features"))
      .def("setIndexParam", &PyStream::set_index_param, py::arg("n_proj"), py::arg("n_repeats") = 1,
           py::arg("top_points") = 1, py::arg("n_threads") = -1, py::arg("random_seed") = -1)
      .def_property("n_probed_vectors", [](const PyStream& s) { return s.get_q(0); },
                    [](PyStream& s, int v) { s.set_q(0, v); })
      .def_property("n_probed_points", [](const PyStream& s) { return s.get_q(1); },
                    [](PyStream& s, int v) { s.set_q(1, v); })
      .def_property("n_cand", [](const PyStream& s) { return s.get_q(2); },
                    [](PyStream& s, int v) { s.set_q(2, v); })
      .def_property("precision", &PyStream::precision, &PyStream::set_precision)
      .def("set_threads", &PyStream::set_threads, py::arg("n_threads"))
      .def("clear", &PyStream::clear)
      .def("build", &PyStream::build, py::arg("dataset"))
      .def("update", &PyStream::update, py::arg("new_dataset"), py::arg("n_delPoints") = 0)
      .def("estimate_search", &PyStream::search<ceos_stream_estimate_search>, py::arg("queries"),
           py::arg("n_neighbors"), py::arg("verbose") = false)
      .def("hash_search", &PyStream::search<ceos_stream_hash_search>, py::arg("queries"),
           py::arg("n_neighbors"), py::arg("verbose") = false);
}
