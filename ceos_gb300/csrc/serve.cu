// Serving loop over a device-resident index (no counterpart in the reference,
// whose searches are one blocking batch call per Python method,
// python/python_wrapper.cpp:36-48, :62-71).
//
// A server owns one worker thread and `n_slots` device slots. Clients submit
// requests (a block of queries with its own n_neighbors and n_probed_vectors,
// or a streamCEOs update) from any thread; the worker
//   * retires slots whose batch finished (event query), copies each request's
//     rows of the result to the caller's buffers and records its latency;
//   * packs the queued query requests, in arrival order, into the next free
//     slot: up to max_batch queries, splitting a request that does not fit
//     (continuous batching: whatever arrived while the other slots were busy
//     goes into the next slot that frees up, and slots run concurrently on
//     their own streams);
//   * runs an update only when no batch is in flight, so every request sees
//     the index as of its place in the queue.
// A slot's batch is one fixed sequence (query upload, row padding, query
// projection, the persistent query kernel, result download) over a
// power-of-two bucket of rows; with graphs on, each (slot, bucket) sequence is
// captured once as a CUDA graph and replayed. The real query count, and each
// query's probes, neighbours, table size and output offset, travel in a small
// metadata block, so one graph serves every mix. A query's result does not
// depend on its batch: the kernel processes each query independently, with
// a hash table sized for that query's own probes and a total order on
// (score, id).
#include <atomic>
#include <condition_variable>
#include <deque>
#include <memory>
#include <thread>
#include <unordered_map>

#include "core.h"

using namespace ceos_host;

namespace {

using Clock = std::chrono::steady_clock;

enum ReqKind { R_QUERY = 0, R_UPDATE = 1, R_DELETE = 2 };

struct Request {
  uint64_t ticket = 0;
  int kind = R_QUERY;
  std::vector<float> data;  // queries (nq x d) or new rows (n_new x d)
  std::vector<int32_t> del;  // ids of a delete
  int nq = 0, k = 0, s = 0, cap = 0;
  int n_new = 0, n_del = 0;
  int32_t* ids = nullptr;
  float* dists = nullptr;
  int next_q = 0;    // first query not yet packed
  int inflight = 0;  // pieces in flight
  int status = CEOS_OK;
  bool done = false;
  Clock::time_point t_submit;
};

struct Piece {
  Request* r;
  int q0, nq;
  long off;  // offset of the piece's results in the slot's output block
};

template <typename T>
struct Pinned {
  T* p = nullptr;
  cudaError_t alloc(size_t n) {
    void* v = nullptr;
    cudaError_t e = cudaHostAlloc(&v, std::max<size_t>(n, 1) * sizeof(T), cudaHostAllocDefault);
    p = reinterpret_cast<T*>(v);
    return e;
  }
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
};

// Metadata block of a slot (host pinned and device): [0] = query count, then
// per query: probes, neighbours, table capacity (int32) and result offset (int64).
struct MetaLayout {
  size_t s_off, k_off, cap_off, o_off, bytes;
  explicit MetaLayout(int B = 0) {
    s_off = 16;
    k_off = s_off + (size_t)B * 4;
    cap_off = k_off + (size_t)B * 4;
    o_off = (cap_off + (size_t)B * 4 + 15) & ~(size_t)15;
    bytes = o_off + (size_t)B * 8;
  }
};

struct Slot {
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  DevBuf dStage, dQ, dQproj, dMeta, dIds, dD, dTable, dSort;
  Pinned<float> hQ;
  Pinned<unsigned char> hMeta;
  Pinned<int32_t> hIds;
  Pinned<float> hD;
  std::vector<Piece> pieces;
  bool busy = false;
  int nq = 0;
  std::unordered_map<int, cudaGraphExec_t> graphs;  // bucket rows -> executable graph
};

}  // namespace

struct ceos_server {
  ceos_server_config cfg{};
  Core* core = nullptr;
  ceos_stream* stream_handle = nullptr;
  int mode = Q_ESTIMATE;
  int d = 0, ldx = 0, C = 0, p = 0, c = 0;
  int max_cap = 0;
  bool table_in_smem = true;
  bool sorted = false;  // estimate searches through k_query_sorted
  long sort_cap = 0;
  size_t smem = 0;
  int grid_max = 1;
  size_t slot_bytes = 0;
  MetaLayout meta;
  std::vector<std::unique_ptr<Slot>> slots;

  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::thread worker;

  // statistics since the last reset (guarded by mu)
  std::vector<double> lat_ms;
  long long n_requests = 0, n_queries = 0, n_batches = 0, n_graph_launches = 0,
            n_graphs_captured = 0, n_updates = 0;
  bool have_first = false;
  Clock::time_point t_first, t_last;

  ~ceos_server() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv_work.notify_all();
    if (worker.joinable()) worker.join();
    if (core && core->device >= 0) cudaSetDevice(core->device);
    for (auto& sl : slots) {
      for (auto& g : sl->graphs) cudaGraphExecDestroy(g.second);
      sl->graphs.clear();
      if (sl->done) cudaEventDestroy(sl->done);
      if (sl->st) cudaStreamDestroy(sl->st);
    }
    slots.clear();
    if (core) core->attached = 0;
  }

  int bucket_rows(int n) const {
    int b = 1;
    while (b < n) b <<= 1;
    return std::min(b, cfg.max_batch);
  }

  QueryArgs slot_args(Slot& sl, int rows) const {
    QueryArgs q = core->query_base(rows, cfg.max_neighbors);
    q.Q = sl.dQ.as<float>();
    q.qproj = sl.dQproj.as<float>();
    q.s = cfg.max_probed_vectors;
    q.k = cfg.max_neighbors;
    q.c = c;
    q.p = p;
    const unsigned char* m = sl.dMeta.as<unsigned char>();
    q.d_nq = reinterpret_cast<const int*>(m);
    q.q_s = reinterpret_cast<const int*>(m + meta.s_off);
    q.q_k = reinterpret_cast<const int*>(m + meta.k_off);
    q.q_cap = reinterpret_cast<const int*>(m + meta.cap_off);
    q.q_off = reinterpret_cast<const long*>(m + meta.o_off);
    q.out_ids = sl.dIds.as<int32_t>();
    q.out_d = sl.dD.as<float>();
    if (q.Xb) q.rescore_per_k = 4;
    q.table_cap = max_cap;
    q.table_in_smem = table_in_smem ? 1 : 0;
    q.gtable = table_in_smem ? nullptr : sl.dTable.as<uint64_t>();
    if (sorted) {
      q.sort_scratch = sl.dSort.as<int2>();
      q.sort_cap = sort_cap;
      int bits = 1;
      while (bits < 31 && (1L << bits) <= core->n_rows) ++bits;
      q.id_bits = bits;  // from the current size: graphs are captured again after updates
    }
    return q;
  }

  // The fixed work of one batch of `rows` rows on the slot's stream.
  int issue(Slot& sl, int rows) {
    const cudaStream_t st = sl.st;
    CUDA_TRY(cudaMemcpyAsync(sl.dMeta.p, sl.hMeta.p, meta.bytes, cudaMemcpyHostToDevice, st));
    const size_t raw = (size_t)rows * d * 4;
    if (ldx == d) {
      CUDA_TRY(cudaMemcpyAsync(sl.dQ.p, sl.hQ.p, raw, cudaMemcpyHostToDevice, st));
    } else {
      CUDA_TRY(cudaMemcpyAsync(sl.dStage.p, sl.hQ.p, raw, cudaMemcpyHostToDevice, st));
      CUDA_TRY(launch_pad_rows(sl.dStage.as<float>(), rows, d, sl.dQ.as<float>(), ldx, st));
    }
    ProjArgs a = core->query_proj_base();
    a.X = sl.dQ.as<float>();
    a.head = 0;
    a.cap_rows = LONG_MAX;
    a.n_rows = rows;
    a.out = sl.dQproj.as<float>();
    CUDA_TRY(launch_project(a, PROJ_ROWS, core->L, core->sms, st));
    QueryArgs q = slot_args(sl, rows);
    const int grid = std::max(1, std::min(rows, grid_max));
    if (sorted)
      CUDA_TRY(launch_query_sorted(q, grid, smem, st));
    else
      CUDA_TRY(launch_query_buckets(q, mode, grid, smem, st));
    const size_t outb = (size_t)rows * cfg.max_neighbors * 4;
    CUDA_TRY(cudaMemcpyAsync(sl.hIds.p, sl.dIds.p, outb, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(sl.hD.p, sl.dD.p, outb, cudaMemcpyDeviceToHost, st));
    return CEOS_OK;
  }

  int graph_for(Slot& sl, int rows, cudaGraphExec_t* out) {
    auto it = sl.graphs.find(rows);
    if (it != sl.graphs.end()) {
      *out = it->second;
      return CEOS_OK;
    }
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(sl.st, cudaStreamCaptureModeRelaxed));
    const int st = issue(sl, rows);
    cudaError_t e = cudaStreamEndCapture(sl.st, &g);
    if (st != CEOS_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    CUDA_TRY(e);
    cudaGraphExec_t ex = nullptr;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    CUDA_TRY(e);
    sl.graphs[rows] = ex;
    {
      std::lock_guard<std::mutex> lk(mu);
      ++n_graphs_captured;
    }
    *out = ex;
    return CEOS_OK;
  }

  void drop_graphs() {
    for (auto& sl : slots) {
      for (auto& g : sl->graphs) cudaGraphExecDestroy(g.second);
      sl->graphs.clear();
    }
  }

  // Fill the slot's staging blocks from its pieces and launch the batch.
  int launch(Slot& sl) {
    unsigned char* m = sl.hMeta.p;
    int* qs = reinterpret_cast<int*>(m + meta.s_off);
    int* qk = reinterpret_cast<int*>(m + meta.k_off);
    int* qc = reinterpret_cast<int*>(m + meta.cap_off);
    long* qo = reinterpret_cast<long*>(m + meta.o_off);
    int row = 0;
    for (const Piece& pc : sl.pieces) {
      const Request* r = pc.r;
      std::memcpy(sl.hQ.p + (size_t)row * d, r->data.data() + (size_t)pc.q0 * d,
                  (size_t)pc.nq * d * 4);
      for (int j = 0; j < pc.nq; ++j) {
        qs[row + j] = r->s;
        qk[row + j] = r->k;
        qc[row + j] = r->cap;
        qo[row + j] = pc.off + (long)j * r->k;
      }
      row += pc.nq;
    }
    reinterpret_cast<int*>(m)[0] = row;
    sl.nq = row;
    const int rows = bucket_rows(row);
    if (cfg.use_graphs) {
      cudaGraphExec_t ex = nullptr;
      ST_TRY(graph_for(sl, rows, &ex));
      CUDA_TRY(cudaGraphLaunch(ex, sl.st));
    } else {
      ST_TRY(issue(sl, rows));
    }
    CUDA_TRY(cudaEventRecord(sl.done, sl.st));
    std::lock_guard<std::mutex> lk(mu);
    ++n_batches;
    n_queries += row;
    if (cfg.use_graphs) ++n_graph_launches;
    return CEOS_OK;
  }

  void complete(Request* r, Clock::time_point now) {  // caller holds mu
    r->done = true;
    if (r->kind != R_QUERY) return;
    ++n_requests;
    lat_ms.push_back(std::chrono::duration<double, std::milli>(now - r->t_submit).count());
    t_last = now;
  }

  void retire(Slot& sl, int status) {
    if (status == CEOS_OK) {
      for (const Piece& pc : sl.pieces) {
        const size_t n = (size_t)pc.nq * pc.r->k;
        std::memcpy(pc.r->ids + (size_t)pc.q0 * pc.r->k, sl.hIds.p + pc.off, n * 4);
        std::memcpy(pc.r->dists + (size_t)pc.q0 * pc.r->k, sl.hD.p + pc.off, n * 4);
      }
    }
    const auto now = Clock::now();
    {
      std::lock_guard<std::mutex> lk(mu);
      for (const Piece& pc : sl.pieces) {
        Request* r = pc.r;
        if (status != CEOS_OK) r->status = status;
        if (--r->inflight == 0 && r->next_q == r->nq) complete(r, now);
      }
    }
    sl.pieces.clear();
    sl.busy = false;
    cv_done.notify_all();
  }

  int run_update(Request* r);

  void loop() {
    cudaSetDevice(core->device);
    for (;;) {
      bool progressed = false;
      for (auto& slp : slots) {
        Slot& sl = *slp;
        if (!sl.busy) continue;
        const cudaError_t e = cudaEventQuery(sl.done);
        if (e == cudaErrorNotReady) continue;
        retire(sl, e == cudaSuccess ? CEOS_OK
                                    : fail(CEOS_ERR_CUDA, "serving batch failed: %s",
                                           cudaGetErrorString(e)));
        progressed = true;
      }
      bool any_busy = false;
      for (auto& slp : slots) any_busy |= slp->busy;
      std::unique_lock<std::mutex> lk(mu);
      if (!queue.empty()) {
        Request* head = queue.front();
        if (head->kind != R_QUERY) {
          if (!any_busy) {
            queue.pop_front();
            lk.unlock();
            const int st = run_update(head);
            lk.lock();
            head->status = st;
            complete(head, Clock::now());
            ++n_updates;
            lk.unlock();
            cv_done.notify_all();
            progressed = true;
            continue;
          }
        } else {
          for (auto& slp : slots) {
            Slot& sl = *slp;
            if (sl.busy || queue.empty() || queue.front()->kind != R_QUERY) continue;
            int packed = 0;
            long off = 0;
            while (!queue.empty() && queue.front()->kind == R_QUERY && packed < cfg.max_batch) {
              Request* r = queue.front();
              const int take = std::min(r->nq - r->next_q, cfg.max_batch - packed);
              sl.pieces.push_back(Piece{r, r->next_q, take, off});
              r->next_q += take;
              ++r->inflight;
              packed += take;
              off += (long)take * r->k;
              if (r->next_q == r->nq) queue.pop_front();
            }
            sl.busy = true;
            lk.unlock();
            const int st = launch(sl);
            if (st != CEOS_OK) {
              cudaStreamSynchronize(sl.st);
              retire(sl, st);
            }
            lk.lock();
            progressed = true;
          }
        }
      } else if (stop && !any_busy) {
        return;
      }
      if (!progressed) {
        if (any_busy) {
          lk.unlock();
          std::this_thread::yield();
        } else if (queue.empty() && !stop) {
          cv_work.wait(lk);
        }
      }
    }
  }
};

int ceos_server::run_update(Request* r) {
  if (!stream_handle) return fail(CEOS_ERR_ARG, "updates need a streamCEOs server");
  const int st = r->kind == R_DELETE
                     ? ceos_host::stream_delete(stream_handle, r->del.data(), (int)r->del.size())
                     : ceos_host::stream_update(stream_handle, r->data.data(), r->n_new, r->n_del);
  if (st != CEOS_OK) return st;
  ST_TRY(core->ensure_bf16());
  CUDA_TRY(cudaStreamSynchronize(core->stream));
  // graphs hold the ring's pointers, head and size: capture again on demand
  drop_graphs();
  return CEOS_OK;
}

namespace {

int server_create(Core& c, ceos_stream* sh, const ceos_server_config* cfg_in, ceos_server** out) {
  if (!out) return fail(CEOS_ERR_ARG, "null output handle");
  *out = nullptr;
  ceos_server_config cfg;
  ceos_server_config_init(&cfg);
  if (cfg_in) cfg = *cfg_in;
  const bool is_stream = sh != nullptr;
  if (is_stream ? c.built != B_STREAM : (c.built != B_COCEOS && c.built != B_HASH))
    return fail(CEOS_ERR_NOT_BUILT, "the server needs a built coCEOs-Est / CEOs-Hash / streamCEOs index");
  if (c.attached) return fail(CEOS_ERR_BUSY, "the index already has a server");
  int mode;
  if (cfg.algo == CEOS_ALGO_COCEOS && (is_stream || c.built == B_COCEOS)) {
    mode = Q_ESTIMATE;
  } else if (cfg.algo == CEOS_ALGO_HASH && (is_stream || c.built == B_HASH)) {
    mode = Q_UNION;
  } else {
    return fail(CEOS_ERR_ARG, "algo %d does not match the built index", cfg.algo);
  }
  if (cfg.n_slots < 1 || cfg.max_batch < 1 || cfg.max_neighbors < 1 || cfg.max_probed_vectors < 1)
    return fail(CEOS_ERR_ARG, "n_slots, max_batch, max_neighbors and max_probed_vectors must be >= 1");
  const int s_limit = is_stream ? c.n_proj : c.C();  // src/CEOs.cpp:457-461, src/streamCEOs.cpp:386-390
  if (cfg.max_probed_vectors > s_limit)
    return fail(CEOS_ERR_PROBED_VECTORS, "max_probed_vectors (%d) exceeds %d", cfg.max_probed_vectors, s_limit);
  if (c.p > c.top_m)
    return fail(CEOS_ERR_PROBED_POINTS, "n_probed_points (%d) exceeds top_m (%d)", c.p, c.top_m);
  ST_TRY(c.ensure_device());
  ST_TRY(c.ensure_bf16());
  CUDA_TRY(cudaStreamSynchronize(c.stream));

  auto srv = std::make_unique<ceos_server>();
  ceos_server& S = *srv;
  S.cfg = cfg;
  S.core = &c;
  S.stream_handle = sh;
  S.mode = mode;
  S.d = c.n_features;
  S.ldx = c.ldx;
  S.C = c.C();
  S.p = c.p;
  S.c = c.c;
  const long tc = table_capacity(cfg.max_probed_vectors, c.p);
  if (tc < 0) return fail(CEOS_ERR_UNSUPPORTED, "max_probed_vectors * n_probed_points too large");
  S.max_cap = (int)tc;
  S.meta = MetaLayout(cfg.max_batch);
  // launch shape of the query kernel for the largest request parameters
  QueryArgs q = c.query_base(cfg.max_batch, cfg.max_neighbors);
  q.s = cfg.max_probed_vectors;
  q.k = cfg.max_neighbors;
  q.table_cap = S.max_cap;
  q.table_in_smem = 1;
  size_t smem = query_buckets_smem(q, mode);
  if (smem > c.smem_optin) {
    q.table_in_smem = 0;
    smem = query_buckets_smem(q, mode);
    if (smem > c.smem_optin)
      return fail(CEOS_ERR_UNSUPPORTED, "query working set (n_cand=%d, max_neighbors=%d) exceeds shared memory",
                  c.c, cfg.max_neighbors);
  }
  S.table_in_smem = q.table_in_smem != 0;
  S.smem = smem;
  int per_sm = std::max(1, query_buckets_blocks_per_sm(mode, smem, S.table_in_smem));
  if (mode == Q_ESTIMATE && c.use_sorted(q)) {
    // the sorted estimate path, for the largest requests
    S.sorted = true;
    S.sort_cap = std::max(1L, (long)cfg.max_probed_vectors * c.p);
    QueryArgs qs = q;
    qs.sort_cap = S.sort_cap;
    S.smem = query_sorted_smem(qs);
    if (S.smem > c.smem_optin)
      return fail(CEOS_ERR_UNSUPPORTED, "query working set (n_cand=%d, max_neighbors=%d) exceeds shared memory",
                  c.c, cfg.max_neighbors);
    S.table_in_smem = true;
    per_sm = std::max(1, query_sorted_blocks_per_sm(S.smem));
  }
  S.grid_max = std::max(1, std::min(cfg.max_batch, c.sms * per_sm));
  // device bytes of one slot
  const size_t B = (size_t)cfg.max_batch;
  const size_t stage = S.ldx == S.d ? 0 : B * S.d * 4;
  const size_t table = S.table_in_smem ? 0 : (size_t)S.grid_max * S.max_cap * 8;
  const size_t sortb = S.sorted ? (size_t)S.grid_max * 2 * S.sort_cap * 8 : 0;
  S.slot_bytes = stage + B * S.ldx * 4 + B * S.C * 4 + S.meta.bytes + 2 * B * cfg.max_neighbors * 4 + table +
                 sortb;
  int n_slots = cfg.n_slots;
  if (cfg.mem_budget_bytes > 0)
    n_slots = (int)std::min<long long>(n_slots, cfg.mem_budget_bytes / (long long)S.slot_bytes);
  if (n_slots < 1)
    return fail(CEOS_ERR_ARG, "mem_budget_bytes (%lld) is below one slot (%zu bytes)",
                cfg.mem_budget_bytes, S.slot_bytes);
  for (int i = 0; i < n_slots; ++i) {
    auto sl = std::make_unique<Slot>();
    CUDA_TRY(cudaStreamCreateWithFlags(&sl->st, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming));
    if (stage) CUDA_TRY(sl->dStage.ensure(stage));
    CUDA_TRY(sl->dQ.ensure(B * S.ldx * 4));
    CUDA_TRY(cudaMemset(sl->dQ.p, 0, B * S.ldx * 4));
    CUDA_TRY(sl->dQproj.ensure(B * S.C * 4));
    CUDA_TRY(sl->dMeta.ensure(S.meta.bytes));
    CUDA_TRY(sl->dIds.ensure(B * cfg.max_neighbors * 4));
    CUDA_TRY(sl->dD.ensure(B * cfg.max_neighbors * 4));
    if (table) CUDA_TRY(sl->dTable.ensure(table));
    if (sortb) CUDA_TRY(sl->dSort.ensure(sortb));
    CUDA_TRY(sl->hQ.alloc(B * S.d));
    std::memset(sl->hQ.p, 0, B * S.d * 4);
    CUDA_TRY(sl->hMeta.alloc(S.meta.bytes));
    std::memset(sl->hMeta.p, 0, S.meta.bytes);
    CUDA_TRY(sl->hIds.alloc(B * cfg.max_neighbors));
    CUDA_TRY(sl->hD.alloc(B * cfg.max_neighbors));
    S.slots.push_back(std::move(sl));
  }
  S.cfg.n_slots = n_slots;
  c.attached = 1;
  S.worker = std::thread([&S] { S.loop(); });
  *out = srv.release();
  return CEOS_OK;
}

}  // namespace

extern "C" {

int ceos_server_config_init(ceos_server_config* cfg) {
  if (!cfg) return fail(CEOS_ERR_ARG, "null config");
  cfg->algo = CEOS_ALGO_COCEOS;
  cfg->n_slots = 4;
  cfg->max_batch = 256;
  cfg->max_neighbors = 100;
  cfg->max_probed_vectors = 80;
  cfg->mem_budget_bytes = 0;
  cfg->use_graphs = 1;
  return CEOS_OK;
}

int ceos_server_create(ceos_index* h, const ceos_server_config* cfg, ceos_server** out) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  return server_create(h->core, nullptr, cfg, out);
}

int ceos_server_create_stream(ceos_stream* h, const ceos_server_config* cfg, ceos_server** out) {
  if (!h) return fail(CEOS_ERR_ARG, "null handle");
  return server_create(h->core, h, cfg, out);
}

void ceos_server_destroy(ceos_server* s) { delete s; }

int ceos_server_submit(ceos_server* s, const float* Q, int n_queries, int n_neighbors,
                       int n_probed_vectors, int32_t* ids, float* dists, uint64_t* ticket) {
  if (!s || !ticket) return fail(CEOS_ERR_ARG, "null handle or ticket");
  if (n_queries < 0) return fail(CEOS_ERR_ARG, "n_queries must be >= 0");
  if (n_queries > 0 && (!Q || !ids || !dists)) return fail(CEOS_ERR_ARG, "null query or output buffer");
  if (n_neighbors < 1 || n_neighbors > s->cfg.max_neighbors)
    return fail(CEOS_ERR_ARG, "n_neighbors (%d) must be in [1, %d]", n_neighbors, s->cfg.max_neighbors);
  const int sq = n_probed_vectors > 0 ? n_probed_vectors : s->core->s;
  if (sq > s->cfg.max_probed_vectors)
    return fail(CEOS_ERR_PROBED_VECTORS, "n_probed_vectors (%d) exceeds the server's max_probed_vectors (%d)",
                sq, s->cfg.max_probed_vectors);
  auto r = std::make_unique<Request>();
  r->t_submit = Clock::now();
  r->kind = R_QUERY;
  r->nq = n_queries;
  r->k = n_neighbors;
  r->s = sq;
  r->cap = (int)table_capacity(sq, s->p);
  r->ids = ids;
  r->dists = dists;
  r->data.assign(Q, Q + (size_t)n_queries * s->d);
  std::unique_lock<std::mutex> lk(s->mu);
  r->ticket = s->next_ticket++;
  *ticket = r->ticket;
  if (!s->have_first) {
    s->have_first = true;
    s->t_first = r->t_submit;
  }
  Request* raw = r.get();
  s->reqs.emplace(raw->ticket, std::move(r));
  if (n_queries == 0) {
    s->complete(raw, Clock::now());
  } else {
    s->queue.push_back(raw);
  }
  lk.unlock();
  s->cv_work.notify_one();
  return CEOS_OK;
}

int ceos_server_submit_update(ceos_server* s, const float* X_new, int n_new, int n_del,
                              uint64_t* ticket) {
  if (!s || !ticket) return fail(CEOS_ERR_ARG, "null handle or ticket");
  if (!s->stream_handle) return fail(CEOS_ERR_ARG, "updates need a server over a streamCEOs index");
  if (n_new < 0 || n_del < 0) return fail(CEOS_ERR_ARG, "n_new and n_delPoints must be >= 0");
  if (n_new > 0 && !X_new) return fail(CEOS_ERR_ARG, "null new rows");
  auto r = std::make_unique<Request>();
  r->t_submit = Clock::now();
  r->kind = R_UPDATE;
  r->n_new = n_new;
  r->n_del = n_del;
  r->data.assign(X_new, X_new + (size_t)n_new * s->d);
  std::unique_lock<std::mutex> lk(s->mu);
  r->ticket = s->next_ticket++;
  *ticket = r->ticket;
  Request* raw = r.get();
  s->reqs.emplace(raw->ticket, std::move(r));
  s->queue.push_back(raw);
  lk.unlock();
  s->cv_work.notify_one();
  return CEOS_OK;
}

int ceos_server_submit_delete(ceos_server* s, const int32_t* ids, int n_ids, uint64_t* ticket) {
  if (!s || !ticket) return fail(CEOS_ERR_ARG, "null handle or ticket");
  if (!s->stream_handle) return fail(CEOS_ERR_ARG, "deletes need a server over a streamCEOs index");
  if (n_ids < 0 || (n_ids > 0 && !ids)) return fail(CEOS_ERR_ARG, "bad id list");
  auto r = std::make_unique<Request>();
  r->t_submit = Clock::now();
  r->kind = R_DELETE;
  r->del.assign(ids, ids + n_ids);
  std::unique_lock<std::mutex> lk(s->mu);
  r->ticket = s->next_ticket++;
  *ticket = r->ticket;
  Request* raw = r.get();
  s->reqs.emplace(raw->ticket, std::move(r));
  s->queue.push_back(raw);
  lk.unlock();
  s->cv_work.notify_one();
  return CEOS_OK;
}

int ceos_server_wait(ceos_server* s, uint64_t ticket, int timeout_ms) {
  if (!s) return fail(CEOS_ERR_ARG, "null handle");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return fail(CEOS_ERR_ARG, "unknown ticket %llu", (unsigned long long)ticket);
  Request* r = it->second.get();
  auto pred = [r] { return r->done; };
  if (timeout_ms < 0) {
    s->cv_done.wait(lk, pred);
  } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) {
    return fail(CEOS_ERR_TIMEOUT, "request %llu still running", (unsigned long long)ticket);
  }
  const int st = r->status;
  s->reqs.erase(it);
  if (st != CEOS_OK) return fail(st, "request %llu failed", (unsigned long long)ticket);
  return CEOS_OK;
}

int ceos_server_get_stats(ceos_server* s, ceos_server_stats* out) {
  if (!s || !out) return fail(CEOS_ERR_ARG, "null handle or output");
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->requests = s->n_requests;
  out->queries = s->n_queries;
  out->batches = s->n_batches;
  out->graph_launches = s->n_graph_launches;
  out->graphs_captured = s->n_graphs_captured;
  out->updates = s->n_updates;
  out->slots = (int)s->slots.size();
  out->slot_bytes = (long long)s->slot_bytes;
  out->mean_batch_queries = s->n_batches ? (double)s->n_queries / (double)s->n_batches : 0.0;
  std::vector<double> v = s->lat_ms;
  if (!v.empty()) {
    std::sort(v.begin(), v.end());
    auto pct = [&](double f) {
      const double pos = f * (double)(v.size() - 1);
      const size_t i = (size_t)pos;
      const double w = pos - (double)i;
      return i + 1 < v.size() ? v[i] * (1.0 - w) + v[i + 1] * w : v[i];
    };
    out->p50_ms = pct(0.50);
    out->p90_ms = pct(0.90);
    out->p99_ms = pct(0.99);
    out->max_ms = v.back();
    double sum = 0;
    for (double x : v) sum += x;
    out->mean_ms = sum / (double)v.size();
  }
  if (s->have_first && s->n_requests > 0)
    out->busy_s = std::chrono::duration<double>(s->t_last - s->t_first).count();
  return CEOS_OK;
}

int ceos_server_reset_stats(ceos_server* s) {
  if (!s) return fail(CEOS_ERR_ARG, "null handle");
  std::lock_guard<std::mutex> lk(s->mu);
  s->lat_ms.clear();
  s->n_requests = s->n_queries = s->n_batches = s->n_graph_launches = s->n_updates = 0;
  s->have_first = false;
  return CEOS_OK;
}

}  // extern "C"
