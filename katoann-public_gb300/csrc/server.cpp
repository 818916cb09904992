// katoann::Server: continuous batching over one Index (include/katoann/server.h).
//
// Two threads. The dispatcher takes the oldest waiting request's k class,
// forms a batch of up to max_batch of its requests, carves the batch's device
// memory (search workspace, queries, results) out of one HBM pool and, once a
// slot (stream, event, pinned buffers) is free, launches copy-in, search and
// copy-out on the slot's stream without waiting. The completer waits for the
// batches in launch order, hands the results to their requests and returns
// the memory and the slot. A batch that does not fit in the free pool waits
// for completions; with nothing in flight it is cut to the size that fits.
// In graph mode every slot owns a full batch's memory instead, and a batch
// replays the slot's captured search for its k and padded size.
#include "katoann/server.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <random>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>

#include "katoann/probe.h"
#include "katoann_gpu.h"

namespace katoann {

namespace {

using Clock = std::chrono::steady_clock;

void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// First-fit allocator over one device block (offsets, 256-byte aligned).
class Pool {
 public:
  void init(size_t bytes) {
    cuda_check(cudaMalloc(&base_, bytes), "server pool");
    size_ = bytes;
    free_[0] = bytes;
  }
  ~Pool() {
    if (base_) cudaFree(base_);
  }
  // offset of a block of `bytes`, or SIZE_MAX
  size_t take(size_t bytes) {
    bytes = align256(bytes);
    for (auto it = free_.begin(); it != free_.end(); ++it)
      if (it->second >= bytes) {
        const size_t at = it->first, rest = it->second - bytes;
        free_.erase(it);
        if (rest) free_[at + bytes] = rest;
        used_ += bytes;
        peak_ = std::max(peak_, used_);
        return at;
      }
    return SIZE_MAX;
  }
  void give(size_t at, size_t bytes) {
    bytes = align256(bytes);
    used_ -= bytes;
    auto it = free_.emplace(at, bytes).first;
    auto next = std::next(it);
    if (next != free_.end() && it->first + it->second == next->first) {
      it->second += next->second;
      free_.erase(next);
    }
    if (it != free_.begin()) {
      auto prev = std::prev(it);
      if (prev->first + prev->second == it->first) {
        prev->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t largest() const {
    size_t m = 0;
    for (const auto &f : free_) m = std::max(m, f.second);
    return m;
  }
  unsigned char *at(size_t off) const { return static_cast<unsigned char *>(base_) + off; }
  size_t peak() const { return peak_; }
  void reset_peak() { peak_ = used_; }

 private:
  void *base_ = nullptr;
  size_t size_ = 0, used_ = 0, peak_ = 0;
  std::map<size_t, size_t> free_;
};

struct Request {
  uint64_t id;
  std::vector<float> q;
  Clock::time_point t;
};

struct Entry {
  bool done = false;
  std::string err;
  ServerResult res;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t start = nullptr;  // recorded before the batch's copies (timing)
  cudaEvent_t event = nullptr;  // after its results' copies (timing, blocking wait)
  float *hq = nullptr;       // pinned: max_batch x dim
  uint32_t *hids = nullptr;  // pinned: max_batch x max_k
  float *hd = nullptr;
  uint32_t *hnp = nullptr;   // pinned: max_batch
  bool busy = false;
  size_t base = SIZE_MAX;    // graph mode: the slot's own block of the pool
  std::map<uint64_t, void *> graph;  // (k << 32 | padded size) -> captured search
};

// Device pointers of one batch of n queries at k within its memory block.
struct Layout {
  unsigned char *ws;
  size_t ws_bytes;
  float *dq;
  uint32_t *dids;
  float *dd;
  uint32_t *dnp;
};

struct Batch {
  Slot *slot;
  uint32_t k, n;
  size_t off, bytes;
  std::vector<Request> reqs;
  std::string err;           // a launch that failed
  double enqueue_ms = 0;     // host time of launch()
  bool graph = false;        // replayed a captured search
};

}  // namespace

struct Server::Impl {
  ServerOptions opt;
  const katoann_gpu_index *view = nullptr;
  uint32_t dim = 0, depth = 0, max_batch = 0;
  int rk = KATO_RANK_PREFIX;
  katoann_gpu_probe_model model{};
  bool use_model = false;
  Pool pool;
  std::vector<Slot> slots;

  mutable std::mutex mu;
  std::condition_variable cv_dispatch, cv_complete, cv_done;
  std::map<uint32_t, std::deque<Request>> waiting;  // by k
  std::unordered_map<uint64_t, Entry> entries;
  std::deque<Batch> launched;
  uint64_t next_id = 1, pending = 0, submitted = 0, nbatches = 0, batched = 0;
  uint32_t in_flight = 0, peak_in_flight = 0;
  double max_enqueue_ms = 0, max_batch_gpu_ms = 0;
  bool stop = false;
  std::thread dispatcher, completer;
  bool graphs = false;        // graph mode (fixed slot memory, captured searches)
  size_t slot_bytes = 0;      // a slot's block in graph mode
  uint64_t graph_batches = 0;
  uint32_t graphs_captured = 0;  // written by the thread that captures, under mu

  size_t batch_bytes(uint32_t n, uint32_t k) const {
    const size_t ws = katoann_gpu_search_workspace(view, n, k, depth, rk, opt.survivors);
    if (ws == 0) return 0;
    return align256(ws) + align256(size_t(n) * dim * 4) + 2 * align256(size_t(n) * k * 4) +
           align256(size_t(n) * 4);
  }

  Layout layout(unsigned char *p, uint32_t n, uint32_t k) const {
    Layout L;
    L.ws = p;
    L.ws_bytes = align256(katoann_gpu_search_workspace(view, n, k, depth, rk, opt.survivors));
    L.dq = reinterpret_cast<float *>(p + L.ws_bytes);
    L.dids = reinterpret_cast<uint32_t *>(p + L.ws_bytes + align256(size_t(n) * dim * 4));
    L.dd = reinterpret_cast<float *>(reinterpret_cast<unsigned char *>(L.dids) +
                                     align256(size_t(n) * k * 4));
    L.dnp = reinterpret_cast<uint32_t *>(reinterpret_cast<unsigned char *>(L.dd) +
                                         align256(size_t(n) * k * 4));
    return L;
  }

  // graph mode: the size a batch of n runs at. Up to 16, the next power of
  // two; above, the next multiple of an eighth of n's octave (at most 12.5%
  // padding); never above max_batch.
  uint32_t padded(uint32_t n) const {
    uint32_t b = 1;
    while (b < n && b < 16) b <<= 1;
    if (n > 16) {
      uint32_t oct = 16;  // oct < n <= 2 oct
      while (2 * oct < n) oct <<= 1;
      const uint32_t step = oct / 8;
      b = (n + step - 1) / step * step;
    }
    return std::min(b, max_batch);
  }

  // The slot's captured search for (k, nb), captured now if it is not yet;
  // null with *err set on failure. Only the thread that owns the slot (the
  // dispatcher, or the constructor before it starts) calls this.
  void *graph_for(Slot &s, uint32_t k, uint32_t nb, std::string *err) {
    const uint64_t key = (uint64_t(k) << 32) | nb;
    auto it = s.graph.find(key);
    if (it != s.graph.end()) return it->second;
    if (batch_bytes(nb, k) > slot_bytes) {
      *err = "server: a batch of " + std::to_string(nb) + " at k " + std::to_string(k) +
             " needs more device memory than a slot holds";
      return nullptr;
    }
    const Layout L = layout(pool.at(s.base), nb, k);
    void *g = nullptr;
    if (katoann_gpu_search_capture(view, L.dq, nb, k, opt.nprobe, rk, opt.survivors, nb, nullptr,
                                   use_model ? &model : nullptr, L.ws, L.ws_bytes, L.dids, L.dd,
                                   L.dnp, reinterpret_cast<katoann_stream_t>(s.stream), &g)) {
      *err = std::string("search graph: ") + katoann_gpu_last_error();
      return nullptr;
    }
    s.graph.emplace(key, g);
    {
      std::lock_guard<std::mutex> lk(mu);
      ++graphs_captured;
    }
    return g;
  }

  // the oldest waiting request's class, or 0
  uint32_t oldest_class() const {
    uint32_t k = 0;
    Clock::time_point t{};
    for (const auto &w : waiting)
      if (!w.second.empty() && (k == 0 || w.second.front().t < t)) {
        k = w.first;
        t = w.second.front().t;
      }
    return k;
  }

  Slot *free_slot() {
    for (auto &s : slots)
      if (!s.busy) return &s;
    return nullptr;
  }

  void launch(Batch &b) {
    const auto h0 = Clock::now();
    struct Timed {  // enqueue time on every return path
      Batch &b;
      Clock::time_point h0;
      ~Timed() { b.enqueue_ms = std::chrono::duration<double, std::milli>(Clock::now() - h0).count(); }
    } timed{b, h0};
    Slot &s = *b.slot;
    const uint32_t n = b.n, k = b.k, nb = graphs ? padded(n) : n;
    for (uint32_t i = 0; i < n; ++i)
      std::memcpy(s.hq + size_t(i) * dim, b.reqs[i].q.data(), size_t(dim) * 4);
    // padding: the batch's own queries again, in turn, so that no query is
    // repeated more than once (thousands of copies of one query would crowd
    // its lists and the candidate records of the CTAs that scan them)
    for (uint32_t i = n; i < nb; ++i)
      std::memcpy(s.hq + size_t(i) * dim, s.hq + size_t(i % n) * dim, size_t(dim) * 4);
    const Layout L = layout(pool.at(graphs ? s.base : b.off), nb, k);
    const auto st = reinterpret_cast<katoann_stream_t>(s.stream);
    void *g = nullptr;
    if (graphs && !(g = graph_for(s, k, nb, &b.err))) return;
    cudaError_t e = cudaEventRecord(s.start, s.stream);
    if (e != cudaSuccess) {
      b.err = std::string("cudaEventRecord: ") + cudaGetErrorString(e);
      return;
    }
    e = cudaMemcpyAsync(L.dq, s.hq, size_t(nb) * dim * 4, cudaMemcpyHostToDevice, s.stream);
    if (e != cudaSuccess) {
      b.err = std::string("copy queries: ") + cudaGetErrorString(e);
      return;
    }
    const int rc = g ? katoann_gpu_graph_launch(g, st)
                     : katoann_gpu_search_budget(view, L.dq, n, k, opt.nprobe, rk, opt.survivors, n,
                                                 nullptr, use_model ? &model : nullptr, L.ws,
                                                 L.ws_bytes, L.dids, L.dd, L.dnp, st, nullptr);
    if (rc) {
      b.err = katoann_gpu_last_error();
      return;
    }
    b.graph = g != nullptr;
    cudaMemcpyAsync(s.hids, L.dids, size_t(n) * k * 4, cudaMemcpyDeviceToHost, s.stream);
    cudaMemcpyAsync(s.hd, L.dd, size_t(n) * k * 4, cudaMemcpyDeviceToHost, s.stream);
    cudaMemcpyAsync(s.hnp, L.dnp, size_t(n) * 4, cudaMemcpyDeviceToHost, s.stream);
    e = cudaEventRecord(s.event, s.stream);
    if (e != cudaSuccess) b.err = std::string("cudaEventRecord: ") + cudaGetErrorString(e);
  }

  void dispatch_loop() {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      // a stopping server still dispatches everything submitted
      cv_dispatch.wait(lk, [&] { return (pending > 0 && free_slot()) || (stop && pending == 0); });
      if (pending == 0) return;
      const uint32_t k = oldest_class();
      auto &q = waiting[k];
      // a partial batch may wait a little for company while the device is busy
      if (opt.max_wait_ms > 0 && in_flight > 0 && q.size() < max_batch && !stop) {
        const auto due = q.front().t + std::chrono::duration<double, std::milli>(opt.max_wait_ms);
        if (Clock::now() < due) {
          cv_dispatch.wait_until(lk, due);
          continue;
        }
      }
      uint32_t n = static_cast<uint32_t>(std::min<size_t>(q.size(), max_batch));
      size_t bytes = graphs ? 0 : batch_bytes(n, k);
      size_t off = graphs ? free_slot()->base : pool.take(bytes);
      if (off == SIZE_MAX) {
        if (in_flight > 0) {  // wait for memory to come back
          cv_dispatch.wait(lk);
          continue;
        }
        // nothing in flight: the largest batch that fits
        const size_t room = pool.largest();
        uint32_t lo = 0, hi = n;
        while (lo < hi) {
          const uint32_t mid = (lo + hi + 1) / 2;
          if (batch_bytes(mid, k) <= room) lo = mid;
          else hi = mid - 1;
        }
        n = lo;
        if (n == 0) {  // not even one query fits: fail the request
          Request r = std::move(q.front());
          q.pop_front();
          --pending;
          Entry &en = entries[r.id];
          en.done = true;
          en.err = "the HBM budget holds no batch of one query";
          cv_done.notify_all();
          continue;
        }
        bytes = batch_bytes(n, k);
        off = pool.take(bytes);
      }
      Batch b{free_slot(), k, n, off, bytes, {}, {}, 0, false};
      b.slot->busy = true;
      b.reqs.reserve(n);
      for (uint32_t i = 0; i < n; ++i) {
        b.reqs.push_back(std::move(q.front()));
        q.pop_front();
      }
      pending -= n;
      ++in_flight;
      peak_in_flight = std::max(peak_in_flight, in_flight);
      ++nbatches;
      batched += n;
      lk.unlock();
      launch(b);  // no lock held while the host copies and enqueues
      lk.lock();
      max_enqueue_ms = std::max(max_enqueue_ms, b.enqueue_ms);
      graph_batches += b.graph ? 1 : 0;
      launched.push_back(std::move(b));
      cv_complete.notify_one();
    }
  }

  void complete_loop() {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      cv_complete.wait(lk, [&] {
        return !launched.empty() || (stop && pending == 0 && in_flight == 0);
      });
      if (launched.empty()) return;
      Batch b = std::move(launched.front());
      launched.pop_front();
      lk.unlock();
      std::string err = b.err;
      float gpu_ms = 0;
      if (err.empty()) {
        const cudaError_t e = cudaEventSynchronize(b.slot->event);
        if (e != cudaSuccess) err = std::string("search: ") + cudaGetErrorString(e);
        else if (cudaEventElapsedTime(&gpu_ms, b.slot->start, b.slot->event) != cudaSuccess)
          gpu_ms = 0;
      } else {
        cudaStreamSynchronize(b.slot->stream);  // whatever was enqueued before the failure
      }
      const auto now = Clock::now();
      std::vector<ServerResult> res(b.n);
      if (err.empty())
        for (uint32_t i = 0; i < b.n; ++i) {
          ServerResult &r = res[i];
          r.ids.assign(b.slot->hids + size_t(i) * b.k, b.slot->hids + size_t(i + 1) * b.k);
          r.dists.assign(b.slot->hd + size_t(i) * b.k, b.slot->hd + size_t(i + 1) * b.k);
          r.nprobe = b.slot->hnp[i];
          r.latency_ms = std::chrono::duration<double, std::milli>(now - b.reqs[i].t).count();
        }
      lk.lock();
      for (uint32_t i = 0; i < b.n; ++i) {
        Entry &en = entries[b.reqs[i].id];
        en.done = true;
        en.err = err;
        en.res = std::move(res[i]);
      }
      if (b.bytes) pool.give(b.off, b.bytes);
      max_batch_gpu_ms = std::max(max_batch_gpu_ms, static_cast<double>(gpu_ms));
      b.slot->busy = false;
      --in_flight;
      cv_done.notify_all();
      cv_dispatch.notify_one();
    }
  }
};

Server::Server(const Index &index, const ServerOptions &opt) : m_(new Impl) {
  Impl &m = *m_;
  if (index.nlist() == 0) throw std::logic_error("server before load");
  if (opt.max_batch == 0 || opt.max_batch > 4096)
    throw std::invalid_argument("server: max_batch must be 1 to 4096");
  if (opt.max_in_flight == 0 || opt.max_in_flight > 16)
    throw std::invalid_argument("server: max_in_flight must be 1 to 16");
  if (opt.max_k == 0 || opt.max_k > 4096) throw std::invalid_argument("server: max_k must be 1 to 4096");
  if (opt.nprobe == 0 || opt.nprobe > index.nlist())
    throw std::invalid_argument("need 1 <= nprobe <= nlist");
  if (opt.ranking == Ranking::kPrefix && index.prefix_dims() == 0)
    throw std::invalid_argument("prefix ranking needs the rotation file (.dimc)");
  m.opt = opt;
  m.view = static_cast<const katoann_gpu_index *>(index.device_view());
  m.dim = index.dim();
  m.max_batch = opt.max_batch;
  m.rk = opt.ranking == Ranking::kFull ? KATO_RANK_FULL
         : opt.ranking == Ranking::kHighBytes ? KATO_RANK_HIGH
                                              : KATO_RANK_PREFIX;
  m.depth = opt.nprobe;
  if (opt.budget) {
    opt.budget->device_model(opt.budget_threshold, &m.model);
    m.use_model = true;
    m.depth = std::max(m.depth, m.model.depth);
    if (m.depth > index.nlist()) throw std::invalid_argument("the probe model's depth exceeds nlist");
  }
  const size_t full = m.batch_bytes(m.max_batch, opt.max_k);
  if (full == 0) throw std::invalid_argument(katoann_gpu_last_error());
  const size_t budget = opt.hbm_budget ? opt.hbm_budget : align256(full) * opt.max_in_flight;
  m.pool.init(budget);
  m.graphs = opt.graphs && budget >= align256(full) * opt.max_in_flight;
  m.slot_bytes = full;
  m.slots.resize(opt.max_in_flight);
  for (Slot &s : m.slots) {
    cuda_check(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking), "server stream");
    cuda_check(cudaEventCreate(&s.start), "server event");
    cuda_check(cudaEventCreateWithFlags(&s.event, cudaEventBlockingSync), "server event");
    cuda_check(cudaMallocHost(&s.hq, size_t(m.max_batch) * m.dim * 4), "server pinned queries");
    cuda_check(cudaMallocHost(&s.hids, size_t(m.max_batch) * opt.max_k * 4), "server pinned ids");
    cuda_check(cudaMallocHost(&s.hd, size_t(m.max_batch) * opt.max_k * 4), "server pinned dists");
    cuda_check(cudaMallocHost(&s.hnp, size_t(m.max_batch) * 4), "server pinned nprobe");
    if (m.graphs) s.base = m.pool.take(full);  // the slot's for good
  }
  if (m.graphs)
    for (const uint32_t k : opt.warm_k) {
      if (k == 0 || k > opt.max_k) throw std::invalid_argument("server: warm k must be 1 to max_k");
      for (Slot &s : m.slots)
        for (uint32_t n = 1, last = 0; n <= m.max_batch; ++n) {
          const uint32_t nb = m.padded(n);
          if (nb == last) continue;
          last = nb;
          std::string err;
          if (!m.graph_for(s, k, nb, &err)) throw std::runtime_error(err);
        }
    }
  m.dispatcher = std::thread([&m] { m.dispatch_loop(); });
  m.completer = std::thread([&m] { m.complete_loop(); });
}

Server::~Server() {
  Impl &m = *m_;
  {
    std::lock_guard<std::mutex> lk(m.mu);
    m.stop = true;
  }
  m.cv_dispatch.notify_all();
  if (m.dispatcher.joinable()) m.dispatcher.join();
  m.cv_complete.notify_all();
  if (m.completer.joinable()) m.completer.join();
  for (Slot &s : m.slots) {
    for (auto &g : s.graph) katoann_gpu_graph_destroy(g.second);
    if (s.event) cudaEventDestroy(s.event);
    if (s.start) cudaEventDestroy(s.start);
    if (s.stream) cudaStreamDestroy(s.stream);
    if (s.hq) cudaFreeHost(s.hq);
    if (s.hids) cudaFreeHost(s.hids);
    if (s.hd) cudaFreeHost(s.hd);
    if (s.hnp) cudaFreeHost(s.hnp);
  }
}

uint64_t Server::submit(const float *query, uint32_t k) {
  Impl &m = *m_;
  if (k == 0 || k > m.opt.max_k) throw std::invalid_argument("server: k must be 1 to max_k");
  Request r{0, std::vector<float>(query, query + m.dim), Clock::now()};
  std::lock_guard<std::mutex> lk(m.mu);
  if (m.stop) throw std::logic_error("server is stopping");
  r.id = m.next_id++;
  m.entries[r.id];
  m.waiting[k].push_back(std::move(r));
  ++m.pending;
  ++m.submitted;
  m.cv_dispatch.notify_one();
  return m.next_id - 1;
}

namespace {
bool take_result(std::unordered_map<uint64_t, Entry> &entries, uint64_t id, ServerResult *out) {
  auto it = entries.find(id);
  if (it == entries.end()) throw std::invalid_argument("unknown request id");
  if (!it->second.done) return false;
  const std::string err = it->second.err;
  if (out) *out = std::move(it->second.res);
  entries.erase(it);
  if (!err.empty()) throw std::runtime_error(err);
  return true;
}
}  // namespace

bool Server::poll(uint64_t id, ServerResult *out) {
  std::lock_guard<std::mutex> lk(m_->mu);
  return take_result(m_->entries, id, out);
}

ServerResult Server::wait(uint64_t id) {
  Impl &m = *m_;
  std::unique_lock<std::mutex> lk(m.mu);
  ServerResult r;
  m.cv_done.wait(lk, [&] {
    auto it = m.entries.find(id);
    return it == m.entries.end() || it->second.done;
  });
  if (!take_result(m.entries, id, &r)) throw std::logic_error("request not done");
  return r;
}

void Server::drain() {
  Impl &m = *m_;
  std::unique_lock<std::mutex> lk(m.mu);
  m.cv_done.wait(lk, [&] { return m.pending == 0 && m.in_flight == 0; });
}

LoadReport run_load(Server &server, const float *queries, uint32_t dim,
                    const std::vector<uint32_t> &pool, double rate, uint32_t n,
                    const std::vector<uint32_t> &kmix, uint64_t seed) {
  if (pool.empty() || kmix.empty() || n == 0 || !(rate > 0))
    throw std::invalid_argument("load: need queries, a k, requests and a positive rate");
  std::mt19937_64 rng(seed);
  std::exponential_distribution<double> gap(rate);
  std::vector<double> arrival(n), lag(n);
  std::vector<uint32_t> which(n), kof(n);
  double t = 0;
  for (uint32_t i = 0; i < n; ++i) {
    t += gap(rng);
    arrival[i] = t;
    which[i] = pool[i % pool.size()];
    kof[i] = kmix[rng() % kmix.size()];
  }
  const ServerStats before = server.stats();
  server.reset_peaks();
  std::vector<uint64_t> rid(n);
  const auto start = Clock::now();
  auto since = [&] { return std::chrono::duration<double>(Clock::now() - start).count(); };
  std::thread client([&] {
    for (uint32_t i = 0; i < n; ++i) {
      const double now = since();
      if (arrival[i] > now) std::this_thread::sleep_for(std::chrono::duration<double>(arrival[i] - now));
      lag[i] = std::max(0.0, since() - arrival[i]);
      rid[i] = server.submit(queries + static_cast<size_t>(which[i]) * dim, kof[i]);
    }
  });
  client.join();
  std::vector<double> lat(n);
  double probes = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const ServerResult r = server.wait(rid[i]);
    lat[i] = lag[i] * 1e3 + r.latency_ms;
    probes += r.nprobe;
  }
  const double span = since();
  const ServerStats st = server.stats();
  std::sort(lat.begin(), lat.end());
  auto pct = [&](double f) {
    const size_t r = static_cast<size_t>(std::ceil(f * lat.size()));
    return lat[std::min(lat.size() - 1, r ? r - 1 : 0)];
  };
  LoadReport rep;
  rep.requests = n;
  rep.achieved_qps = n / span;
  rep.p50_ms = pct(0.50);
  rep.p95_ms = pct(0.95);
  rep.p99_ms = pct(0.99);
  rep.max_ms = lat.back();
  rep.batches = st.batches - before.batches;
  rep.mean_batch = rep.batches ? double(n) / double(rep.batches) : 0;
  rep.mean_nprobe = probes / n;
  rep.peak_in_flight = st.peak_in_flight;
  rep.peak_hbm_bytes = st.peak_hbm_bytes;
  rep.max_lag_ms = *std::max_element(lag.begin(), lag.end()) * 1e3;
  rep.max_enqueue_ms = st.max_enqueue_ms;
  rep.max_batch_gpu_ms = st.max_batch_gpu_ms;
  return rep;
}

ServerStats Server::stats() const {
  const Impl &m = *m_;
  std::lock_guard<std::mutex> lk(m.mu);
  ServerStats s;
  s.requests = m.submitted;
  s.batches = m.nbatches;
  s.peak_in_flight = m.peak_in_flight;
  s.peak_hbm_bytes = m.pool.peak();
  s.mean_batch = m.nbatches ? double(m.batched) / double(m.nbatches) : 0;
  s.max_enqueue_ms = m.max_enqueue_ms;
  s.max_batch_gpu_ms = m.max_batch_gpu_ms;
  s.graph_batches = m.graph_batches;
  s.graphs = m.graphs_captured;
  return s;
}

void Server::reset_peaks() {
  Impl &m = *m_;
  std::lock_guard<std::mutex> lk(m.mu);
  m.peak_in_flight = m.in_flight;
  m.pool.reset_peak();
  m.max_enqueue_ms = 0;
  m.max_batch_gpu_ms = 0;
}

}  // namespace katoann
