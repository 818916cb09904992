// Continuous-batching search server over one katoann::Index (no counterpart
// in the reference, whose `katoann load` runs one batch at a time and blocks
// until it is done: tools/katoann.cpp:304-321).
//
// Requests (one query each, with its own k) are submitted from any thread.
// A dispatcher forms batches from the waiting requests of one k, oldest
// first, whenever a slot is free and the batch's device memory fits in the
// HBM budget; each batch runs on its own CUDA stream with its own workspace,
// so batches that arrive while others are on the device overlap with them
// (copies, kernels and host work). A completion thread finishes requests in
// the order their batches were launched. Every query's result is the one a
// search of that query alone gives: nothing in the pipeline mixes queries.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>

#include "katoann/index.h"

namespace katoann {

struct ServerOptions {
  uint32_t max_batch = 4096;      // queries per batch (at most the index's max_batch)
  uint32_t max_in_flight = 3;     // batches on the device at once
  size_t hbm_budget = 0;          // bytes of device memory for in-flight batches;
                                  // 0: room for max_in_flight batches of max_batch at max_k
  uint32_t max_k = 128;           // largest k a request may ask for
  uint32_t nprobe = 64;           // nprobe, or the cap of a learned budget
  Ranking ranking = Ranking::kPrefix;
  uint32_t survivors = 32;
  const ProbeModel *budget = nullptr;  // learned per-query nprobe (null: fixed)
  float budget_threshold = 0.95f;
  double max_wait_ms = 0;         // a partial batch waits this long for more requests
  // Replay captured CUDA graphs: each slot owns a full batch's device memory
  // and keeps one captured search per (k, padded batch size: the next power
  // of two up to 16, above that the next multiple of an eighth of the size's
  // octave), captured on first use; a batch's queries are padded to that
  // size with its own queries again. Enqueuing a batch is then one graph
  // launch and four copies. Needs an HBM budget of max_in_flight full batches
  // (the default); with less, batches are carved from the pool and launched
  // kernel by kernel.
  bool graphs = true;
  std::vector<uint32_t> warm_k;   // k whose graphs are captured for every slot and size up front
};

struct ServerResult {
  std::vector<uint32_t> ids;      // k, nearest first
  std::vector<float> dists;
  uint32_t nprobe = 0;            // lists the query probed
  double latency_ms = 0;          // from submit to completion
};

struct ServerStats {
  uint64_t requests = 0, batches = 0;
  uint32_t peak_in_flight = 0;
  size_t peak_hbm_bytes = 0;      // device memory held by in-flight batches at most
  double mean_batch = 0;
  // where a batch's time goes, at most (since construction or reset_peaks):
  double max_enqueue_ms = 0;      // host: staging the queries and enqueuing copies and kernels
  double max_batch_gpu_ms = 0;    // device: the batch's copies and search, on its stream
  uint64_t graph_batches = 0;     // batches run as a graph replay
  uint32_t graphs = 0;            // graphs captured
};

struct LoadReport {
  uint32_t requests = 0;
  double achieved_qps = 0, p50_ms = 0, p95_ms = 0, p99_ms = 0, max_ms = 0;
  uint64_t batches = 0;
  double mean_batch = 0, mean_nprobe = 0;
  uint32_t peak_in_flight = 0;
  size_t peak_hbm_bytes = 0;
  // a latency outlier's source: the client behind its schedule, a slow host
  // enqueue, or a slow batch on the device (this run's maxima)
  double max_lag_ms = 0, max_enqueue_ms = 0, max_batch_gpu_ms = 0;
};

class Server;

// A Poisson stream of n requests at `rate` per second through `server`: each
// takes a query from `pool` (indices into queries, nq x dim; round-robin) and
// a k drawn uniformly from kmix, and is submitted at its arrival time by a
// native client thread. Latency runs from the scheduled arrival to
// completion (the reference's `katoann load` measure, tools/katoann.cpp:
// 317-327). Returns after every request is done.
LoadReport run_load(Server &server, const float *queries, uint32_t dim,
                    const std::vector<uint32_t> &pool, double rate, uint32_t n,
                    const std::vector<uint32_t> &kmix, uint64_t seed);

class Server {
 public:
  Server(const Index &index, const ServerOptions &opt = {});
  ~Server();  // finishes every submitted request
  Server(const Server &) = delete;
  Server &operator=(const Server &) = delete;

  // Copies the query (dim floats; normalized by the caller like Index::search)
  // and queues it; returns its id. Thread-safe.
  uint64_t submit(const float *query, uint32_t k);
  // The result once the request is done (true), or false at once.
  bool poll(uint64_t id, ServerResult *out);
  // Blocks until the request is done.
  ServerResult wait(uint64_t id);
  // Blocks until every submitted request is done.
  void drain();
  ServerStats stats() const;
  // Restarts the maxima of stats(): in-flight batches and device memory (from
  // their current values), enqueue and batch times (from zero).
  void reset_peaks();

  struct Impl;

 private:
  std::unique_ptr<Impl> m_;
};

}  // namespace katoann
