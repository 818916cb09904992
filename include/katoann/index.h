// katoann::Index on one GB300: the reference's build / load / search API
// (include/katoann/index.h of KatoANN) with the search running as sm_103a
// kernels through libkatoann_gpu.so (include/katoann_gpu.h).
//
// Same option structs, same enums, same file format, same exceptions:
//   std::invalid_argument  bad k / nprobe / prefix_dims / dimension / nlist
//   std::runtime_error     unreadable or inconsistent index files, CUDA errors
//   std::logic_error       search before load
// Differences, all additive: Engine gains kGpu (what engine() reports);
// load_arrays() loads an index from memory (host or device) instead of files;
// search_device() searches device-resident queries into device outputs on a
// caller stream; memory_bytes() counts device memory too.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace katoann {

// The reference's engines are CPU matrix engines; this build has one engine.
enum class Engine { kAmx, kAvx512, kGpu };

// Always false here: no CPU matrix engine is used (reference: kernels.h:174-175).
bool amx_available();

constexpr uint32_t kMaxDim = 4096;

struct BuildOptions {
  uint32_t nlist = 2048;
  uint32_t train_size = 256000;
  uint32_t kmeans_iters = 12;
  uint64_t seed = 0;            // k-means++ seed; 0 picks a random seed
  bool normalized = false;      // record that the vectors are unit-length
  uint32_t rotation_sample = 100000;
  uint32_t jacobi_sweeps = 8;
};

enum class Precision {
  kSq16,  // 16-bit codes in high and low byte planes (default)
  kBf16,  // the reference's bfloat16 comparison mode; not part of the GPU path
};

struct LoadOptions {
  Precision precision = Precision::kSq16;
  bool use_amx = true;          // accepted and ignored (no CPU engine)
  uint32_t prefix_dims = 0;     // dimensions of the prefix ranking pass;
                                // 0 takes the value stored in P.dimc
  bool batched_coarse = true;   // coarse search as one matrix product per batch
  uint32_t max_batch = 4096;    // queries per device pass (workspace size)
  // Use the device-code cache P.gpucodes (see Index::save_codes): load from it
  // when it was made from the same index files with the same prefix_dims,
  // otherwise load the files and write it.
  bool code_cache = false;
};

enum class Ranking {
  kFull,       // exact distance of every candidate
  kHighBytes,  // rank by the high bytes, refine the survivors exactly
  kPrefix,     // rank by the high bytes of the leading rotated dimensions
};

enum class Selection {
  kThreshold,  // one running top-S per query
  kLocal,      // a top-S per (query, list), merged after the scan
};

class ProbeModel;  // include/katoann/probe.h

struct SearchParams {
  uint32_t k = 10;
  uint32_t nprobe = 64;
  Ranking ranking = Ranking::kPrefix;
  uint32_t survivors = 32;      // candidates refined per query (at least k)
  Selection selection = Selection::kThreshold;
  // Additions: a per-query nprobe, capped at nprobe. Either given
  // (nprobe_per_query, nq values) or chosen by a learned model (budget, with
  // its cumulative-probability threshold); nprobe_used receives every query's
  // nprobe. Host memory in search(), device memory in search_device().
  const ProbeModel *budget = nullptr;
  float budget_threshold = 0.95f;
  const uint32_t *nprobe_per_query = nullptr;
  uint32_t *nprobe_used = nullptr;
  // Run the search's kernels as a CUDA graph, captured the first time these
  // pointers and parameters are seen (the index keeps the last 16) and
  // replayed in one launch after that. search_device captures the whole
  // call; search captures each pass on the index's own device buffers and
  // keeps the copies of the queries and results outside the graph.
  bool graph = false;
};

// An index given as arrays (lists concatenated in list order). Pointers are
// host memory, or device memory when on_device is true.
struct IndexArrays {
  uint32_t dim = 0, nlist = 0, npts = 0;
  bool normalized = false;
  const float *centroids = nullptr;    // nlist x dim, unrotated
  const uint32_t *list_sizes = nullptr;  // nlist (always host memory)
  const uint32_t *ids = nullptr;       // npts
  const float *vectors = nullptr;      // npts x dim, unrotated
  const float *rotation = nullptr;     // dim x dim (row j = basis j), or null
  bool has_dimc = false;               // a P.dimc exists (rotation and/or head dims)
  uint32_t head_dims = 0;              // head dims stored in P.dimc
  bool on_device = false;
};

// A partition as Index::build computes it, before any file is written.
struct BuildResult {
  std::vector<float> centroids;  // nlist x dim
  std::vector<uint32_t> assign;  // per vector: its list
  std::vector<float> rotation;   // dim x dim (row j = basis j); empty without one
  uint32_t head_dims = 0;        // the default prefix dims (src/index.cpp:512)
};

// A search whose device pipeline gave up on a bounded wait (no counterpart in
// the reference, which has no device): the kernel returned early and the
// results are incomplete; the index stays usable.
struct timeout_error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// min(max(64, round_up(dim / 4, 64)), dim rounded up to 64).
uint32_t default_head_dims(uint32_t dim);

class Index {
 public:
  Index();
  ~Index();
  Index(const Index &) = delete;
  Index &operator=(const Index &) = delete;
  Index(Index &&) noexcept;
  Index &operator=(Index &&) noexcept;

  // Partitions data (n x dim, row-major) with k-means, writes the index files,
  // and computes the rotation for the prefix ranking pass.
  static void build(const float *data, uint32_t n, uint32_t dim, const BuildOptions &opt,
                    const std::string &prefix);
  // The same partition, on the GPU, without writing files (data may be
  // device memory): k-means on a strided training sample, every vector's
  // list, and the PCA rotation with the default head dims.
  static BuildResult partition(const float *data, uint32_t n, uint32_t dim, const BuildOptions &opt,
                               bool on_device = false);

  void load(const std::string &prefix, const LoadOptions &opt = {});
  void load_arrays(const IndexArrays &a, const LoadOptions &opt = {});

  // The device-code cache (no counterpart in the reference): the loaded
  // index as it lives on the device - codes, norms, ids, list offsets,
  // centroid planes, rotation and scale - in one file, so that a later load
  // skips reading the float vectors and coding them (for 10M x 1024, 41 GB
  // of floats against 21 GB of codes). The file records which index files it
  // was made from (sizes and content hashes) when it came from load().
  void save_codes(const std::string &path) const;
  void load_codes(const std::string &path, const LoadOptions &opt = {});

  // Searches nq queries (host memory) together. ids and dists (host memory)
  // are nq x k, nearest first.
  void search(const float *queries, uint32_t nq, const SearchParams &p, uint32_t *ids,
              float *dists) const;

  // The same with device pointers on `stream` (a cudaStream_t; nullptr = the
  // index's own stream). Returns without synchronising.
  // `timer` (from katoann_gpu_timer_create, may be null) records the phase
  // events of every device pass.
  void search_device(const float *d_queries, uint32_t nq, const SearchParams &p, uint32_t *d_ids,
                     float *d_dists, void *stream = nullptr, void *timer = nullptr) const;

  uint32_t dim() const;
  uint32_t nlist() const;
  uint32_t size() const;
  bool normalized() const;
  Engine engine() const { return Engine::kGpu; }
  Precision precision() const { return Precision::kSq16; }
  uint32_t prefix_dims() const;
  bool rotated() const;
  bool batched_coarse() const;
  std::vector<uint32_t> list_sizes() const;
  size_t memory_bytes() const;

  // The autotuner (no counterpart in the reference): times a search of these
  // queries (host; the first max_batch of them) with `p` under every
  // candidate setting of the ranking pass's knobs and keeps the fastest for
  // the process (katoann_gpu_autotune). Results never depend on the knobs.
  struct Tuning {
    uint32_t seed_rows, schedule, width;
    double us_per_search;
  };
  Tuning autotune(const float *queries, uint32_t nq, const SearchParams &p);

  // Diagnostics of the last search: coarse boundary ties, survivor boundary
  // ties, queries (see katoann_gpu_workspace_stats).
  std::vector<uint64_t> last_search_stats() const;
  // The device view handed to the kernels (const katoann_gpu_index *).
  const void *device_view() const;

 private:
  struct State;
  static void set_view(State &s);
  void load_files(const std::string &prefix, const LoadOptions &opt);
  std::unique_ptr<State> s_;
};

// Scales each row to unit length as the reference's CLI and Python module do
// before searching a normalized index (tools/katoann.cpp:102-111).
void normalize_rows(float *rows, size_t n, uint32_t dim);

}  // namespace katoann
