// Host side of katoann::Index: reads the reference's index files, uploads
// them, codes them on the GPU and runs searches through libkatoann_gpu.so.
//
// Load follows Index::load (src/index.cpp:777-807): read .meta / .centroids /
// .invlist / .dimc (:550-611), rotate the lists (:613-629), one global 16-bit
// scale from the min and max rotated value (:632-650), codes and norms
// (:656-689), head norms over the prefix dims (:694-715) and the centroid
// planes coded with the database scale (:718-750) - all of it on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <fstream>
#include <mutex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "katoann/index.h"
#include "katoann/probe.h"
#include "katoann_gpu.h"

namespace katoann {

namespace {

constexpr uint32_t kDimcMagic = 0x434D4944u;  // "DIMC"

void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

void gpu_check(int rc) {
  if (rc == KATO_OK) return;
  const std::string msg = katoann_gpu_last_error();
  if (rc == KATO_EINVAL) throw std::invalid_argument(msg);
  if (rc == KATO_ELOGIC) throw std::logic_error(msg);
  throw std::runtime_error(msg);
}

uint32_t round_up(uint32_t x, uint32_t m) { return (x + m - 1) / m * m; }

struct DevBuf {
  void *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { reset(); }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t bytes) {
    reset();
    if (bytes == 0) bytes = 256;
    cuda_check(cudaMalloc(&p, bytes), "cudaMalloc");
    n = bytes;
  }
  void ensure(size_t bytes) {
    if (bytes > n) alloc(bytes);
  }
  template <class T>
  T *as() const {
    return static_cast<T *>(p);
  }
};

}  // namespace

struct Index::State {
  uint32_t dim = 0, nlist = 0, npts = 0, dc = 0, head = 0, max_list = 0, max_batch = 4096;
  bool normalized = false, rotated = false;
  float lo = 0;
  double inv_step = 0, step = 0, step_sq = 0;
  std::vector<uint32_t> sizes;
  uint64_t source[4] = {0, 0, 0, 0};  // the index files the codes came from (code cache)
  uint32_t req_prefix = 0;            // the prefix_dims the load was asked for
  DevBuf rot, hi, lop, norm, hinorm, headnorm, ids, list_off, chi, clo, cnorm, chi16, clo16, cterm;
  DevBuf rot_t;  // the rotation in the k-major layout the query rotation reads (made at load)
  katoann_gpu_index view{};
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  mutable std::mutex mu;
  mutable DevBuf ws, dq, dids, ddists, dnp_in, dnp_out;
  // captured searches of search_device (SearchParams::graph), most recent last
  struct Graph {
    std::vector<uint64_t> key;
    void *handle;
  };
  mutable std::vector<Graph> graphs;
  void drop_graphs() const {
    for (auto &g : graphs) katoann_gpu_graph_destroy(g.handle);
    graphs.clear();
  }
  // The captured search of these device buffers and parameters (every
  // pointer and size the capture bakes in; model: the device probe model or
  // null), captured now if it is not yet. At most 16 are kept, the least
  // recently used dropped first. The caller holds mu.
  void *graph_of(const float *d_queries, uint32_t nq, const SearchParams &p, int rk,
                 const katoann_gpu_probe_model *model, uint32_t *d_ids, float *d_dists,
                 const uint32_t *d_npin, uint32_t *d_npout, cudaStream_t st) const {
    const std::vector<uint64_t> key = {
        reinterpret_cast<uint64_t>(d_queries), nq, reinterpret_cast<uint64_t>(d_ids),
        reinterpret_cast<uint64_t>(d_dists), p.k, p.nprobe, static_cast<uint64_t>(rk),
        p.survivors, reinterpret_cast<uint64_t>(d_npin), reinterpret_cast<uint64_t>(d_npout),
        model ? reinterpret_cast<uint64_t>(model->d_w1) : 0,
        model ? (uint64_t(model->nclass) << 32 | model->depth) : 0,
        model ? static_cast<uint64_t>(std::llround(double(p.budget_threshold) * 1e9)) : 0,
        reinterpret_cast<uint64_t>(st), reinterpret_cast<uint64_t>(ws.p), ws.n};
    for (size_t i = 0; i < graphs.size(); ++i)
      if (graphs[i].key == key) {
        void *h = graphs[i].handle;
        std::rotate(graphs.begin() + i, graphs.begin() + i + 1, graphs.end());
        return h;
      }
    void *h = nullptr;
    gpu_check(katoann_gpu_search_capture(&view, d_queries, nq, p.k, p.nprobe, rk, p.survivors,
                                         max_batch, d_npin, model, ws.p, ws.n, d_ids, d_dists,
                                         d_npout, reinterpret_cast<katoann_stream_t>(st), &h));
    if (graphs.size() >= 16) {
      katoann_gpu_graph_destroy(graphs.front().handle);
      graphs.erase(graphs.begin());
    }
    graphs.push_back({key, h});
    return h;
  }
  mutable void *last_stream = nullptr;
  // per device pass of a host search: the pass's count of CTAs whose bounded
  // pipeline wait ran out (workspace statistic 3), copied back with the results
  mutable uint64_t *hwait = nullptr;
  mutable uint32_t hwait_n = 0;
  uint64_t *wait_counts(uint32_t passes) const {
    if (passes > hwait_n) {
      if (hwait) cudaFreeHost(hwait);
      hwait = nullptr;
      hwait_n = 0;
      cuda_check(cudaMallocHost(reinterpret_cast<void **>(&hwait), passes * sizeof(uint64_t)),
                 "cudaMallocHost");
      hwait_n = passes;
    }
    return hwait;
  }

  ~State() {
    if (hwait) cudaFreeHost(hwait);
    drop_graphs();
    if (done) cudaEventDestroy(done);
    if (stream) cudaStreamDestroy(stream);
  }
};

bool amx_available() { return false; }

void normalize_rows(float *v, size_t n, uint32_t d) {
  for (size_t i = 0; i < n; ++i) {
    float *r = v + i * d;
    double s = 0;
    for (uint32_t k = 0; k < d; ++k) s += static_cast<double>(r[k]) * r[k];
    if (s > 0) {
      const float inv = static_cast<float>(1.0 / std::sqrt(s));
      for (uint32_t k = 0; k < d; ++k) r[k] *= inv;
    }
  }
}

Index::Index() = default;
Index::~Index() = default;
Index::Index(Index &&) noexcept = default;
Index &Index::operator=(Index &&) noexcept = default;

// ------------------------------------------------------------ code cache
// File: a CodeHeader, then the arrays below in order, each as a uint64 byte
// count and the bytes.
namespace {

constexpr uint32_t kCodeMagic = 0x4443474Bu;  // "KGCD"
constexpr uint32_t kCodeVersion = 1;

struct CodeHeader {
  uint32_t magic, version, dim, nlist, npts, dc, head, max_list, rotated, normalized, req_prefix,
      pad;
  float lo, pad2;
  double inv_step, step, step_sq;
  uint64_t source[4];
};

uint64_t fnv1a(uint64_t h, const char *p, size_t n) {
  for (size_t i = 0; i < n; ++i) h = (h ^ static_cast<unsigned char>(p[i])) * 0x100000001B3ull;
  return h;
}

// Sizes and content hashes of the index files: .meta, .centroids and .dimc
// whole; .invlist by its size and its first and last MiB.
void file_signature(const std::string &prefix, uint64_t out[4]) {
  uint64_t h = 0xCBF29CE484222325ull, sizes = 0;
  std::vector<char> buf;
  for (const char *ext : {".meta", ".centroids", ".dimc", ".invlist"}) {
    std::ifstream f(prefix + ext, std::ios::binary | std::ios::ate);
    const uint64_t n = f ? static_cast<uint64_t>(f.tellg()) : 0;
    sizes = sizes * 0x9E3779B97F4A7C15ull + n + 1;
    if (!f || n == 0) continue;
    const bool whole = std::string(ext) != ".invlist";
    const uint64_t part = whole ? n : std::min<uint64_t>(n, 1u << 20);
    buf.resize(part);
    f.seekg(0);
    f.read(buf.data(), static_cast<std::streamsize>(part));
    h = fnv1a(h, buf.data(), part);
    if (!whole && n > part) {
      f.seekg(static_cast<std::streamoff>(n - part));
      f.read(buf.data(), static_cast<std::streamsize>(part));
      h = fnv1a(h, buf.data(), part);
    }
  }
  out[0] = sizes;
  out[1] = h;
  out[2] = out[3] = 0;
}

// Device <-> file through one pinned bounce buffer.
struct Pinned {
  void *p = nullptr;
  size_t n = 0;
  explicit Pinned(size_t bytes) : n(bytes) { cuda_check(cudaMallocHost(&p, bytes), "cudaMallocHost"); }
  ~Pinned() { cudaFreeHost(p); }
};

void put(std::ofstream &f, const void *dev, uint64_t bytes, Pinned &pin) {
  f.write(reinterpret_cast<const char *>(&bytes), 8);
  for (uint64_t o = 0; o < bytes; o += pin.n) {
    const size_t c = static_cast<size_t>(std::min<uint64_t>(pin.n, bytes - o));
    cuda_check(cudaMemcpy(pin.p, static_cast<const char *>(dev) + o, c, cudaMemcpyDeviceToHost), "save codes");
    f.write(static_cast<const char *>(pin.p), static_cast<std::streamsize>(c));
  }
  if (!f) throw std::runtime_error("cannot write the code cache");
}

void get(std::ifstream &f, DevBuf &b, uint64_t expect, Pinned &pin, const std::string &path) {
  uint64_t bytes = 0;
  f.read(reinterpret_cast<char *>(&bytes), 8);
  if (!f || bytes != expect) throw std::runtime_error("bad array in " + path);
  b.alloc(static_cast<size_t>(bytes));
  for (uint64_t o = 0; o < bytes; o += pin.n) {
    const size_t c = static_cast<size_t>(std::min<uint64_t>(pin.n, bytes - o));
    f.read(static_cast<char *>(pin.p), static_cast<std::streamsize>(c));
    if (!f) throw std::runtime_error("truncated " + path);
    cuda_check(cudaMemcpy(static_cast<char *>(b.p) + o, pin.p, c, cudaMemcpyHostToDevice), "load codes");
  }
}

}  // namespace

void Index::save_codes(const std::string &path) const {
  if (!s_) throw std::logic_error("save_codes before load");
  const State &s = *s_;
  cuda_check(cudaStreamSynchronize(s.stream), "save codes");
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f) throw std::runtime_error("cannot open " + path);
  CodeHeader h{};
  h.magic = kCodeMagic;
  h.version = kCodeVersion;
  h.dim = s.dim, h.nlist = s.nlist, h.npts = s.npts, h.dc = s.dc, h.head = s.head;
  h.max_list = s.max_list, h.rotated = s.rotated, h.normalized = s.normalized;
  h.req_prefix = s.req_prefix;
  h.lo = s.lo, h.inv_step = s.inv_step, h.step = s.step, h.step_sq = s.step_sq;
  std::memcpy(h.source, s.source, sizeof(h.source));
  f.write(reinterpret_cast<const char *>(&h), sizeof(h));
  const uint64_t L = s.nlist;
  f.write(reinterpret_cast<const char *>(s.sizes.data()), static_cast<std::streamsize>(L * 4));
  Pinned pin(64u << 20);
  const uint64_t n = s.npts, dc = s.dc;
  put(f, s.ids.p, n * 4, pin);
  put(f, s.hi.p, n * dc, pin);
  put(f, s.lop.p, n * dc, pin);
  put(f, s.norm.p, n * 8, pin);
  put(f, s.hinorm.p, n * 8, pin);
  if (s.head) put(f, s.headnorm.p, n * 8, pin);
  if (s.rotated) put(f, s.rot.p, static_cast<uint64_t>(s.dim) * s.dim * 4, pin);
  put(f, s.chi.p, L * dc, pin);
  put(f, s.clo.p, L * dc, pin);
  put(f, s.cnorm.p, L * 8, pin);
  put(f, s.chi16.p, L * dc * 2, pin);
  put(f, s.clo16.p, L * dc * 2, pin);
  put(f, s.cterm.p, L * 8, pin);
  f.flush();
  if (!f) throw std::runtime_error("cannot write " + path);
}

void Index::load_codes(const std::string &path, const LoadOptions &opt) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + path);
  CodeHeader h{};
  f.read(reinterpret_cast<char *>(&h), sizeof(h));
  if (!f || h.magic != kCodeMagic || h.version != kCodeVersion || h.dim == 0 || h.dim > kMaxDim ||
      h.nlist == 0 || h.dc != round_up(h.dim, 64u) || h.head > h.dc)
    throw std::runtime_error("bad header in " + path);
  s_.reset();
  auto st = std::make_unique<State>();
  State &s = *st;
  s.dim = h.dim, s.nlist = h.nlist, s.npts = h.npts, s.dc = h.dc, s.head = h.head;
  s.rotated = h.rotated != 0, s.normalized = h.normalized != 0, s.req_prefix = h.req_prefix;
  s.lo = h.lo, s.inv_step = h.inv_step, s.step = h.step, s.step_sq = h.step_sq;
  std::memcpy(s.source, h.source, sizeof(s.source));
  s.max_batch = std::max(1u, opt.max_batch);
  const uint64_t L = s.nlist, n = s.npts, dc = s.dc;
  s.sizes.assign(L, 0);
  f.read(reinterpret_cast<char *>(s.sizes.data()), static_cast<std::streamsize>(L * 4));
  if (!f) throw std::runtime_error("truncated " + path);
  std::vector<uint32_t> off(L + 1, 0);
  for (uint64_t c = 0; c < L; ++c) {
    off[c + 1] = off[c] + s.sizes[c];
    s.max_list = std::max(s.max_list, s.sizes[c]);
  }
  if (off[L] != n || s.max_list != h.max_list) throw std::runtime_error("bad list sizes in " + path);
  cuda_check(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking), "cudaStreamCreate");
  cuda_check(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming), "cudaEventCreate");
  s.list_off.alloc((L + 1) * 4);
  cuda_check(cudaMemcpy(s.list_off.p, off.data(), (L + 1) * 4, cudaMemcpyHostToDevice), "upload");
  Pinned pin(64u << 20);
  get(f, s.ids, n * 4, pin, path);
  get(f, s.hi, n * dc, pin, path);
  get(f, s.lop, n * dc, pin, path);
  get(f, s.norm, n * 8, pin, path);
  get(f, s.hinorm, n * 8, pin, path);
  if (s.head) get(f, s.headnorm, n * 8, pin, path);
  if (s.rotated) get(f, s.rot, static_cast<uint64_t>(s.dim) * s.dim * 4, pin, path);
  get(f, s.chi, L * dc, pin, path);
  get(f, s.clo, L * dc, pin, path);
  get(f, s.cnorm, L * 8, pin, path);
  get(f, s.chi16, L * dc * 2, pin, path);
  get(f, s.clo16, L * dc * 2, pin, path);
  get(f, s.cterm, L * 8, pin, path);
  set_view(s);
  s_ = std::move(st);
}

void Index::load(const std::string &prefix, const LoadOptions &opt) {
  uint64_t sig[4] = {0, 0, 0, 0};
  if (opt.code_cache) {
    file_signature(prefix, sig);
    const std::string path = prefix + ".gpucodes";
    std::ifstream f(path, std::ios::binary);
    CodeHeader h{};
    if (f && f.read(reinterpret_cast<char *>(&h), sizeof(h)) && h.magic == kCodeMagic &&
        h.version == kCodeVersion && std::memcmp(h.source, sig, sizeof(sig)) == 0 &&
        h.req_prefix == opt.prefix_dims && opt.precision == Precision::kSq16 && opt.batched_coarse) {
      f.close();
      load_codes(path, opt);
      return;
    }
  }
  load_files(prefix, opt);
  if (opt.code_cache) {
    std::memcpy(s_->source, sig, sizeof(sig));
    s_->req_prefix = opt.prefix_dims;
    try {
      save_codes(prefix + ".gpucodes");
    } catch (const std::runtime_error &) {
      std::remove((prefix + ".gpucodes").c_str());  // a read-only place: no cache, same index
    }
  }
}

namespace {

// One index file read front to back. take() fills its target completely or
// reports a short read; the file is closed with the reader.
class FileIn {
 public:
  explicit FileIn(std::string path) : path_(std::move(path)), f_(std::fopen(path_.c_str(), "rb")) {}
  ~FileIn() {
    if (f_) std::fclose(f_);
  }
  FileIn(const FileIn &) = delete;
  FileIn &operator=(const FileIn &) = delete;
  bool open() const { return f_ != nullptr; }
  const std::string &path() const { return path_; }
  template <typename T>
  bool take(T *dst, size_t count) {
    return count == 0 || std::fread(dst, sizeof(T), count, f_) == count;
  }
  // A file the index cannot do without: "cannot open <path>" if it is absent.
  FileIn &required() {
    if (!f_) throw std::runtime_error("cannot open " + path_);
    return *this;
  }

 private:
  std::string path_;
  FILE *f_;
};

}  // namespace

// The reference's index files (src/index.cpp:482-505 and :535-545 write them):
//   .meta       u32 dim, nlist, rows [, metric (0 = L2), normalized]
//   .centroids  nlist x dim f32
//   .invlist    per list: u32 size, size u32 ids, size x dim f32 vectors
//   .dimc       u32 magic, version, dim, nlist, rows, head dims, rotated, 0
//               [, dim x dim f32 rotation]  (optional file)
void Index::load_files(const std::string &prefix, const LoadOptions &opt) {
  IndexArrays a;
  std::vector<float> centroids, vectors, rotation;
  std::vector<uint32_t> sizes, ids;

  FileIn meta(prefix + ".meta");
  meta.required();
  uint32_t head[5] = {0, 0, 0, 0, 0};
  if (!meta.take(head, 3)) throw std::runtime_error("truncated " + meta.path());
  if (meta.take(head + 3, 2)) {  // the metric and normalization words came later
    if (head[3] != 0) throw std::runtime_error("only the L2 metric is supported");
    a.normalized = head[4] != 0;
  }
  a.dim = head[0];
  a.nlist = head[1];
  a.npts = head[2];
  if (a.dim == 0 || a.dim > kMaxDim || a.nlist == 0)
    throw std::runtime_error("bad header in " + meta.path());

  FileIn cen(prefix + ".centroids");
  centroids.resize(static_cast<size_t>(a.nlist) * a.dim);
  if (!cen.open() || !cen.take(centroids.data(), centroids.size()))
    throw std::runtime_error("cannot read " + cen.path());

  // lists in file order; the sizes must add up to the rows of .meta exactly
  FileIn inv(prefix + ".invlist");
  inv.required();
  sizes.assign(a.nlist, 0);
  ids.reserve(a.npts);
  vectors.reserve(static_cast<size_t>(a.npts) * a.dim);
  uint64_t rows = 0;
  bool whole = true;
  for (uint32_t c = 0; c < a.nlist && whole; ++c) {
    uint32_t n = 0;
    whole = inv.take(&n, 1) && rows + n <= a.npts;
    if (!whole) break;
    ids.resize(rows + n);
    vectors.resize((rows + n) * a.dim);
    whole = inv.take(ids.data() + rows, n) && inv.take(vectors.data() + rows * a.dim, size_t{n} * a.dim);
    sizes[c] = n;
    rows += n;
  }
  if (!whole || rows != a.npts) throw std::runtime_error("truncated " + inv.path());

  FileIn dimc(prefix + ".dimc");  // optional: without it, no rotation and no prefix ranking
  if (dimc.open()) {
    uint32_t h[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // magic, version, dim, nlist, rows, head, rotated, 0
    if (!dimc.take(h, 8) || h[0] != kDimcMagic || h[1] < 1u || h[1] > 2u)
      throw std::runtime_error("bad header in " + dimc.path());
    if (h[2] != a.dim || h[3] != a.nlist || h[4] != a.npts)
      throw std::runtime_error(dimc.path() + " does not match the index");
    a.has_dimc = true;
    a.head_dims = h[5];
    if (h[6] == 1u) {
      rotation.resize(static_cast<size_t>(a.dim) * a.dim);
      if (!dimc.take(rotation.data(), rotation.size()))
        throw std::runtime_error("truncated rotation in " + dimc.path());
      a.rotation = rotation.data();
    }
  }
  a.centroids = centroids.data();
  a.list_sizes = sizes.data();
  a.ids = ids.data();
  a.vectors = vectors.data();
  load_arrays(a, opt);
}

void Index::load_arrays(const IndexArrays &a, const LoadOptions &opt) {
  if (opt.precision == Precision::kBf16)
    throw std::invalid_argument("bf16 precision is not part of the GPU search path");
  if (!opt.batched_coarse)
    throw std::invalid_argument("the per-query float coarse search is not part of the GPU search path");
  if (a.dim == 0 || a.dim > kMaxDim || a.nlist == 0)
    throw std::invalid_argument("bad index shape: dimension must be 1 to 4096 and nlist >= 1");
  s_.reset();
  auto st = std::make_unique<State>();
  State &s = *st;
  s.dim = a.dim;
  s.nlist = a.nlist;
  s.npts = a.npts;
  s.normalized = a.normalized;
  s.dc = round_up(a.dim, 64u);
  s.max_batch = std::max(1u, opt.max_batch);
  cuda_check(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking), "cudaStreamCreate");
  cuda_check(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming), "cudaEventCreate");
  katoann_stream_t ks = reinterpret_cast<katoann_stream_t>(s.stream);
  const cudaMemcpyKind up = a.on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const uint32_t d = s.dim, dc = s.dc, n = s.npts, L = s.nlist;

  s.sizes.assign(a.list_sizes, a.list_sizes + L);
  std::vector<uint32_t> off(L + 1, 0);
  for (uint32_t c = 0; c < L; ++c) {
    off[c + 1] = off[c] + s.sizes[c];
    s.max_list = std::max(s.max_list, s.sizes[c]);
  }
  if (off[L] != n) throw std::invalid_argument("list sizes do not add up to the vector count");
  s.list_off.alloc((L + 1) * 4ull);
  cuda_check(cudaMemcpy(s.list_off.p, off.data(), (L + 1) * 4ull, cudaMemcpyHostToDevice), "upload");
  s.ids.alloc(static_cast<size_t>(n) * 4);
  if (n) cuda_check(cudaMemcpy(s.ids.p, a.ids, static_cast<size_t>(n) * 4, up), "upload ids");

  // Vectors, rotated on the device when the index has a rotation.
  DevBuf raw, rotd;
  const size_t nv = static_cast<size_t>(n) * d;
  const float *vec = a.vectors;
  if (!a.on_device) {
    raw.alloc(nv * 4);
    if (nv) cuda_check(cudaMemcpy(raw.p, a.vectors, nv * 4, cudaMemcpyHostToDevice), "upload vectors");
    vec = raw.as<float>();
  }
  s.rotated = a.rotation != nullptr;
  if (s.rotated) {
    s.rot.alloc(static_cast<size_t>(d) * d * 4);
    cuda_check(cudaMemcpy(s.rot.p, a.rotation, static_cast<size_t>(d) * d * 4, up), "upload rotation");
    rotd.alloc(nv * 4);
    gpu_check(katoann_gpu_rotate_rows(vec, n, d, s.rot.as<float>(), rotd.as<float>(), ks));
    vec = rotd.as<float>();
    raw.reset();
  }
  // Global scale (src/index.cpp:634-650).
  float glo = FLT_MAX, ghi = -FLT_MAX;
  if (nv) {
    DevBuf keys;
    keys.alloc(8);
    float mm[2];
    gpu_check(katoann_gpu_minmax(vec, nv, keys.as<uint32_t>(), mm, ks));
    glo = mm[0];
    ghi = mm[1];
  }
  s.lo = glo;
  const double rng = static_cast<double>(ghi) - glo;
  s.inv_step = 65535.0 / rng;
  s.step = rng / 65535.0;
  s.step_sq = s.step * s.step;
  // Head dims (src/index.cpp:792-793, :695-696).
  const uint32_t dims = opt.prefix_dims ? opt.prefix_dims : a.head_dims;
  if (a.has_dimc && dims) {
    if (dims % 64 || dims > dc)
      throw std::invalid_argument("prefix_dims must be a multiple of 64 within the dimension");
    s.head = dims;
  }
  s.hi.alloc(static_cast<size_t>(n) * dc);
  s.lop.alloc(static_cast<size_t>(n) * dc);
  s.norm.alloc(static_cast<size_t>(n) * 8);
  s.hinorm.alloc(static_cast<size_t>(n) * 8);
  if (s.head) s.headnorm.alloc(static_cast<size_t>(n) * 8);
  gpu_check(katoann_gpu_quantize_rows(vec, n, d, dc, s.lo, s.inv_step, s.head, s.hi.as<uint8_t>(),
                                      s.lop.as<uint8_t>(), s.norm.as<int64_t>(),
                                      s.hinorm.as<int64_t>(),
                                      s.head ? s.headnorm.as<int64_t>() : nullptr, ks));
  // Centroid planes with the database scale (src/index.cpp:718-750).
  {
    DevBuf cen, cenr, chn;
    cen.alloc(static_cast<size_t>(L) * d * 4);
    cuda_check(cudaMemcpy(cen.p, a.centroids, static_cast<size_t>(L) * d * 4, up), "upload centroids");
    const float *cv = cen.as<float>();
    if (s.rotated) {
      cenr.alloc(static_cast<size_t>(L) * d * 4);
      gpu_check(katoann_gpu_rotate_rows(cv, L, d, s.rot.as<float>(), cenr.as<float>(), ks));
      cv = cenr.as<float>();
    }
    s.chi.alloc(static_cast<size_t>(L) * dc);
    s.clo.alloc(static_cast<size_t>(L) * dc);
    s.cnorm.alloc(static_cast<size_t>(L) * 8);
    chn.alloc(static_cast<size_t>(L) * 8);
    gpu_check(katoann_gpu_quantize_rows(cv, L, d, dc, s.lo, s.inv_step, 0, s.chi.as<uint8_t>(),
                                        s.clo.as<uint8_t>(), s.cnorm.as<int64_t>(),
                                        chn.as<int64_t>(), nullptr, ks));
    // the same planes centred as fp16 for the tensor-core coarse product
    s.chi16.alloc(static_cast<size_t>(L) * dc * 2);
    s.clo16.alloc(static_cast<size_t>(L) * dc * 2);
    s.cterm.alloc(static_cast<size_t>(L) * 8);
    gpu_check(katoann_gpu_centre_planes(s.chi.as<uint8_t>(), s.clo.as<uint8_t>(),
                                        s.cnorm.as<int64_t>(), L, dc, s.chi16.as<uint16_t>(),
                                        s.clo16.as<uint16_t>(), s.cterm.as<int64_t>(), ks));
    cuda_check(cudaStreamSynchronize(s.stream), "load");
  }
  cuda_check(cudaStreamSynchronize(s.stream), "load");
  rotd.reset();
  set_view(s);
  s_ = std::move(st);
}

void Index::set_view(State &s) {
  const uint32_t d = s.dim, dc = s.dc, n = s.npts, L = s.nlist;
  if (s.rotated && !s.rot_t.p && katoann_gpu_rotation_kmajor_bytes(d)) {
    s.rot_t.alloc(katoann_gpu_rotation_kmajor_bytes(d));
    gpu_check(katoann_gpu_rotation_kmajor(s.rot.as<float>(), d, s.rot_t.as<float>(),
                                          reinterpret_cast<katoann_stream_t>(s.stream)));
    cuda_check(cudaStreamSynchronize(s.stream), "load");
  }
  katoann_gpu_index &v = s.view;
  v.dim = d;
  v.dc = dc;
  v.nlist = L;
  v.npts = n;
  v.head_dims = s.head;
  v.rotated = s.rotated ? 1 : 0;
  v.max_list = s.max_list;
  v.lo = s.lo;
  v.inv_step = s.inv_step;
  v.step_sq = s.step_sq;
  v.d_rotation = s.rot.as<float>();
  v.d_hi = s.hi.as<uint8_t>();
  v.d_lo = s.lop.as<uint8_t>();
  v.d_norm = s.norm.as<int64_t>();
  v.d_hinorm = s.hinorm.as<int64_t>();
  v.d_headnorm = s.head ? s.headnorm.as<int64_t>() : nullptr;
  v.d_ids = s.ids.as<uint32_t>();
  v.d_list_off = s.list_off.as<uint32_t>();
  v.d_chi = s.chi.as<uint8_t>();
  v.d_clo = s.clo.as<uint8_t>();
  v.d_cnorm = s.cnorm.as<int64_t>();
  v.d_chi16 = s.chi16.as<uint16_t>();
  v.d_clo16 = s.clo16.as<uint16_t>();
  v.d_cterm = s.cterm.as<int64_t>();
  v.d_rotation_t = s.rot_t.p ? s.rot_t.as<float>() : nullptr;
}

namespace {

int ranking_code(Ranking r) {
  return r == Ranking::kFull ? KATO_RANK_FULL : r == Ranking::kHighBytes ? KATO_RANK_HIGH : KATO_RANK_PREFIX;
}

// src/index.cpp:879-892
void validate(const void *state, uint32_t nlist, uint32_t head, const SearchParams &p) {
  if (!state || nlist == 0) throw std::logic_error("search before load");
  if (p.k == 0 || p.nprobe == 0 || p.nprobe > nlist)
    throw std::invalid_argument("need k >= 1 and 1 <= nprobe <= nlist");
  if (p.ranking == Ranking::kPrefix && head == 0)
    throw std::invalid_argument("prefix ranking needs the rotation file (.dimc)");
}

// The per-query budget of a search: the device model (when the params carry
// one and no explicit budgets) and the selection depth the workspace needs.
struct BudgetPlan {
  bool active = false;
  bool use_model = false;
  katoann_gpu_probe_model model{};
  uint32_t depth = 0;
};

BudgetPlan budget_plan(const SearchParams &p, uint32_t nlist) {
  BudgetPlan b;
  b.depth = p.nprobe;
  b.active = p.budget || p.nprobe_per_query;
  if (p.budget && !p.nprobe_per_query) {
    if (p.budget->empty()) throw std::invalid_argument("empty probe model");
    p.budget->device_model(p.budget_threshold, &b.model);
    b.use_model = true;
    b.depth = std::max(b.depth, b.model.depth);
    if (b.depth > nlist) throw std::invalid_argument("the probe model's depth exceeds nlist");
  }
  return b;
}

}  // namespace


void Index::search(const float *queries, uint32_t nq, const SearchParams &p, uint32_t *ids,
                   float *dists) const {
  if (nq == 0) return;
  validate(s_.get(), s_ ? s_->nlist : 0, s_ ? s_->head : 0, p);
  State &s = *s_;
  const BudgetPlan bp = budget_plan(p, s.nlist);
  std::lock_guard<std::mutex> lock(s.mu);
  const uint32_t mb = s.max_batch, b = std::min(nq, mb);
  const int rk = ranking_code(p.ranking);
  const size_t need = katoann_gpu_search_workspace(&s.view, b, p.k, bp.depth, rk, p.survivors);
  if (need == 0) gpu_check(KATO_EINVAL);
  if (need > s.ws.n) {
    cuda_check(cudaStreamSynchronize(s.stream), "workspace resize");
    s.drop_graphs();  // they hold the old workspace
    s.ws.ensure(need);
  }
  s.dq.ensure(static_cast<size_t>(b) * s.dim * 4);
  s.dids.ensure(static_cast<size_t>(b) * p.k * 4);
  s.ddists.ensure(static_cast<size_t>(b) * p.k * 4);
  if (p.nprobe_per_query) s.dnp_in.ensure(static_cast<size_t>(b) * 4);
  if (p.nprobe_used) s.dnp_out.ensure(static_cast<size_t>(b) * 4);
  if (s.last_stream && s.last_stream != s.stream)
    cuda_check(cudaStreamWaitEvent(s.stream, s.done, 0), "cudaStreamWaitEvent");
  const uint32_t passes = (nq + mb - 1) / mb;
  uint64_t *waits = s.wait_counts(passes);
  for (uint32_t q0 = 0; q0 < nq; q0 += mb) {
    const uint32_t nb = std::min(mb, nq - q0);
    cuda_check(cudaMemcpyAsync(s.dq.p, queries + static_cast<size_t>(q0) * s.dim,
                               static_cast<size_t>(nb) * s.dim * 4, cudaMemcpyHostToDevice, s.stream),
               "copy queries");
    if (p.graph) {
      // the kernels as one captured graph of the index's own buffers; the
      // copies in and out stay outside it
      if (p.nprobe_per_query)
        cuda_check(cudaMemcpyAsync(s.dnp_in.p, p.nprobe_per_query + q0, static_cast<size_t>(nb) * 4,
                                   cudaMemcpyHostToDevice, s.stream),
                   "copy budgets");
      void *h = s.graph_of(s.dq.as<float>(), nb, p, rk, bp.use_model ? &bp.model : nullptr,
                           s.dids.as<uint32_t>(), s.ddists.as<float>(),
                           p.nprobe_per_query ? s.dnp_in.as<uint32_t>() : nullptr,
                           p.nprobe_used ? s.dnp_out.as<uint32_t>() : nullptr, s.stream);
      gpu_check(katoann_gpu_graph_launch(h, reinterpret_cast<katoann_stream_t>(s.stream)));
      if (p.nprobe_used)
        cuda_check(cudaMemcpyAsync(p.nprobe_used + q0, s.dnp_out.p, static_cast<size_t>(nb) * 4,
                                   cudaMemcpyDeviceToHost, s.stream),
                   "copy budgets");
    } else if (bp.active || p.nprobe_used) {
      if (p.nprobe_per_query)
        cuda_check(cudaMemcpyAsync(s.dnp_in.p, p.nprobe_per_query + q0, static_cast<size_t>(nb) * 4,
                                   cudaMemcpyHostToDevice, s.stream),
                   "copy budgets");
      gpu_check(katoann_gpu_search_budget(
          &s.view, s.dq.as<float>(), nb, p.k, p.nprobe, rk, p.survivors, mb,
          p.nprobe_per_query ? s.dnp_in.as<uint32_t>() : nullptr,
          bp.use_model ? &bp.model : nullptr, s.ws.p, s.ws.n, s.dids.as<uint32_t>(),
          s.ddists.as<float>(), p.nprobe_used ? s.dnp_out.as<uint32_t>() : nullptr,
          reinterpret_cast<katoann_stream_t>(s.stream), nullptr));
      if (p.nprobe_used)
        cuda_check(cudaMemcpyAsync(p.nprobe_used + q0, s.dnp_out.p, static_cast<size_t>(nb) * 4,
                                   cudaMemcpyDeviceToHost, s.stream),
                   "copy budgets");
    } else {
      gpu_check(katoann_gpu_search(&s.view, s.dq.as<float>(), nb, p.k, p.nprobe, rk, p.survivors,
                                   mb, s.ws.p, s.ws.n, s.dids.as<uint32_t>(),
                                   s.ddists.as<float>(), reinterpret_cast<katoann_stream_t>(s.stream)));
    }
    cuda_check(cudaMemcpyAsync(ids + static_cast<size_t>(q0) * p.k, s.dids.p,
                               static_cast<size_t>(nb) * p.k * 4, cudaMemcpyDeviceToHost, s.stream),
               "copy ids");
    cuda_check(cudaMemcpyAsync(dists + static_cast<size_t>(q0) * p.k, s.ddists.p,
                               static_cast<size_t>(nb) * p.k * 4, cudaMemcpyDeviceToHost, s.stream),
               "copy dists");
    cuda_check(cudaMemcpyAsync(waits + q0 / mb, static_cast<const char *>(s.ws.p) + 3 * sizeof(uint64_t),
                               sizeof(uint64_t), cudaMemcpyDeviceToHost, s.stream),
               "copy statistics");
  }
  cuda_check(cudaEventRecord(s.done, s.stream), "cudaEventRecord");
  s.last_stream = s.stream;
  cuda_check(cudaStreamSynchronize(s.stream), "search");
  for (uint32_t i = 0; i < passes; ++i)
    if (waits[i])
      throw timeout_error("search: a bounded pipeline wait in a tensor-core kernel ran out (" +
                          std::to_string(waits[i]) + " CTAs); the results are incomplete");
}

void Index::search_device(const float *d_queries, uint32_t nq, const SearchParams &p,
                          uint32_t *d_ids, float *d_dists, void *stream, void *timer) const {
  if (nq == 0) return;
  validate(s_.get(), s_ ? s_->nlist : 0, s_ ? s_->head : 0, p);
  State &s = *s_;
  std::lock_guard<std::mutex> lock(s.mu);
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : s.stream;
  const int rk = ranking_code(p.ranking);
  const BudgetPlan bp = budget_plan(p, s.nlist);
  const size_t need =
      katoann_gpu_search_workspace(&s.view, std::min(nq, s.max_batch), p.k, bp.depth, rk, p.survivors);
  if (need == 0) gpu_check(KATO_EINVAL);
  if (need > s.ws.n) {
    cuda_check(cudaDeviceSynchronize(), "workspace resize");
    s.drop_graphs();  // they hold the old workspace
    s.ws.ensure(need);
  }
  if (s.last_stream && s.last_stream != st)
    cuda_check(cudaStreamWaitEvent(st, s.done, 0), "cudaStreamWaitEvent");
  if (p.graph) {
    if (timer) throw std::invalid_argument("a graph search records no phase events");
    void *h = s.graph_of(d_queries, nq, p, rk, bp.use_model ? &bp.model : nullptr, d_ids, d_dists,
                         p.nprobe_per_query, p.nprobe_used, st);
    gpu_check(katoann_gpu_graph_launch(h, reinterpret_cast<katoann_stream_t>(st)));
  } else if (bp.active || p.nprobe_used)
    gpu_check(katoann_gpu_search_budget(&s.view, d_queries, nq, p.k, p.nprobe, rk, p.survivors,
                                        s.max_batch, p.nprobe_per_query,
                                        bp.use_model ? &bp.model : nullptr, s.ws.p, s.ws.n, d_ids,
                                        d_dists, p.nprobe_used,
                                        reinterpret_cast<katoann_stream_t>(st), timer));
  else
    gpu_check(katoann_gpu_search_timed(&s.view, d_queries, nq, p.k, p.nprobe, rk, p.survivors,
                                       s.max_batch, s.ws.p, s.ws.n, d_ids, d_dists,
                                       reinterpret_cast<katoann_stream_t>(st), timer));
  cuda_check(cudaEventRecord(s.done, st), "cudaEventRecord");
  s.last_stream = st;
}

Index::Tuning Index::autotune(const float *queries, uint32_t nq, const SearchParams &p) {
  if (nq == 0) throw std::invalid_argument("autotune needs queries");
  validate(s_.get(), s_ ? s_->nlist : 0, s_ ? s_->head : 0, p);
  State &s = *s_;
  const BudgetPlan bp = budget_plan(p, s.nlist);
  std::lock_guard<std::mutex> lock(s.mu);
  const uint32_t b = std::min(nq, s.max_batch);
  const int rk = ranking_code(p.ranking);
  // room for every candidate item width
  uint32_t knobs[3];
  katoann_gpu_rank_knobs(knobs);
  size_t need = 0;
  for (uint32_t w : {0u, 32u}) {
    gpu_check(katoann_gpu_set_rank_width(w));
    need = std::max(need, katoann_gpu_search_workspace(&s.view, b, p.k, bp.depth, rk, p.survivors));
  }
  gpu_check(katoann_gpu_set_rank_width(knobs[2]));
  if (need == 0) gpu_check(KATO_EINVAL);
  cuda_check(cudaStreamSynchronize(s.stream), "autotune");
  s.drop_graphs();
  s.ws.ensure(need);
  s.dq.ensure(static_cast<size_t>(b) * s.dim * 4);
  cuda_check(cudaMemcpy(s.dq.p, queries, static_cast<size_t>(b) * s.dim * 4, cudaMemcpyHostToDevice),
             "copy queries");
  uint32_t out[4] = {0, 0, 0, 0};
  gpu_check(katoann_gpu_autotune(&s.view, s.dq.as<float>(), b, p.k, p.nprobe, rk, p.survivors, b,
                                 nullptr, bp.use_model ? &bp.model : nullptr, s.ws.p, s.ws.n,
                                 reinterpret_cast<katoann_stream_t>(s.stream), out));
  return Tuning{out[0], out[1], out[2], static_cast<double>(out[3])};
}

std::vector<uint64_t> Index::last_search_stats() const {
  std::vector<uint64_t> out(48, 0);
  if (!s_ || !s_->ws.p) return out;
  std::lock_guard<std::mutex> lock(s_->mu);
  cuda_check(cudaEventSynchronize(s_->done), "stats");
  gpu_check(katoann_gpu_workspace_stats(s_->ws.p, out.data(), 48,
                                        reinterpret_cast<katoann_stream_t>(s_->stream)));
  return out;
}

const void *Index::device_view() const { return s_ ? &s_->view : nullptr; }

uint32_t Index::dim() const { return s_ ? s_->dim : 0; }
uint32_t Index::nlist() const { return s_ ? s_->nlist : 0; }
uint32_t Index::size() const { return s_ ? s_->npts : 0; }
bool Index::normalized() const { return s_ && s_->normalized; }
uint32_t Index::prefix_dims() const { return s_ ? s_->head : 0; }
bool Index::rotated() const { return s_ && s_->rotated; }
bool Index::batched_coarse() const { return s_ != nullptr; }
std::vector<uint32_t> Index::list_sizes() const { return s_ ? s_->sizes : std::vector<uint32_t>{}; }

size_t Index::memory_bytes() const {
  if (!s_) return 0;
  const State &s = *s_;
  return s.rot.n + s.hi.n + s.lop.n + s.norm.n + s.hinorm.n + s.headnorm.n + s.ids.n +
         s.list_off.n + s.chi.n + s.clo.n + s.cnorm.n + s.chi16.n + s.clo16.n + s.cterm.n +
         s.rot_t.n + s.sizes.size() * 4;
}

}  // namespace katoann
