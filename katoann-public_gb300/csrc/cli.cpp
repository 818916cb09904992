// The katoann command-line tool on the GPU. It keeps the interface of the
// reference's tool (tools/katoann.cpp:339-352, README.md:179-198): the
// commands build, search and load, their flags, the JSON lines they print,
// the error messages and the exit codes (2 for a usage error, 1 for any other
// error, printed as "katoann: <message>"). It adds `budget`, which trains the
// learned probe-budget model that `load --budget` serves.
//
// Everything is driven by one table of flags (kFlags): the parser checks each
// argument against the command's rows, fills in the table's defaults, and the
// usage text is printed from the same rows. `load` serves Poisson arrivals
// through the continuous-batching katoann::Server (several batches in flight,
// per-request k, an HBM budget), where the reference answers one batch at a
// time; latency still runs from a request's arrival to its completion.
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "katoann/index.h"
#include "katoann/probe.h"
#include "katoann/server.h"

namespace {

// ------------------------------------------------------------------ flags
enum Command : unsigned { kBuild = 1u, kSearch = 2u, kLoad = 4u, kBudget = 8u };
constexpr unsigned kQuerying = kSearch | kLoad | kBudget;  // commands that load an index

struct Flag {
  const char *name;
  const char *meta;   // value placeholder in the usage text; null for a switch
  const char *dflt;   // default value (null: none)
  unsigned used;      // commands that accept the flag
  unsigned required;  // commands that need it
};

// The reference's flags first (same names, same defaults), then the GPU
// tool's additions. Order matters twice: the usage text follows it, and the
// first missing required flag in this order is the one reported.
const Flag kFlags[] = {
    {"data", "BASE.fbin", nullptr, kBuild, kBuild},
    {"index", "PREFIX", nullptr, kQuerying, kQuerying},
    {"queries", "Q.fbin", nullptr, kQuerying, kQuerying},
    {"out", "PREFIX", nullptr, kBuild | kSearch | kBudget, kBuild | kBudget},
    {"nlist", "N", "2048", kBuild, 0},
    {"normalize", nullptr, nullptr, kBuild, 0},
    {"normalized", nullptr, nullptr, kBuild, 0},
    {"train-size", "N", "256000", kBuild, 0},
    {"iters", "N", "12", kBuild, 0},
    {"seed", "S", nullptr, kBuild | kLoad | kBudget, 0},
    {"threads", "T", "0", kBuild | kQuerying, 0},
    {"gt", "GT.bin", nullptr, kSearch, 0},
    {"k", "K", "10", kQuerying, 0},
    {"nprobe", "64,128", "64", kQuerying, 0},
    {"ranking", "prefix|high|full", "prefix", kQuerying, 0},
    {"survivors", "S", "32", kQuerying, 0},
    {"prefix-dims", "D", "0", kQuerying, 0},
    {"selection", "threshold|local", "threshold", kQuerying, 0},
    {"batch", "B", "4096", kQuerying, 0},
    {"precision", "sq16", "sq16", kQuerying, 0},
    {"engine", "gpu", "gpu", kQuerying, 0},
    {"coarse", "batched", "batched", kQuerying, 0},
    {"repeat", "R", "3", kSearch, 0},
    {"query-ids", "FILE", nullptr, kQuerying, 0},
    {"rate", "QPS", "1000", kLoad, 0},
    {"requests", "N", "10000", kLoad, 0},
    {"max-batch", "B", "4096", kQuerying, 0},
    {"code-cache", nullptr, nullptr, kQuerying, 0},
    {"k-mix", "10,100", nullptr, kLoad, 0},
    {"in-flight", "N", "3", kLoad, 0},
    {"hbm-budget-gb", "G", "0", kLoad, 0},
    {"max-wait-ms", "MS", "0", kLoad, 0},
    {"budget", "MODEL.kprb", nullptr, kLoad, 0},
    {"threshold", "P", "0.95", kLoad, 0},
    {"ladder", "8,16,...", nullptr, kBudget, 0},
    {"depth", "D", nullptr, kBudget, 0},
    {"label-nprobe", "N", "0", kBudget, 0},
    {"label-ranking", "full|prefix|high", "full", kBudget, 0},
    {"label-survivors", "S", "0", kBudget, 0},
    {"epochs", "E", "24", kBudget, 0},
    {"train-batch", "B", "1024", kBudget, 0},
};

const Flag *find_flag(const std::string &name) {
  for (const Flag &f : kFlags)
    if (name == f.name) return &f;
  return nullptr;
}

const char *command_name(unsigned c) {
  return c == kBuild ? "build" : c == kSearch ? "search" : c == kLoad ? "load" : "budget";
}

void usage() {
  std::string text = "usage:";
  for (unsigned c : {kBuild, kSearch, kLoad, kBudget}) {
    std::string line = std::string(text.size() > 6 ? "      " : "") + " katoann " + command_name(c);
    const size_t indent = 15;
    for (const Flag &f : kFlags) {
      if (!(f.used & c)) continue;
      std::string item = std::string("--") + f.name + (f.meta ? std::string(" ") + f.meta : "");
      if (!(f.required & c)) item = "[" + item + "]";
      const size_t last_nl = line.rfind('\n');
      const size_t width = line.size() - (last_nl == std::string::npos ? 0 : last_nl + 1);
      if (width + 1 + item.size() > 92) line += "\n" + std::string(indent, ' ');
      line += " " + item;
    }
    text += line + "\n";
  }
  std::fputs(text.c_str(), stderr);
}

// The parsed command line of one command: every value the table allows, the
// switches that were given, and typed access with the table's defaults.
class Options {
 public:
  Options(unsigned cmd, int argc, char **argv) {
    for (int i = 2; i < argc; ++i) {
      const std::string arg = argv[i];
      if (arg.compare(0, 2, "--") != 0) throw std::invalid_argument("unexpected argument " + arg);
      std::string name = arg.substr(2), value;
      const size_t eq = name.find('=');
      const bool inline_value = eq != std::string::npos;
      if (inline_value) value = name.substr(eq + 1), name.resize(eq);
      const Flag *f = find_flag(name);
      if (!f || !(f->used & cmd))
        throw std::invalid_argument("unknown option --" + name + " for " + command_name(cmd));
      if (!f->meta) {
        if (inline_value) throw std::invalid_argument("--" + name + " takes no value");
        switches_.insert(name);
        continue;
      }
      if (!inline_value) {
        if (i + 1 >= argc) throw std::invalid_argument("missing value for --" + name);
        value = argv[++i];
      }
      values_[name] = value;
    }
    for (const Flag &f : kFlags)
      if ((f.required & cmd) && !values_.count(f.name))
        throw std::invalid_argument(std::string("missing --") + f.name);
  }

  bool given(const char *name) const { return values_.count(name) || switches_.count(name); }
  bool on(const char *name) const { return switches_.count(name) != 0; }
  std::string text(const char *name) const {
    const auto it = values_.find(name);
    if (it != values_.end()) return it->second;
    const Flag *f = find_flag(name);
    return f && f->dflt ? f->dflt : "";
  }
  uint32_t u32(const char *name) const { return static_cast<uint32_t>(std::stoul(text(name))); }
  uint32_t u32_or(const char *name, uint32_t fallback) const {
    return given(name) ? u32(name) : fallback;
  }
  uint64_t u64_or(const char *name, uint64_t fallback) const {
    return given(name) ? std::stoull(text(name)) : fallback;
  }
  double real(const char *name) const { return std::stod(text(name)); }
  std::vector<uint32_t> list(const char *name) const {
    std::vector<uint32_t> out;
    const std::string s = text(name);
    size_t at = 0;
    while (at <= s.size() && !s.empty()) {
      const size_t comma = std::min(s.find(',', at), s.size());
      out.push_back(static_cast<uint32_t>(std::stoul(s.substr(at, comma - at))));
      at = comma + 1;
    }
    return out;
  }
  // One of several spellings, mapped to its value; anything else is `complaint`.
  template <typename T>
  T choice(const char *name, std::initializer_list<std::pair<const char *, T>> table,
           const char *complaint) const {
    const std::string v = text(name);
    for (const auto &entry : table)
      if (v == entry.first) return entry.second;
    throw std::invalid_argument(complaint);
  }

 private:
  std::map<std::string, std::string> values_;
  std::set<std::string> switches_;
};

// ------------------------------------------------------------- file I/O
// .fbin vectors and ground-truth files share one layout: uint32 rows, uint32
// columns, then rows x columns values of 4 bytes.
template <typename T>
struct Table {
  uint32_t rows = 0, cols = 0;
  std::vector<T> cells;
  const T *row(size_t i) const { return cells.data() + i * cols; }
};

template <typename T>
Table<T> read_table(const std::string &path) {
  static_assert(sizeof(T) == 4, "4-byte cells");
  std::unique_ptr<FILE, int (*)(FILE *)> f(std::fopen(path.c_str(), "rb"), &std::fclose);
  if (!f) throw std::runtime_error("cannot open " + path);
  uint32_t head[2] = {0, 0};
  Table<T> t;
  if (std::fread(head, sizeof(uint32_t), 2, f.get()) == 2) {
    t.rows = head[0];
    t.cols = head[1];
    t.cells.resize(static_cast<size_t>(t.rows) * t.cols);
    if (std::fread(t.cells.data(), sizeof(T), t.cells.size(), f.get()) == t.cells.size()) return t;
  }
  throw std::runtime_error("truncated " + path);
}

void write_results(const std::string &path, uint32_t rows, uint32_t k,
                   const std::vector<uint32_t> &ids, const std::vector<float> &dists) {
  std::unique_ptr<FILE, int (*)(FILE *)> f(std::fopen(path.c_str(), "wb"), &std::fclose);
  if (!f) throw std::runtime_error("cannot write " + path);
  const uint32_t head[2] = {rows, k};
  std::fwrite(head, sizeof(uint32_t), 2, f.get());
  std::fwrite(ids.data(), sizeof(uint32_t), ids.size(), f.get());
  std::fwrite(dists.data(), sizeof(float), dists.size(), f.get());
}

// ------------------------------------------------------------ JSON lines
class JsonLine {
 public:
  JsonLine &str(const char *key, const std::string &v) { return put(key, "\"" + v + "\""); }
  JsonLine &count(const char *key, unsigned long long v) { return put(key, std::to_string(v)); }
  JsonLine &sint(const char *key, long long v) { return put(key, std::to_string(v)); }
  JsonLine &fixed(const char *key, double v, int digits) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.*f", digits, v);
    return put(key, buf);
  }
  JsonLine &flag(const char *key, bool v) { return put(key, v ? "true" : "false"); }
  JsonLine &list(const char *key, const std::vector<uint64_t> &v) {
    std::string s = "[";
    for (size_t i = 0; i < v.size(); ++i) s += (i ? ", " : "") + std::to_string(v[i]);
    return put(key, s + "]");
  }
  void print() const {
    std::printf("{%s}\n", body_.c_str());
    std::fflush(stdout);
  }

 private:
  JsonLine &put(const char *key, const std::string &v) {
    body_ += (body_.empty() ? "\"" : ", \"") + std::string(key) + "\": " + v;
    return *this;
  }
  std::string body_;
};

using Clock = std::chrono::steady_clock;
double since(Clock::time_point t) { return std::chrono::duration<double>(Clock::now() - t).count(); }

// ------------------------------------------------------ shared settings
void apply_threads(const Options &o) {
  omp_set_dynamic(0);
  if (const uint32_t t = o.u32("threads")) omp_set_num_threads(static_cast<int>(t));
}

katoann::LoadOptions load_options(const Options &o) {
  katoann::LoadOptions lo;
  lo.precision = o.choice<katoann::Precision>(
      "precision", {{"sq16", katoann::Precision::kSq16}, {"bf16", katoann::Precision::kBf16}},
      "--precision is sq16 or bf16");
  // the reference's CPU engines are accepted and name the one GPU engine
  lo.use_amx = o.choice<bool>("engine", {{"gpu", true}, {"amx", true}, {"avx512", false}},
                              "--engine is gpu, amx or avx512");
  lo.prefix_dims = o.u32("prefix-dims");
  lo.batched_coarse = o.choice<bool>("coarse", {{"batched", true}, {"flat", false}},
                                     "--coarse is batched or flat");
  lo.max_batch = std::max(o.u32("batch"), o.u32("max-batch"));
  lo.code_cache = o.on("code-cache");
  return lo;
}

katoann::SearchParams search_params(const Options &o) {
  katoann::SearchParams p;
  p.k = o.u32("k");
  p.ranking = o.choice<katoann::Ranking>("ranking",
                                         {{"prefix", katoann::Ranking::kPrefix},
                                          {"high", katoann::Ranking::kHighBytes},
                                          {"full", katoann::Ranking::kFull}},
                                         "--ranking is prefix, high, or full");
  p.survivors = o.u32("survivors");
  p.selection = o.choice<katoann::Selection>(
      "selection", {{"threshold", katoann::Selection::kThreshold}, {"local", katoann::Selection::kLocal}},
      "--selection is threshold or local");
  return p;
}

// An index with its query file: the index loaded (and timed), the queries
// normalized as the index was, and the subset --query-ids names (default: all).
struct Workload {
  katoann::Index index;
  double load_s = 0;
  Table<float> queries;
  std::vector<uint32_t> chosen;

  explicit Workload(const Options &o) {
    const auto t0 = Clock::now();
    index.load(o.text("index"), load_options(o));
    load_s = since(t0);
    queries = read_table<float>(o.text("queries"));
    if (queries.cols != index.dim()) throw std::runtime_error("query dimension does not match the index");
    if (index.normalized()) katoann::normalize_rows(queries.cells.data(), queries.rows, queries.cols);
    choose(o.text("query-ids"));
  }
  uint32_t dim() const { return queries.cols; }
  // the chosen queries, back to back
  std::vector<float> gathered() const {
    std::vector<float> out(chosen.size() * static_cast<size_t>(dim()));
    for (size_t i = 0; i < chosen.size(); ++i)
      std::copy_n(queries.row(chosen[i]), dim(), out.data() + i * dim());
    return out;
  }

 private:
  void choose(const std::string &path) {
    if (path.empty()) {
      chosen.resize(queries.rows);
      for (uint32_t i = 0; i < queries.rows; ++i) chosen[i] = i;
      return;
    }
    std::unique_ptr<FILE, int (*)(FILE *)> f(std::fopen(path.c_str(), "r"), &std::fclose);
    if (!f) throw std::runtime_error("cannot open " + path);
    unsigned long v = 0;
    while (std::fscanf(f.get(), "%lu", &v) == 1) {
      if (v >= queries.rows) throw std::runtime_error("query id out of range in " + path);
      chosen.push_back(static_cast<uint32_t>(v));
    }
    if (chosen.empty()) throw std::runtime_error("no query ids in " + path);
  }
};

// recall@k: the share of each result row's ids found among the first k ids
// of its query's ground-truth row.
double recall(const std::vector<uint32_t> &ids, uint32_t k, const std::vector<uint32_t> &chosen,
              const Table<uint32_t> &gt) {
  size_t hits = 0;
  std::vector<uint32_t> truth(k);
  for (size_t i = 0; i < chosen.size(); ++i) {
    std::copy_n(gt.row(chosen[i]), k, truth.begin());
    std::sort(truth.begin(), truth.end());
    for (uint32_t j = 0; j < k; ++j)
      hits += std::binary_search(truth.begin(), truth.end(), ids[i * k + j]) ? 1 : 0;
  }
  return static_cast<double>(hits) / (static_cast<double>(chosen.size()) * k);
}

// One untimed pass, then `repeat` timed ones; their times sorted ascending.
template <typename Pass>
std::vector<double> timed_passes(uint32_t repeat, Pass pass) {
  pass();
  std::vector<double> secs(std::max(1u, repeat));
  for (double &s : secs) {
    const auto t0 = Clock::now();
    pass();
    s = since(t0);
  }
  std::sort(secs.begin(), secs.end());
  return secs;
}

// --------------------------------------------------------------- commands
int run_build(const Options &o) {
  apply_threads(o);
  Table<float> data = read_table<float>(o.text("data"));
  katoann::BuildOptions bo;
  bo.nlist = o.u32("nlist");
  bo.train_size = o.u32("train-size");
  bo.kmeans_iters = o.u32("iters");
  bo.seed = o.u64_or("seed", 0);
  if (o.on("normalize")) katoann::normalize_rows(data.cells.data(), data.rows, data.cols);
  bo.normalized = o.on("normalize") || o.on("normalized");
  const auto t0 = Clock::now();
  katoann::Index::build(data.cells.data(), data.rows, data.cols, bo, o.text("out"));
  JsonLine()
      .count("vectors", data.rows)
      .count("dim", data.cols)
      .count("nlist", bo.nlist)
      .fixed("build_s", since(t0), 1)
      .print();
  return 0;
}

int run_search(const Options &o) {
  apply_threads(o);
  Workload w(o);
  const std::vector<float> q = w.gathered();
  katoann::SearchParams p = search_params(o);
  Table<uint32_t> gt;
  const bool scored = o.given("gt");
  if (scored) {
    gt = read_table<uint32_t>(o.text("gt"));
    if (gt.rows < w.queries.rows || gt.cols < p.k) throw std::runtime_error("ground truth too small");
  }
  const uint32_t batch = o.u32("batch");
  const size_t total = w.chosen.size();
  JsonLine()
      .str("index", o.text("index"))
      .str("engine", "gpu")
      .sint("threads", omp_get_max_threads())
      .fixed("load_s", w.load_s, 1)
      .fixed("memory_gb", w.index.memory_bytes() / 1e9, 2)
      .count("queries", total)
      .count("prefix_dims", w.index.prefix_dims())
      .print();
  std::vector<uint32_t> ids(total * p.k);
  std::vector<float> dists(total * p.k);
  for (const uint32_t nprobe : o.list("nprobe")) {
    p.nprobe = nprobe;
    // the chosen queries in batches of --batch, in order
    const std::vector<double> secs = timed_passes(o.u32("repeat"), [&] {
      for (size_t at = 0; at < total; at += batch) {
        const uint32_t n = static_cast<uint32_t>(std::min<size_t>(batch, total - at));
        w.index.search(q.data() + at * w.dim(), n, p, ids.data() + at * p.k, dists.data() + at * p.k);
      }
    });
    const double median = secs[secs.size() / 2];
    JsonLine line;
    line.count("nprobe", nprobe)
        .count("k", p.k)
        .count("survivors", p.survivors)
        .count("batch", batch)
        .fixed("qps", total / median, 1)
        .fixed("seconds_median", median, 4)
        .fixed("seconds_min", secs.front(), 4)
        .fixed("seconds_max", secs.back(), 4);
    if (scored) line.fixed("recall", recall(ids, p.k, w.chosen, gt), 5);
    line.print();
    if (o.given("out"))
      write_results(o.text("out") + ".np" + std::to_string(nprobe) + ".bin",
                    static_cast<uint32_t>(total), p.k, ids, dists);
  }
  return 0;
}

int run_budget(const Options &o) {
  apply_threads(o);
  Workload w(o);
  const katoann::SearchParams sp = search_params(o);
  katoann::ProbeTrainOptions to;
  if (o.given("ladder")) to.ladder = o.list("ladder");
  // ladder values beyond the index's lists cannot be probed
  to.ladder.erase(std::remove_if(to.ladder.begin(), to.ladder.end(),
                                 [&](uint32_t v) { return v > w.index.nlist(); }),
                  to.ladder.end());
  to.depth = o.u32_or("depth", std::min(256u, w.index.nlist()));
  to.k = sp.k;
  to.label_nprobe = o.u32("label-nprobe");
  to.label_ranking = o.choice<katoann::Ranking>("label-ranking",
                                                {{"full", katoann::Ranking::kFull},
                                                 {"prefix", katoann::Ranking::kPrefix},
                                                 {"high", katoann::Ranking::kHighBytes}},
                                                "--label-ranking is full, prefix or high");
  to.label_survivors = o.u32("label-survivors");
  to.ranking = sp.ranking;
  to.survivors = sp.survivors;
  to.epochs = o.u32("epochs");
  to.batch = o.u32("train-batch");
  to.seed = o.u64_or("seed", 0);
  const std::vector<float> q = w.gathered();
  const auto t0 = Clock::now();
  const katoann::ProbeModel m =
      katoann::ProbeModel::train(w.index, q.data(), static_cast<uint32_t>(w.chosen.size()), to);
  m.save(o.text("out"));
  std::vector<uint64_t> per_class(m.classes(), 0);
  for (const uint8_t label : m.labels()) ++per_class[label];
  JsonLine()
      .count("queries", w.chosen.size())
      .count("classes", m.classes())
      .count("depth", m.depth())
      .fixed("train_s", since(t0), 2)
      .fixed("loss_first", m.loss().front(), 4)
      .fixed("loss_last", m.loss().back(), 4)
      .list("label_histogram", per_class)
      .print();
  return 0;
}

int run_load(const Options &o) {
  apply_threads(o);
  Workload w(o);
  const katoann::SearchParams sp = search_params(o);
  // per-request k: one value, or a list drawn uniformly per request
  const std::vector<uint32_t> kmix = o.given("k-mix") ? o.list("k-mix") : std::vector<uint32_t>{sp.k};
  if (kmix.empty()) throw std::invalid_argument("empty --k-mix");
  katoann::ServerOptions so;
  so.max_batch = std::max(1u, std::min(4096u, o.u32("max-batch")));
  so.max_in_flight = o.u32("in-flight");
  so.hbm_budget = static_cast<size_t>(o.real("hbm-budget-gb") * 1e9);
  so.max_k = *std::max_element(kmix.begin(), kmix.end());
  so.nprobe = o.u32("nprobe");
  so.ranking = sp.ranking;
  so.survivors = sp.survivors;
  so.max_wait_ms = o.real("max-wait-ms");
  katoann::ProbeModel model;
  if (o.given("budget")) {  // learned per-query nprobe, capped at --nprobe
    model = katoann::ProbeModel::load(o.text("budget"));
    so.budget = &model;
    so.budget_threshold = static_cast<float>(o.real("threshold"));
  }
  const double rate = o.real("rate");
  const uint32_t requests = o.u32("requests");
  katoann::Server server(w.index, so);
  // warm-up: one full batch per k of the mix
  const uint32_t warm = std::min<uint32_t>(so.max_batch, static_cast<uint32_t>(w.chosen.size()));
  std::vector<uint64_t> tickets;
  for (const uint32_t k : kmix)
    for (uint32_t i = 0; i < warm; ++i) tickets.push_back(server.submit(w.queries.row(w.chosen[i]), k));
  for (const uint64_t t : tickets) server.wait(t);
  const katoann::LoadReport r = katoann::run_load(server, w.queries.cells.data(), w.dim(), w.chosen,
                                                  rate, requests, kmix, o.u64_or("seed", 42));
  JsonLine()
      .fixed("rate", rate, 1)
      .count("requests", requests)
      .count("nprobe", so.nprobe)
      .str("engine", "gpu")
      .fixed("achieved_qps", r.achieved_qps, 1)
      .fixed("p50_ms", r.p50_ms, 2)
      .fixed("p95_ms", r.p95_ms, 2)
      .fixed("p99_ms", r.p99_ms, 2)
      .fixed("max_ms", r.max_ms, 2)
      .count("batches", r.batches)
      .fixed("mean_batch", r.mean_batch, 1)
      .count("in_flight", so.max_in_flight)
      .count("peak_in_flight", r.peak_in_flight)
      .fixed("peak_hbm_gb", r.peak_hbm_bytes / 1e9, 3)
      .flag("learned", so.budget != nullptr)
      .fixed("mean_nprobe", r.mean_nprobe, 2)
      .fixed("max_lag_ms", r.max_lag_ms, 2)
      .fixed("max_enqueue_ms", r.max_enqueue_ms, 2)
      .fixed("max_batch_gpu_ms", r.max_batch_gpu_ms, 2)
      .print();
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  const std::pair<const char *, std::pair<unsigned, int (*)(const Options &)>> commands[] = {
      {"build", {kBuild, run_build}},
      {"search", {kSearch, run_search}},
      {"load", {kLoad, run_load}},
      {"budget", {kBudget, run_budget}},
  };
  const std::string name = argc > 1 ? argv[1] : "";
  for (const auto &c : commands) {
    if (name != c.first) continue;
    try {
      return c.second.second(Options(c.second.first, argc, argv));
    } catch (const std::exception &e) {
      std::fprintf(stderr, "katoann: %s\n", e.what());
      return 1;
    }
  }
  usage();
  return 2;
}
