// The katoann command-line tool on the GPU: the reference's three commands
// with the same flags and the same JSON lines (tools/katoann.cpp:339-352,
// README.md:179-198), over katoann::Index from libkatoann.so.
//
//   katoann build  --data BASE.fbin --out PREFIX [--nlist 2048] [--normalize]
//                  [--train-size 256000] [--iters 12] [--seed 0] [--threads T]
//   katoann search --index PREFIX --queries Q.fbin [--gt GT.bin] [--k 10]
//                  [--nprobe 64,128] [--ranking prefix|high|full] [--survivors 32]
//                  [--prefix-dims D] [--selection threshold|local] [--batch 4096]
//                  [--precision sq16] [--engine gpu|amx|avx512] [--coarse batched]
//                  [--repeat 3] [--threads T] [--query-ids FILE] [--out PREFIX]
//                  [--code-cache]
//   katoann load   --index PREFIX --queries Q.fbin --rate QPS [--requests 10000]
//                  [--nprobe 64] [--max-batch 4096] [--seed 42] [--k-mix 10,100]
//                  [--in-flight 3] [--hbm-budget-gb G] [--max-wait-ms 0]
//                  [--budget MODEL.kprb --threshold 0.95] and the search flags
//   katoann budget --index PREFIX --queries TRAIN.fbin --out MODEL.kprb [--ladder ...]
//                  [--depth 256] [--label-nprobe N] [--epochs 24] and the search flags
//
// `load` serves requests that arrive as a Poisson process (tools/katoann.cpp:
// 263-337), here through the continuous-batching katoann::Server: arrivals are
// batched per k while earlier batches are still on the device (up to
// --in-flight batches within --hbm-budget-gb), optionally with the learned
// per-query nprobe of a ProbeModel file; latency runs from a request's
// arrival to its completion. Errors print to stderr and exit 1, as the
// reference's main does.
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <random>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "katoann/index.h"
#include "katoann/probe.h"
#include "katoann/server.h"

namespace {

using Clock = std::chrono::steady_clock;

double seconds_since(Clock::time_point t) {
  return std::chrono::duration<double>(Clock::now() - t).count();
}

// --key value pairs and the value-less switches.
struct Args {
  std::map<std::string, std::string> kv;
  std::set<std::string> flags;

  bool has(const std::string &k) const { return flags.count(k) != 0; }
  std::string get(const std::string &k, const std::string &dflt = "") const {
    const auto it = kv.find(k);
    return it == kv.end() ? dflt : it->second;
  }
  std::string need(const std::string &k) const {
    const auto it = kv.find(k);
    if (it == kv.end()) throw std::invalid_argument("missing --" + k);
    return it->second;
  }
  uint32_t u32(const std::string &k, uint32_t dflt) const {
    const auto it = kv.find(k);
    return it == kv.end() ? dflt : static_cast<uint32_t>(std::stoul(it->second));
  }
  double num(const std::string &k, double dflt) const {
    const auto it = kv.find(k);
    return it == kv.end() ? dflt : std::stod(it->second);
  }
};

Args parse(int argc, char **argv, int first) {
  static const std::set<std::string> kSwitches = {"normalize", "normalized", "code-cache"};
  Args a;
  for (int i = first; i < argc; ++i) {
    std::string s = argv[i];
    if (s.rfind("--", 0) != 0) throw std::invalid_argument("unexpected argument " + s);
    s = s.substr(2);
    if (kSwitches.count(s)) {
      a.flags.insert(s);
    } else {
      if (i + 1 >= argc) throw std::invalid_argument("missing value for --" + s);
      a.kv[s] = argv[++i];
    }
  }
  return a;
}

std::vector<uint32_t> u32_list(const std::string &s) {
  std::vector<uint32_t> out;
  std::stringstream in(s);
  std::string item;
  while (std::getline(in, item, ',')) out.push_back(static_cast<uint32_t>(std::stoul(item)));
  return out;
}

// .fbin: uint32 rows, uint32 dim, float32 rows.
std::vector<float> read_fbin(const std::string &path, uint32_t &n, uint32_t &d) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + path);
  f.read(reinterpret_cast<char *>(&n), 4);
  f.read(reinterpret_cast<char *>(&d), 4);
  std::vector<float> rows(static_cast<size_t>(n) * d);
  f.read(reinterpret_cast<char *>(rows.data()), static_cast<std::streamsize>(rows.size() * 4));
  if (!f) throw std::runtime_error("truncated " + path);
  return rows;
}

// Ground truth: uint32 rows, uint32 k, rows x k uint32 ids.
std::vector<uint32_t> read_gt(const std::string &path, uint32_t &n, uint32_t &k) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + path);
  f.read(reinterpret_cast<char *>(&n), 4);
  f.read(reinterpret_cast<char *>(&k), 4);
  std::vector<uint32_t> ids(static_cast<size_t>(n) * k);
  f.read(reinterpret_cast<char *>(ids.data()), static_cast<std::streamsize>(ids.size() * 4));
  if (!f) throw std::runtime_error("truncated " + path);
  return ids;
}

katoann::LoadOptions load_options(const Args &a) {
  katoann::LoadOptions o;
  const std::string prec = a.get("precision", "sq16");
  if (prec == "bf16") o.precision = katoann::Precision::kBf16;
  else if (prec != "sq16") throw std::invalid_argument("--precision is sq16 or bf16");
  const std::string eng = a.get("engine", "gpu");  // the CPU engines name the one GPU engine
  if (eng == "avx512") o.use_amx = false;
  else if (eng != "amx" && eng != "gpu") throw std::invalid_argument("--engine is gpu, amx or avx512");
  o.prefix_dims = a.u32("prefix-dims", 0);
  const std::string coarse = a.get("coarse", "batched");
  if (coarse == "flat") o.batched_coarse = false;
  else if (coarse != "batched") throw std::invalid_argument("--coarse is batched or flat");
  o.max_batch = std::max(a.u32("batch", 4096), a.u32("max-batch", 4096));
  o.code_cache = a.has("code-cache");  // PREFIX.gpucodes (an addition to the reference's flags)
  return o;
}

katoann::SearchParams search_params(const Args &a) {
  katoann::SearchParams p;
  p.k = a.u32("k", 10);
  const std::string r = a.get("ranking", "prefix");
  if (r == "full") p.ranking = katoann::Ranking::kFull;
  else if (r == "high") p.ranking = katoann::Ranking::kHighBytes;
  else if (r == "prefix") p.ranking = katoann::Ranking::kPrefix;
  else throw std::invalid_argument("--ranking is prefix, high, or full");
  p.survivors = a.u32("survivors", 32);
  const std::string s = a.get("selection", "threshold");
  if (s == "local") p.selection = katoann::Selection::kLocal;
  else if (s != "threshold") throw std::invalid_argument("--selection is threshold or local");
  return p;
}

// recall@k of ids (one row per query of `qid`) against the first k ground-truth ids.
double recall_at(const std::vector<uint32_t> &ids, const std::vector<uint32_t> &qid, uint32_t k,
                 const std::vector<uint32_t> &gt, uint32_t gk) {
  double hits = 0;
  for (size_t i = 0; i < qid.size(); ++i) {
    const uint32_t *truth = gt.data() + static_cast<size_t>(qid[i]) * gk;
    const std::set<uint32_t> t(truth, truth + k);
    for (uint32_t j = 0; j < k; ++j) hits += t.count(ids[i * k + j]);
  }
  return hits / (static_cast<double>(qid.size()) * k);
}

// The queries to use: --query-ids (whitespace-separated indices) or all.
std::vector<uint32_t> query_ids(const Args &a, uint32_t nq) {
  std::vector<uint32_t> ids;
  const std::string path = a.get("query-ids");
  if (path.empty()) {
    for (uint32_t i = 0; i < nq; ++i) ids.push_back(i);
    return ids;
  }
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open " + path);
  uint32_t id;
  while (f >> id) {
    if (id >= nq) throw std::runtime_error("query id out of range in " + path);
    ids.push_back(id);
  }
  if (ids.empty()) throw std::runtime_error("no query ids in " + path);
  return ids;
}

void set_threads(const Args &a) {
  const uint32_t t = a.u32("threads", 0);
  omp_set_dynamic(0);
  if (t) omp_set_num_threads(static_cast<int>(t));
}

std::vector<float> load_queries(const Args &a, const katoann::Index &idx, uint32_t &nq) {
  uint32_t d = 0;
  std::vector<float> q = read_fbin(a.need("queries"), nq, d);
  if (d != idx.dim()) throw std::runtime_error("query dimension does not match the index");
  if (idx.normalized()) katoann::normalize_rows(q.data(), nq, d);
  return q;
}

int cmd_build(const Args &a) {
  set_threads(a);
  uint32_t n = 0, d = 0;
  std::vector<float> data = read_fbin(a.need("data"), n, d);
  katoann::BuildOptions o;
  o.nlist = a.u32("nlist", 2048);
  o.train_size = a.u32("train-size", 256000);
  o.kmeans_iters = a.u32("iters", 12);
  o.seed = std::stoull(a.get("seed", "0"));
  if (a.has("normalize")) katoann::normalize_rows(data.data(), n, d);
  o.normalized = a.has("normalize") || a.has("normalized");
  const auto t0 = Clock::now();
  katoann::Index::build(data.data(), n, d, o, a.need("out"));
  std::printf("{\"vectors\": %u, \"dim\": %u, \"nlist\": %u, \"build_s\": %.1f}\n", n, d, o.nlist,
              seconds_since(t0));
  return 0;
}

int cmd_search(const Args &a) {
  set_threads(a);
  katoann::Index idx;
  auto t0 = Clock::now();
  idx.load(a.need("index"), load_options(a));
  const double load_s = seconds_since(t0);
  uint32_t nq = 0;
  const std::vector<float> queries = load_queries(a, idx, nq);
  const uint32_t d = idx.dim();
  const std::vector<uint32_t> qid = query_ids(a, nq);
  std::vector<float> q(qid.size() * static_cast<size_t>(d));
  for (size_t i = 0; i < qid.size(); ++i)
    std::memcpy(q.data() + i * d, queries.data() + static_cast<size_t>(qid[i]) * d, d * sizeof(float));
  uint32_t gn = 0, gk = 0;
  std::vector<uint32_t> gt;
  if (!a.get("gt").empty()) gt = read_gt(a.get("gt"), gn, gk);
  katoann::SearchParams p = search_params(a);
  if (!gt.empty() && (gn < nq || gk < p.k)) throw std::runtime_error("ground truth too small");
  const uint32_t batch = a.u32("batch", 4096), repeat = std::max(1u, a.u32("repeat", 3));
  const std::string out = a.get("out");
  std::printf("{\"index\": \"%s\", \"engine\": \"gpu\", \"threads\": %d, \"load_s\": %.1f, "
              "\"memory_gb\": %.2f, \"queries\": %zu, \"prefix_dims\": %u}\n",
              a.need("index").c_str(), omp_get_max_threads(), load_s, idx.memory_bytes() / 1e9,
              qid.size(), idx.prefix_dims());
  const size_t total = qid.size();
  std::vector<uint32_t> ids(total * p.k);
  std::vector<float> dists(total * p.k);
  for (const uint32_t np : u32_list(a.get("nprobe", "64"))) {
    p.nprobe = np;
    auto pass = [&]() {
      for (size_t off = 0; off < total; off += batch) {
        const uint32_t b = static_cast<uint32_t>(std::min<size_t>(batch, total - off));
        idx.search(q.data() + off * d, b, p, ids.data() + off * p.k, dists.data() + off * p.k);
      }
    };
    pass();  // warm-up
    std::vector<double> secs;
    for (uint32_t r = 0; r < repeat; ++r) {
      t0 = Clock::now();
      pass();
      secs.push_back(seconds_since(t0));
    }
    std::sort(secs.begin(), secs.end());
    const double med = secs[secs.size() / 2];
    std::printf("{\"nprobe\": %u, \"k\": %u, \"survivors\": %u, \"batch\": %u, \"qps\": %.1f, "
                "\"seconds_median\": %.4f, \"seconds_min\": %.4f, \"seconds_max\": %.4f",
                np, p.k, p.survivors, batch, total / med, med, secs.front(), secs.back());
    if (!gt.empty()) std::printf(", \"recall\": %.5f", recall_at(ids, qid, p.k, gt, gk));
    std::printf("}\n");
    std::fflush(stdout);
    if (!out.empty()) {  // uint32 rows, uint32 k, ids, dists (tools/katoann.cpp:253-259)
      std::ofstream f(out + ".np" + std::to_string(np) + ".bin", std::ios::binary);
      const uint32_t hdr[2] = {static_cast<uint32_t>(total), p.k};
      f.write(reinterpret_cast<const char *>(hdr), sizeof(hdr));
      f.write(reinterpret_cast<const char *>(ids.data()), static_cast<std::streamsize>(ids.size() * 4));
      f.write(reinterpret_cast<const char *>(dists.data()),
              static_cast<std::streamsize>(dists.size() * 4));
    }
  }
  return 0;
}

// The learned probe budget for `load --budget`: labels the training queries by
// searching the index and trains the model on the GPU (katoann::ProbeModel).
int cmd_budget(const Args &a) {
  set_threads(a);
  katoann::Index idx;
  idx.load(a.need("index"), load_options(a));
  uint32_t nq = 0;
  const std::vector<float> queries = load_queries(a, idx, nq);
  const katoann::SearchParams sp = search_params(a);
  katoann::ProbeTrainOptions o;
  if (!a.get("ladder").empty()) o.ladder = u32_list(a.get("ladder"));
  o.depth = a.u32("depth", std::min(256u, idx.nlist()));
  o.k = sp.k;
  o.label_nprobe = a.u32("label-nprobe", 0);
  if (a.get("label-ranking", "full") == "prefix") o.label_ranking = katoann::Ranking::kPrefix;
  else if (a.get("label-ranking", "full") == "high") o.label_ranking = katoann::Ranking::kHighBytes;
  o.label_survivors = a.u32("label-survivors", 0);
  o.ranking = sp.ranking;
  o.survivors = sp.survivors;
  o.epochs = a.u32("epochs", 24);
  o.batch = a.u32("train-batch", 1024);
  o.seed = std::stoull(a.get("seed", "0"));
  std::vector<uint32_t> ladder;
  for (uint32_t v : o.ladder)
    if (v <= idx.nlist()) ladder.push_back(v);
  o.ladder = ladder;
  const auto t0 = Clock::now();
  const katoann::ProbeModel m = katoann::ProbeModel::train(idx, queries.data(), nq, o);
  m.save(a.need("out"));
  std::vector<uint64_t> hist(m.classes(), 0);
  for (uint8_t l : m.labels()) ++hist[l];
  std::printf("{\"queries\": %u, \"classes\": %u, \"depth\": %u, \"train_s\": %.2f, "
              "\"loss_first\": %.4f, \"loss_last\": %.4f, \"label_histogram\": [",
              nq, m.classes(), m.depth(), seconds_since(t0), m.loss().front(), m.loss().back());
  for (size_t i = 0; i < hist.size(); ++i)
    std::printf("%s%llu", i ? ", " : "", static_cast<unsigned long long>(hist[i]));
  std::printf("]}\n");
  return 0;
}

int cmd_load(const Args &a) {
  set_threads(a);
  katoann::Index idx;
  idx.load(a.need("index"), load_options(a));
  uint32_t nq = 0;
  const std::vector<float> queries = load_queries(a, idx, nq);
  const uint32_t d = idx.dim();
  const std::vector<uint32_t> pool = query_ids(a, nq);
  const katoann::SearchParams sp = search_params(a);
  // per-request k: one value, or a list drawn uniformly per request
  const std::vector<uint32_t> kmix = u32_list(a.get("k-mix", std::to_string(sp.k)));
  if (kmix.empty()) throw std::invalid_argument("empty --k-mix");
  katoann::ProbeModel model;
  katoann::ServerOptions so;
  so.max_batch = std::max(1u, std::min(4096u, a.u32("max-batch", 4096)));
  so.max_in_flight = a.u32("in-flight", 3);
  so.hbm_budget = static_cast<size_t>(a.num("hbm-budget-gb", 0) * 1e9);
  so.max_k = *std::max_element(kmix.begin(), kmix.end());
  so.nprobe = a.u32("nprobe", 64);
  so.ranking = sp.ranking;
  so.survivors = sp.survivors;
  so.max_wait_ms = a.num("max-wait-ms", 0);
  if (!a.get("budget").empty()) {  // learned per-query nprobe, capped at --nprobe
    model = katoann::ProbeModel::load(a.get("budget"));
    so.budget = &model;
    so.budget_threshold = static_cast<float>(a.num("threshold", 0.95));
  }
  const double rate = a.num("rate", 1000);
  const uint32_t n = a.u32("requests", 10000);
  katoann::Server server(idx, so);
  {  // warm-up: one full batch of each k
    std::vector<uint64_t> ids;
    for (uint32_t k : kmix)
      for (uint32_t w = 0; w < std::min<uint32_t>(so.max_batch, static_cast<uint32_t>(pool.size())); ++w)
        ids.push_back(server.submit(queries.data() + static_cast<size_t>(pool[w]) * d, k));
    for (uint64_t id : ids) server.wait(id);
  }
  // Poisson arrivals, queries round-robin from the pool, k uniform over the mix
  const katoann::LoadReport r =
      katoann::run_load(server, queries.data(), d, pool, rate, n, kmix, a.u32("seed", 42));
  std::printf("{\"rate\": %.1f, \"requests\": %u, \"nprobe\": %u, \"engine\": \"gpu\", "
              "\"achieved_qps\": %.1f, \"p50_ms\": %.2f, \"p95_ms\": %.2f, \"p99_ms\": %.2f, "
              "\"max_ms\": %.2f, \"batches\": %llu, \"mean_batch\": %.1f, \"in_flight\": %u, "
              "\"peak_in_flight\": %u, \"peak_hbm_gb\": %.3f, \"learned\": %s, "
              "\"mean_nprobe\": %.2f, \"max_lag_ms\": %.2f, \"max_enqueue_ms\": %.2f, "
              "\"max_batch_gpu_ms\": %.2f}\n",
              rate, n, so.nprobe, r.achieved_qps, r.p50_ms, r.p95_ms, r.p99_ms, r.max_ms,
              static_cast<unsigned long long>(r.batches), r.mean_batch, so.max_in_flight,
              r.peak_in_flight, r.peak_hbm_bytes / 1e9, so.budget ? "true" : "false",
              r.mean_nprobe, r.max_lag_ms, r.max_enqueue_ms, r.max_batch_gpu_ms);
  return 0;
}

void usage() {
  std::fprintf(stderr,
               "usage: katoann build  --data BASE.fbin --out PREFIX [--nlist 2048] [--normalize]\n"
               "                      [--train-size 256000] [--iters 12] [--seed 0] [--threads T]\n"
               "       katoann search --index PREFIX --queries Q.fbin [--gt GT.bin] [--k 10]\n"
               "                      [--nprobe 64,128] [--ranking prefix|high|full] [--survivors 32]\n"
               "                      [--prefix-dims D] [--selection threshold|local] [--batch 4096]\n"
               "                      [--precision sq16] [--engine gpu] [--coarse batched]\n"
               "                      [--repeat 3] [--threads T] [--query-ids FILE] [--out PREFIX]\n"
               "                      [--code-cache]\n"
               "       katoann load   --index PREFIX --queries Q.fbin --rate QPS [--requests 10000]\n"
               "                      [--nprobe 64] [--max-batch 4096] [--seed 42] [--k-mix 10,100]\n"
               "                      [--in-flight 3] [--hbm-budget-gb G] [--max-wait-ms 0]\n"
               "                      [--budget MODEL.kprb --threshold 0.95] and the search flags\n"
               "       katoann budget --index PREFIX --queries TRAIN.fbin --out MODEL.kprb\n"
               "                      [--ladder 8,16,...] [--depth 256] [--label-nprobe N]\n"
               "                      [--label-ranking full|prefix] [--label-survivors S]\n"
               "                      [--epochs 24] [--train-batch 1024] and the search flags\n");
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 2) {
    usage();
    return 2;
  }
  try {
    const std::string cmd = argv[1];
    const Args a = parse(argc, argv, 2);
    if (cmd == "build") return cmd_build(a);
    if (cmd == "search") return cmd_search(a);
    if (cmd == "load") return cmd_load(a);
    if (cmd == "budget") return cmd_budget(a);
    usage();
    return 2;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "katoann: %s\n", e.what());
    return 1;
  }
}
