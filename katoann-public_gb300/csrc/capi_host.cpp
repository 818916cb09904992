// extern "C" surface of libkatoann.so (include/katoann_c.h).
#include <algorithm>
#include <stdexcept>
#include <string>

#include "dist_value.h"
#include "katoann/index.h"
#include "katoann/probe.h"
#include "katoann/server.h"
#include "katoann_c.h"

namespace {

thread_local std::string g_error;

template <class F>
int guarded(F &&f) {
  try {
    f();
    return 0;
  } catch (const std::invalid_argument &e) {
    g_error = e.what();
    return -1;
  } catch (const katoann::timeout_error &e) {
    g_error = e.what();
    return -5;
  } catch (const std::logic_error &e) {
    g_error = e.what();
    return -3;
  } catch (const std::exception &e) {
    g_error = e.what();
    return -2;
  }
}

katoann::Index *I(void *p) { return static_cast<katoann::Index *>(p); }
const katoann::ProbeModel *M(const void *p) { return static_cast<const katoann::ProbeModel *>(p); }

katoann::Ranking ranking_of(int r) {
  return r == 0 ? katoann::Ranking::kFull
         : r == 1 ? katoann::Ranking::kHighBytes
                  : katoann::Ranking::kPrefix;
}

katoann::ProbeTrainOptions train_options(const uint32_t *ladder, uint32_t nladder, uint32_t depth,
                                         uint32_t epochs, uint32_t batch, float lr, float wd,
                                         uint64_t seed) {
  katoann::ProbeTrainOptions o;
  if (ladder) o.ladder.assign(ladder, ladder + nladder);
  if (depth) o.depth = depth;
  if (epochs) o.epochs = epochs;
  if (batch) o.batch = batch;
  if (lr > 0) o.lr = lr;
  if (wd >= 0) o.weight_decay = wd;
  o.seed = seed;
  return o;
}

katoann::SearchParams params(uint32_t k, uint32_t nprobe, int ranking, uint32_t survivors,
                             int selection) {
  katoann::SearchParams p;
  p.k = k;
  p.nprobe = nprobe;
  p.ranking = ranking == 0 ? katoann::Ranking::kFull
              : ranking == 1 ? katoann::Ranking::kHighBytes
                             : katoann::Ranking::kPrefix;
  p.survivors = survivors;
  p.selection = selection == 1 ? katoann::Selection::kLocal : katoann::Selection::kThreshold;
  return p;
}

}  // namespace

extern "C" {

const char *katoann_last_error(void) { return g_error.c_str(); }

int katoann_amx_available(void) { return katoann::amx_available() ? 1 : 0; }

int katoann_build(const float *data, uint32_t n, uint32_t dim, uint32_t nlist, uint32_t train_size,
                  uint32_t kmeans_iters, uint64_t seed, int normalized, uint32_t rotation_sample,
                  uint32_t jacobi_sweeps, const char *prefix) {
  return guarded([&] {
    katoann::BuildOptions o;
    o.nlist = nlist;
    o.train_size = train_size;
    o.kmeans_iters = kmeans_iters;
    o.seed = seed;
    o.normalized = normalized != 0;
    o.rotation_sample = rotation_sample;
    o.jacobi_sweeps = jacobi_sweeps;
    katoann::Index::build(data, n, dim, o, prefix);
  });
}

int katoann_build_partition(const float *data, int on_device, uint32_t n, uint32_t dim,
                            uint32_t nlist, uint32_t train_size, uint32_t kmeans_iters,
                            uint64_t seed, uint32_t rotation_sample, uint32_t jacobi_sweeps,
                            float *centroids, uint32_t *assign, float *rotation,
                            uint32_t *rotated, uint32_t *head_dims) {
  return guarded([&] {
    katoann::BuildOptions o;
    o.nlist = nlist;
    o.train_size = train_size;
    o.kmeans_iters = kmeans_iters;
    o.seed = seed;
    o.rotation_sample = rotation_sample;
    o.jacobi_sweeps = jacobi_sweeps;
    const katoann::BuildResult b = katoann::Index::partition(data, n, dim, o, on_device != 0);
    std::copy(b.centroids.begin(), b.centroids.end(), centroids);
    std::copy(b.assign.begin(), b.assign.end(), assign);
    *rotated = b.rotation.empty() ? 0u : 1u;
    if (!b.rotation.empty()) std::copy(b.rotation.begin(), b.rotation.end(), rotation);
    *head_dims = b.head_dims;
  });
}

void *katoann_index_new(void) { return new katoann::Index(); }
void katoann_index_free(void *index) { delete I(index); }

int katoann_index_load(void *index, const char *prefix, int precision, int use_amx,
                       uint32_t prefix_dims, int batched_coarse, uint32_t max_batch) {
  return guarded([&] {
    katoann::LoadOptions o;
    o.precision = precision == 1 ? katoann::Precision::kBf16 : katoann::Precision::kSq16;
    o.use_amx = use_amx != 0;
    o.prefix_dims = prefix_dims;
    o.batched_coarse = batched_coarse != 0;
    if (max_batch) o.max_batch = max_batch;
    I(index)->load(prefix, o);
  });
}

int katoann_index_load_cached(void *index, const char *prefix, uint32_t prefix_dims,
                              uint32_t max_batch) {
  return guarded([&] {
    katoann::LoadOptions o;
    o.prefix_dims = prefix_dims;
    o.code_cache = true;
    if (max_batch) o.max_batch = max_batch;
    I(index)->load(prefix, o);
  });
}

int katoann_index_save_codes(void *index, const char *path) {
  return guarded([&] { I(index)->save_codes(path); });
}

int katoann_index_load_codes(void *index, const char *path, uint32_t max_batch) {
  return guarded([&] {
    katoann::LoadOptions o;
    if (max_batch) o.max_batch = max_batch;
    I(index)->load_codes(path, o);
  });
}

int katoann_index_load_arrays(void *index, uint32_t dim, uint32_t nlist, uint32_t npts,
                              int normalized, const float *centroids, const uint32_t *list_sizes,
                              const uint32_t *ids, const float *vectors, const float *rotation,
                              int has_dimc, uint32_t head_dims, int on_device,
                              uint32_t prefix_dims, uint32_t max_batch) {
  return guarded([&] {
    katoann::IndexArrays a;
    a.dim = dim;
    a.nlist = nlist;
    a.npts = npts;
    a.normalized = normalized != 0;
    a.centroids = centroids;
    a.list_sizes = list_sizes;
    a.ids = ids;
    a.vectors = vectors;
    a.rotation = rotation;
    a.has_dimc = has_dimc != 0;
    a.head_dims = head_dims;
    a.on_device = on_device != 0;
    katoann::LoadOptions o;
    o.prefix_dims = prefix_dims;
    if (max_batch) o.max_batch = max_batch;
    I(index)->load_arrays(a, o);
  });
}

int katoann_index_search(void *index, const float *queries, uint32_t nq, uint32_t k,
                         uint32_t nprobe, int ranking, uint32_t survivors, int selection,
                         uint32_t *ids, float *dists) {
  return guarded([&] {
    I(index)->search(queries, nq, params(k, nprobe, ranking, survivors, selection), ids, dists);
  });
}

int katoann_index_search_device(void *index, const float *d_queries, uint32_t nq, uint32_t k,
                                uint32_t nprobe, int ranking, uint32_t survivors, int selection,
                                uint32_t *d_ids, float *d_dists, void *stream, void *timer) {
  return guarded([&] {
    I(index)->search_device(d_queries, nq, params(k, nprobe, ranking, survivors, selection), d_ids,
                            d_dists, stream, timer);
  });
}

int katoann_index_info(void *index, uint32_t *info) {
  const katoann::Index &x = *I(index);
  info[0] = x.dim();
  info[1] = x.nlist();
  info[2] = x.size();
  info[3] = x.prefix_dims();
  info[4] = x.rotated() ? 1 : 0;
  info[5] = x.normalized() ? 1 : 0;
  info[6] = x.batched_coarse() ? 1 : 0;
  info[7] = 2;
  return 0;
}

size_t katoann_index_memory_bytes(void *index) { return I(index)->memory_bytes(); }

int katoann_index_list_sizes(void *index, uint32_t *sizes) {
  const auto v = I(index)->list_sizes();
  for (size_t i = 0; i < v.size(); ++i) sizes[i] = v[i];
  return 0;
}

int katoann_index_stats(void *index, uint64_t *stats, uint32_t n) {
  return guarded([&] {
    const auto v = I(index)->last_search_stats();
    for (uint32_t i = 0; i < n && i < v.size(); ++i) stats[i] = v[i];
  });
}

const void *katoann_index_device_view(void *index) { return I(index)->device_view(); }

int katoann_server_new(void *index, uint32_t max_batch, uint32_t max_in_flight,
                       uint64_t hbm_budget, uint32_t max_k, uint32_t nprobe, int ranking,
                       uint32_t survivors, const void *model, float threshold,
                       double max_wait_ms, int graphs, const uint32_t *warm_k, uint32_t n_warm,
                       void **server) {
  return guarded([&] {
    katoann::ServerOptions o;
    o.max_batch = max_batch;
    o.max_in_flight = max_in_flight;
    o.hbm_budget = hbm_budget;
    o.max_k = max_k;
    o.nprobe = nprobe;
    o.ranking = ranking_of(ranking);
    o.survivors = survivors;
    o.budget = M(model);
    o.budget_threshold = threshold;
    o.max_wait_ms = max_wait_ms;
    o.graphs = graphs != 0;
    if (warm_k) o.warm_k.assign(warm_k, warm_k + n_warm);
    *server = new katoann::Server(*I(index), o);
  });
}

void katoann_server_free(void *server) { delete static_cast<katoann::Server *>(server); }

namespace {
katoann::Server *SV(void *p) { return static_cast<katoann::Server *>(p); }
void put_result(const katoann::ServerResult &r, uint32_t *ids, float *dists, uint32_t *nprobe,
                double *latency_ms) {
  if (ids) std::copy(r.ids.begin(), r.ids.end(), ids);
  if (dists) std::copy(r.dists.begin(), r.dists.end(), dists);
  if (nprobe) *nprobe = r.nprobe;
  if (latency_ms) *latency_ms = r.latency_ms;
}
}  // namespace

int katoann_server_submit(void *server, const float *query, uint32_t k, uint64_t *id) {
  return guarded([&] { *id = SV(server)->submit(query, k); });
}

int katoann_server_wait(void *server, uint64_t id, uint32_t *ids, float *dists,
                        uint32_t *nprobe, double *latency_ms) {
  return guarded([&] { put_result(SV(server)->wait(id), ids, dists, nprobe, latency_ms); });
}

int katoann_server_poll(void *server, uint64_t id, uint32_t *ids, float *dists,
                        uint32_t *nprobe, double *latency_ms, int *done) {
  return guarded([&] {
    katoann::ServerResult r;
    *done = SV(server)->poll(id, &r) ? 1 : 0;
    if (*done) put_result(r, ids, dists, nprobe, latency_ms);
  });
}

int katoann_server_drain(void *server) {
  return guarded([&] { SV(server)->drain(); });
}

int katoann_server_load(void *server, const float *queries, uint32_t nq, uint32_t dim, double rate,
                        uint32_t n, const uint32_t *kmix, uint32_t nk, uint64_t seed,
                        double *report) {
  return guarded([&] {
    std::vector<uint32_t> pool(nq);
    for (uint32_t i = 0; i < nq; ++i) pool[i] = i;
    const katoann::LoadReport r = katoann::run_load(*SV(server), queries, dim, pool, rate, n,
                                                    std::vector<uint32_t>(kmix, kmix + nk), seed);
    const double v[13] = {r.achieved_qps,   r.p50_ms,      r.p95_ms,
                          r.p99_ms,         r.max_ms,      static_cast<double>(r.batches),
                          r.mean_batch,     r.mean_nprobe, static_cast<double>(r.peak_in_flight),
                          static_cast<double>(r.peak_hbm_bytes), r.max_lag_ms,
                          r.max_enqueue_ms, r.max_batch_gpu_ms};
    std::copy(v, v + 13, report);
  });
}

int katoann_server_stats(void *server, uint64_t *stats) {
  return guarded([&] {
    const katoann::ServerStats s = SV(server)->stats();
    stats[0] = s.requests;
    stats[1] = s.batches;
    stats[2] = s.peak_in_flight;
    stats[3] = s.peak_hbm_bytes;
    stats[4] = static_cast<uint64_t>(s.mean_batch * 1000.0);
    stats[5] = static_cast<uint64_t>(s.max_enqueue_ms * 1000.0);
    stats[6] = static_cast<uint64_t>(s.max_batch_gpu_ms * 1000.0);
    stats[7] = s.graph_batches;
    stats[8] = s.graphs;
  });
}

int katoann_index_search_budget(void *index, const float *queries, uint32_t nq, uint32_t k,
                                uint32_t nprobe, int ranking, uint32_t survivors, int selection,
                                const void *model, float threshold, const uint32_t *nprobe_in,
                                uint32_t *nprobe_out, uint32_t *ids, float *dists, int graph) {
  return guarded([&] {
    katoann::SearchParams p = params(k, nprobe, ranking, survivors, selection);
    p.budget = M(model);
    p.budget_threshold = threshold;
    p.nprobe_per_query = nprobe_in;
    p.nprobe_used = nprobe_out;
    p.graph = graph != 0;
    I(index)->search(queries, nq, p, ids, dists);
  });
}

int katoann_index_search_device_budget(void *index, const float *d_queries, uint32_t nq,
                                       uint32_t k, uint32_t nprobe, int ranking,
                                       uint32_t survivors, int selection, const void *model,
                                       float threshold, const uint32_t *d_nprobe_in,
                                       uint32_t *d_nprobe_out, uint32_t *d_ids, float *d_dists,
                                       void *stream, void *timer, int graph) {
  return guarded([&] {
    katoann::SearchParams p = params(k, nprobe, ranking, survivors, selection);
    p.budget = M(model);
    p.budget_threshold = threshold;
    p.nprobe_per_query = d_nprobe_in;
    p.nprobe_used = d_nprobe_out;
    p.graph = graph != 0;
    I(index)->search_device(d_queries, nq, p, d_ids, d_dists, stream, timer);
  });
}

int katoann_index_autotune(void *index, const float *queries, uint32_t nq, uint32_t k,
                           uint32_t nprobe, int ranking, uint32_t survivors, const void *model,
                           float threshold, uint32_t *out) {
  return guarded([&] {
    katoann::SearchParams p = params(k, nprobe, ranking, survivors, 0);
    p.budget = M(model);
    p.budget_threshold = threshold;
    const katoann::Index::Tuning t = I(index)->autotune(queries, nq, p);
    out[0] = t.seed_rows;
    out[1] = t.schedule;
    out[2] = t.width;
    out[3] = static_cast<uint32_t>(t.us_per_search);
  });
}

int katoann_probe_train(void *index, const float *queries, uint32_t nq, const uint32_t *ladder,
                        uint32_t nladder, uint32_t depth, uint32_t k, uint32_t label_nprobe,
                        int label_ranking, uint32_t label_survivors, int ranking,
                        uint32_t survivors, uint32_t epochs, uint32_t batch, float lr,
                        float weight_decay, uint64_t seed, void **model) {
  return guarded([&] {
    katoann::ProbeTrainOptions o =
        train_options(ladder, nladder, depth, epochs, batch, lr, weight_decay, seed);
    if (k) o.k = k;
    o.label_nprobe = label_nprobe;
    o.label_ranking = ranking_of(label_ranking);
    o.label_survivors = label_survivors;
    o.ranking = ranking_of(ranking);
    if (survivors) o.survivors = survivors;
    *model = new katoann::ProbeModel(katoann::ProbeModel::train(*I(index), queries, nq, o));
  });
}

int katoann_probe_fit(const float *z, const uint8_t *labels, uint32_t n, const uint32_t *ladder,
                      uint32_t nladder, uint32_t depth, uint32_t epochs, uint32_t batch,
                      float lr, float weight_decay, uint64_t seed, void **model) {
  return guarded([&] {
    const katoann::ProbeTrainOptions o =
        train_options(ladder, nladder, depth, epochs, batch, lr, weight_decay, seed);
    *model = new katoann::ProbeModel(katoann::ProbeModel::fit(z, labels, n, o));
  });
}

int katoann_probe_load(const char *path, void **model) {
  return guarded([&] { *model = new katoann::ProbeModel(katoann::ProbeModel::load(path)); });
}

int katoann_probe_save(const void *model, const char *path) {
  return guarded([&] { M(model)->save(path); });
}

void katoann_probe_free(void *model) { delete static_cast<katoann::ProbeModel *>(model); }

int katoann_probe_info(const void *model, uint32_t *info, uint32_t *ladder, uint32_t *ranks) {
  return guarded([&] {
    const katoann::ProbeModel &m = *M(model);
    info[0] = m.classes();
    info[1] = m.depth();
    if (ladder) std::copy(m.ladder().begin(), m.ladder().end(), ladder);
    if (ranks) std::copy(m.feature_ranks().begin(), m.feature_ranks().end(), ranks);
  });
}

int katoann_probe_record(const void *model, uint8_t *labels, uint32_t *n, float *loss,
                         uint32_t *epochs) {
  return guarded([&] {
    const katoann::ProbeModel &m = *M(model);
    if (labels) std::copy(m.labels().begin(), m.labels().end(), labels);
    if (n) *n = static_cast<uint32_t>(m.labels().size());
    if (loss) std::copy(m.loss().begin(), m.loss().end(), loss);
    if (epochs) *epochs = static_cast<uint32_t>(m.loss().size());
  });
}

int katoann_probe_weights(const void *model, float *shift, float *scale, uint16_t *w1, float *b1,
                          uint16_t *w2, float *b2, uint16_t *w3, float *b3) {
  return guarded([&] { M(model)->weights(shift, scale, w1, b1, w2, b2, w3, b3); });
}

int katoann_probe_features(void *index, const float *queries, uint32_t nq, uint32_t depth,
                           float *z) {
  return guarded([&] { katoann::ProbeModel::features(*I(index), queries, nq, depth, z); });
}

int katoann_probe_predict(const void *model, const float *z, uint32_t n, float threshold,
                          uint32_t cap, float *probs, uint32_t *nprobe) {
  return guarded([&] { M(model)->predict(z, n, threshold, cap, probs, nprobe); });
}

void katoann_normalize_rows(float *rows, size_t n, uint32_t dim) {
  katoann::normalize_rows(rows, n, dim);
}

float katoann_dist_value(int64_t l2, double step_sq) {
  return kato::dist_value(l2, kato::make_dist_scale(step_sq));
}

}  // extern "C"
