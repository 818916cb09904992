/* C ABI of libkatoann.so, the host library around katoann::Index. This is the
 * surface a foreign-function binding uses (the Python module binds it with
 * ctypes); it replaces the reference's pybind11 module
 * (python/katoann_module.cpp:34-129) one call for one call. Statuses: 0 ok,
 * -1 invalid argument (std::invalid_argument), -2 runtime error
 * (std::runtime_error, CUDA), -3 logic error (std::logic_error), -5 a
 * bounded wait in a device pipeline ran out (katoann::timeout_error);
 * katoann_last_error() gives the message. Pointers are host memory unless
 * named d_*. */
#ifndef KATOANN_C_H_
#define KATOANN_C_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

const char *katoann_last_error(void);

/* katoann.amx_available (python/katoann_module.cpp:36-37): always 0 here. */
int katoann_amx_available(void);

/* katoann.build (python/katoann_module.cpp:39-58). */
int katoann_build(const float *data, uint32_t n, uint32_t dim, uint32_t nlist,
                  uint32_t train_size, uint32_t kmeans_iters, uint64_t seed, int normalized,
                  uint32_t rotation_sample, uint32_t jacobi_sweeps, const char *prefix);

/* The partition katoann_build writes, computed on the GPU without writing
 * files (no counterpart in the reference's module): data (n x dim, host
 * memory, or device memory when on_device) -> centroids (host, nlist x dim),
 * assign (host, n: each vector's list), rotation (host, dim x dim; *rotated
 * is 0 when none was computed) and *head_dims (the default prefix dims). */
int katoann_build_partition(const float *data, int on_device, uint32_t n, uint32_t dim,
                            uint32_t nlist, uint32_t train_size, uint32_t kmeans_iters,
                            uint64_t seed, uint32_t rotation_sample, uint32_t jacobi_sweeps,
                            float *centroids, uint32_t *assign, float *rotation,
                            uint32_t *rotated, uint32_t *head_dims);

void *katoann_index_new(void);
void katoann_index_free(void *index);

/* Index.load (python/katoann_module.cpp:62-76); precision 0 sq16, 1 bf16. */
int katoann_index_load(void *index, const char *prefix, int precision, int use_amx,
                       uint32_t prefix_dims, int batched_coarse, uint32_t max_batch);

/* katoann_index_load through the device-code cache PREFIX.gpucodes
 * (LoadOptions::code_cache): loads the codes when they were made from the
 * same files with the same prefix_dims, else loads the files and writes them. */
int katoann_index_load_cached(void *index, const char *prefix, uint32_t prefix_dims,
                              uint32_t max_batch);

/* Index::save_codes / Index::load_codes: the loaded index as it lives on the
 * device, to and from one file (no counterpart in the reference). */
int katoann_index_save_codes(void *index, const char *path);
int katoann_index_load_codes(void *index, const char *path, uint32_t max_batch);

/* An index from arrays (lists concatenated in list order); on_device selects
 * device pointers for ids, vectors, centroids and rotation. */
int katoann_index_load_arrays(void *index, uint32_t dim, uint32_t nlist, uint32_t npts,
                              int normalized, const float *centroids, const uint32_t *list_sizes,
                              const uint32_t *ids, const float *vectors, const float *rotation,
                              int has_dimc, uint32_t head_dims, int on_device,
                              uint32_t prefix_dims, uint32_t max_batch);

/* Index.search (python/katoann_module.cpp:77-119) without the normalisation,
 * which the caller applies (katoann_normalize_rows). ranking 0 full, 1 high,
 * 2 prefix; selection 0 threshold, 1 local. */
int katoann_index_search(void *index, const float *queries, uint32_t nq, uint32_t k,
                         uint32_t nprobe, int ranking, uint32_t survivors, int selection,
                         uint32_t *ids, float *dists);

/* The same on device memory and a caller stream (cudaStream_t, NULL = the
 * index's stream); asynchronous. timer: katoann_gpu_timer_create() or NULL. */
int katoann_index_search_device(void *index, const float *d_queries, uint32_t nq, uint32_t k,
                                uint32_t nprobe, int ranking, uint32_t survivors, int selection,
                                uint32_t *d_ids, float *d_dists, void *stream, void *timer);

/* Index.search with a per-query nprobe (SearchParams::budget /
 * nprobe_per_query / nprobe_used; no counterpart in the reference): model is
 * a katoann_probe_* handle or NULL, nprobe_in (nq values, capped at nprobe)
 * or NULL, nprobe_out (nq values) or NULL; graph != 0 replays each pass's
 * kernels as a captured CUDA graph (SearchParams::graph). */
int katoann_index_search_budget(void *index, const float *queries, uint32_t nq, uint32_t k,
                                uint32_t nprobe, int ranking, uint32_t survivors, int selection,
                                const void *model, float threshold, const uint32_t *nprobe_in,
                                uint32_t *nprobe_out, uint32_t *ids, float *dists, int graph);

/* katoann_index_search_device with the per-query nprobe of
 * katoann_index_search_budget (d_nprobe_in / d_nprobe_out: device memory);
 * graph != 0 replays a captured CUDA graph of the call (SearchParams::graph). */
int katoann_index_search_device_budget(void *index, const float *d_queries, uint32_t nq,
                                       uint32_t k, uint32_t nprobe, int ranking,
                                       uint32_t survivors, int selection, const void *model,
                                       float threshold, const uint32_t *d_nprobe_in,
                                       uint32_t *d_nprobe_out, uint32_t *d_ids, float *d_dists,
                                       void *stream, void *timer, int graph);

/* Index::autotune: out[4] = {seed rows, split weight, item width,
 * microseconds per search}; model NULL: fixed nprobe. */
int katoann_index_autotune(void *index, const float *queries, uint32_t nq, uint32_t k,
                           uint32_t nprobe, int ranking, uint32_t survivors, const void *model,
                           float threshold, uint32_t *out);

/* ------------------------------------------------ learned probe budget
 * katoann::ProbeModel (include/katoann/probe.h). train: labels nq queries by
 * searching the index and trains on the device; options as in
 * ProbeTrainOptions (rankings 0 full, 1 high, 2 prefix). */
int katoann_probe_train(void *index, const float *queries, uint32_t nq, const uint32_t *ladder,
                        uint32_t nladder, uint32_t depth, uint32_t k, uint32_t label_nprobe,
                        int label_ranking, uint32_t label_survivors, int ranking,
                        uint32_t survivors, uint32_t epochs, uint32_t batch, float lr,
                        float weight_decay, uint64_t seed, void **model);
/* ProbeModel::fit on given raw features (n x 64) and class labels. */
int katoann_probe_fit(const float *z, const uint8_t *labels, uint32_t n, const uint32_t *ladder,
                      uint32_t nladder, uint32_t depth, uint32_t epochs, uint32_t batch,
                      float lr, float weight_decay, uint64_t seed, void **model);
int katoann_probe_load(const char *path, void **model);
int katoann_probe_save(const void *model, const char *path);
void katoann_probe_free(void *model);
/* info[2] = {classes, depth}; ladder and ranks (64) may be NULL. */
int katoann_probe_info(const void *model, uint32_t *info, uint32_t *ladder, uint32_t *ranks);
/* Training record: labels (n values) and per-epoch loss (epochs values);
 * *n and *epochs receive the counts when the arrays are NULL. */
int katoann_probe_record(const void *model, uint8_t *labels, uint32_t *n, float *loss,
                         uint32_t *epochs);
/* The weights as the device uses them: shift, scale (64 each), w1 (64 x 256
 * bf16), b1 (256), w2 (256 x 256 bf16), b2 (256), w3 (256 x classes bf16),
 * b3 (classes). */
int katoann_probe_weights(const void *model, float *shift, float *scale, uint16_t *w1, float *b1,
                          uint16_t *w2, float *b2, uint16_t *w3, float *b3);
/* Raw features of nq queries at `depth` (nq x 64) and the model's output on
 * feature rows (probs n x classes and nprobe n, either may be NULL). */
int katoann_probe_features(void *index, const float *queries, uint32_t nq, uint32_t depth,
                           float *z);
int katoann_probe_predict(const void *model, const float *z, uint32_t n, float threshold,
                          uint32_t cap, float *probs, uint32_t *nprobe);

/* ------------------------------------------- continuous-batching server
 * katoann::Server (include/katoann/server.h); supersedes the serial loop of
 * the reference's `katoann load` (tools/katoann.cpp:304-321). hbm_budget 0:
 * room for max_in_flight full batches; model NULL: fixed nprobe. graphs != 0:
 * replay captured searches (ServerOptions::graphs), those of the n_warm k in
 * warm_k captured up front. */
int katoann_server_new(void *index, uint32_t max_batch, uint32_t max_in_flight,
                       uint64_t hbm_budget, uint32_t max_k, uint32_t nprobe, int ranking,
                       uint32_t survivors, const void *model, float threshold,
                       double max_wait_ms, int graphs, const uint32_t *warm_k, uint32_t n_warm,
                       void **server);
void katoann_server_free(void *server);
/* Queues one query (dim floats) with its k; *id receives the request id. */
int katoann_server_submit(void *server, const float *query, uint32_t k, uint64_t *id);
/* Blocks until request `id` is done: ids and dists (k each), its nprobe and
 * its latency from submit to completion. */
int katoann_server_wait(void *server, uint64_t id, uint32_t *ids, float *dists,
                        uint32_t *nprobe, double *latency_ms);
/* The same without blocking: *done = 0 when the request is still running. */
int katoann_server_poll(void *server, uint64_t id, uint32_t *ids, float *dists,
                        uint32_t *nprobe, double *latency_ms, int *done);
int katoann_server_drain(void *server);
/* stats[9] = {requests, batches, peak_in_flight, peak_hbm_bytes, mean_batch x 1000,
 * max_enqueue_ms x 1000, max_batch_gpu_ms x 1000, graph_batches, graphs} */
int katoann_server_stats(void *server, uint64_t *stats);
/* katoann::run_load: n Poisson arrivals at `rate` from a native client, queries
 * round-robin from queries (nq x dim), k uniform over kmix. report[13] =
 * {achieved_qps, p50_ms, p95_ms, p99_ms, max_ms, batches, mean_batch,
 * mean_nprobe, peak_in_flight, peak_hbm_bytes, max_lag_ms, max_enqueue_ms,
 * max_batch_gpu_ms}. */
int katoann_server_load(void *server, const float *queries, uint32_t nq, uint32_t dim, double rate,
                        uint32_t n, const uint32_t *kmix, uint32_t nk, uint64_t seed,
                        double *report);

/* info[8] = {dim, nlist, size, prefix_dims, rotated, normalized, batched_coarse, engine=2} */
int katoann_index_info(void *index, uint32_t *info);
size_t katoann_index_memory_bytes(void *index);
int katoann_index_list_sizes(void *index, uint32_t *sizes);
/* [0] coarse boundary ties, [1] survivor boundary ties of the last search. */
int katoann_index_stats(void *index, uint64_t *stats, uint32_t n);
/* The device view (const katoann_gpu_index *) for direct kernel calls. */
const void *katoann_index_device_view(void *index);

/* Unit-length rows as the reference's CLI and module compute them. */
void katoann_normalize_rows(float *rows, size_t n, uint32_t dim);

/* float(double(l2) * step_sq) by the integer method the kernels use. */
float katoann_dist_value(int64_t l2, double step_sq);

#ifdef __cplusplus
}
#endif

#endif /* KATOANN_C_H_ */
