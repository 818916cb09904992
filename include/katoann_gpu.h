/* C ABI of libkatoann_gpu.so: the sm_103a kernels of KatoANN's batched IVF
 * search over 16-bit split-byte codes.
 *
 * Plain pointers and sizes only. Every pointer named d_* is device memory;
 * every call is asynchronous on the given stream (0 = the legacy default
 * stream) unless it says otherwise. Calls return 0 on success or a negative
 * status and never throw:
 *   KATO_EINVAL  bad argument       (the reference throws std::invalid_argument)
 *   KATO_ERUNTIME CUDA/runtime error (std::runtime_error)
 *   KATO_ELOGIC  call out of order   (std::logic_error)
 *   KATO_ENOMEM  workspace too small or allocation failed
 *   KATO_ETIMEOUT a bounded pipeline wait inside a kernel ran out (the
 *                kernel returned without finishing; results are invalid)
 * katoann_gpu_last_error() gives the message of the calling thread's last
 * failure.
 *
 * Codes are stored row-major, one row per database vector, lists concatenated
 * in list order (list c owns rows [list_off[c], list_off[c+1])). The high
 * bytes and the low bytes of the 16-bit codes are two planes of dc bytes per
 * row (dc = dim rounded up to 64, padding bytes zero). The reference packs the
 * same bytes in AMX tile order (src/kernels.cpp:263-275); row-major rows are
 * what TMA and coalesced loads want on the GPU. */
#ifndef KATOANN_GPU_H_
#define KATOANN_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *katoann_stream_t; /* = cudaStream_t */

enum {
  KATO_OK = 0,
  KATO_EINVAL = -1,
  KATO_ERUNTIME = -2,
  KATO_ELOGIC = -3,
  KATO_ENOMEM = -4,
  KATO_ETIMEOUT = -5  /* a bounded wait in a device pipeline ran out */
};

/* Ranking of SearchParams (include/katoann/index.h:45-49 of the reference). */
enum { KATO_RANK_FULL = 0, KATO_RANK_HIGH = 1, KATO_RANK_PREFIX = 2 };

/* A device-resident index, as the host library uploads it. All arrays are
 * owned by the caller (the host Index). */
typedef struct {
  uint32_t dim, dc, nlist, npts;
  uint32_t head_dims;    /* prefix dims of the ranking pass, 0 if none */
  uint32_t rotated;      /* queries are rotated by d_rotation first */
  uint32_t max_list;     /* largest list size */
  uint32_t reserved;
  float lo;              /* global minimum of the rotated list values */
  float pad;
  double inv_step;       /* 65535 / (hi - lo) */
  double step_sq;        /* ((hi - lo) / 65535)^2 */
  const float *d_rotation;   /* dim x dim, row j = basis j; NULL if !rotated */
  const uint8_t *d_hi;       /* npts x dc */
  const uint8_t *d_lo;       /* npts x dc */
  const int64_t *d_norm;     /* npts: sum of code^2 */
  const int64_t *d_hinorm;   /* npts: sum of high byte^2 over dc */
  const int64_t *d_headnorm; /* npts: sum of high byte^2 over head_dims; NULL if none */
  const uint32_t *d_ids;     /* npts */
  const uint32_t *d_list_off;/* nlist + 1 */
  const uint8_t *d_chi;      /* nlist x dc, centroids coded with the database scale */
  const uint8_t *d_clo;      /* nlist x dc */
  const int64_t *d_cnorm;    /* nlist */
  /* Optional (NULL: the coarse step runs on the CUDA cores): the centroid
   * planes re-centred to (byte - 128) as fp16, nlist x dc each, and the
   * per-centroid term of the tensor-core coarse product; see
   * katoann_gpu_centre_planes. */
  const uint16_t *d_chi16;
  const uint16_t *d_clo16;
  const int64_t *d_cterm;
  /* Optional (NULL: each search transposes d_rotation): d_rotation in the
   * k-major layout the query rotation stages from; see
   * katoann_gpu_rotation_kmajor. */
  const float *d_rotation_t;
} katoann_gpu_index;

const char *katoann_gpu_last_error(void);
int katoann_gpu_version(void);

/* out[i][j] = <in_i, rot_j> with the reference's float arithmetic
 * (rotate_rows, src/index.cpp:214-270, and rotate_rows_serial, :139-180,
 * which give identical bits), nrows x d row-major in and out. */
int katoann_gpu_rotate_rows(const float *d_in, uint32_t nrows, uint32_t d, const float *d_rot,
                            float *d_out, katoann_stream_t stream);

/* d_rot (d x d, row j = basis j) in the k-major layout the search's query
 * rotation reads: entry [k][j] = rot[j][k] for k < (d & ~15), j < (d & ~3),
 * rows of round_up(d & ~3, 32) floats, zero beyond d & ~3. Made once per index
 * (katoann_gpu_index.d_rotation_t) instead of once per search;
 * katoann_gpu_rotation_kmajor_bytes(d) bytes at d_out. */
size_t katoann_gpu_rotation_kmajor_bytes(uint32_t d);
int katoann_gpu_rotation_kmajor(const float *d_rot, uint32_t d, float *d_out,
                                katoann_stream_t stream);

/* Global minimum and maximum of n floats, written to h_out[0..1] (host);
 * d_scratch is 8 bytes of device memory. Synchronous. Replaces the reduction
 * of quantize_sq16_ (src/index.cpp:634-645). */
int katoann_gpu_minmax(const float *d_x, size_t n, uint32_t *d_scratch, float *h_out,
                       katoann_stream_t stream);

/* 16-bit codes of nrows x d floats: v = clamp(lround((x - lo) * inv_step)),
 * high/low byte planes nrows x dc (padding zero), and the squared norms of
 * the codes (norm), of the high bytes (hinorm) and of the high bytes of the
 * leading head_dims dimensions (headnorm, skipped when NULL). Follows
 * src/index.cpp:632-689 (lists), :717-750 (centroids), :917-943 (queries). */
int katoann_gpu_quantize_rows(const float *d_x, uint32_t nrows, uint32_t d, uint32_t dc, float lo,
                              double inv_step, uint32_t head_dims, uint8_t *d_hi, uint8_t *d_lo,
                              int64_t *d_norm, int64_t *d_hinorm, int64_t *d_headnorm,
                              katoann_stream_t stream);

/* The reference's sq16_l2 (include/katoann/kernels.h:187-193) on row-major
 * device planes: out[m][n] = float(double(qn + xn - 2 q.x) * step_sq), exact. */
int katoann_gpu_sq16_l2(const uint8_t *d_qhi, const uint8_t *d_qlo, const uint8_t *d_xhi,
                        const uint8_t *d_xlo, const int64_t *d_qnorm, const int64_t *d_xnorm,
                        double step_sq, uint32_t m, uint32_t n, uint32_t dims, float *d_out,
                        katoann_stream_t stream);

/* The reference's sq16_high_l2 (include/katoann/kernels.h:195-205): high bytes
 * only, over the leading `dims` of rows that are plane_dim bytes apart. */
int katoann_gpu_sq16_high_l2(const uint8_t *d_qhi, const uint8_t *d_xhi, const int64_t *d_qnorm,
                             const int64_t *d_xnorm, double step_sq, uint32_t m, uint32_t n,
                             uint32_t dims, uint32_t plane_dim, float *d_out,
                             katoann_stream_t stream);

/* Coarse step of the batched search (coarse_batched_sq16_,
 * src/index.cpp:846-877): exact SQ16 distances of nq quantized queries to the
 * centroid planes and the nprobe nearest lists per query, ascending by
 * (distance, list), into d_probed (nq x nprobe). d_dists (nq x nlist floats)
 * is caller scratch that receives the distances. When the view carries the
 * centred centroid planes (d_chi16, d_clo16, d_cterm) and dc <= 1024, the
 * product runs on the tensor cores with stream-ordered scratch for the
 * queries' planes, and the call synchronizes the stream to check that the
 * pipeline completed; otherwise it runs on the CUDA cores, asynchronously. */
int katoann_gpu_coarse(const katoann_gpu_index *index, const uint8_t *d_qhi, const uint8_t *d_qlo,
                       const int64_t *d_qnorm, uint32_t nq, uint32_t nprobe, float *d_dists,
                       uint32_t *d_probed, katoann_stream_t stream);

/* katoann_gpu_coarse for callers that cannot allocate device memory (a host
 * that owns every byte of device memory through its own allocator, or a
 * latency-bound loop that cannot afford cudaMalloc's device-wide
 * synchronisation). The nq x nlist distance scratch lives in a static device
 * array of 1,048,576 floats (4 MiB, held by every GPU that loads the library
 * until exit); nq * nlist above that is rejected with KATO_EINVAL. The first
 * call on a device resolves the array's address (make it before any stream
 * capture). Calls share the array: calls that overlap on the GPU race. This
 * entry point has no counterpart in the reference. */
int katoann_gpu_coarse_noalloc(const katoann_gpu_index *index, const uint8_t *d_qhi,
                               const uint8_t *d_qlo, const int64_t *d_qnorm, uint32_t nq,
                               uint32_t nprobe, uint32_t *d_probed, katoann_stream_t stream);

/* Bytes of device workspace that katoann_gpu_search needs for up to
 * max_batch queries per pass with these parameters. */
size_t katoann_gpu_search_workspace(const katoann_gpu_index *index, uint32_t max_batch,
                                    uint32_t k, uint32_t nprobe, int ranking, uint32_t survivors);

/* Index::search on the device (src/index.cpp:879-1219): rotation and
 * quantization of the queries, coarse product and top-nprobe, inversion of
 * the probe lists, ranking pass with per-query top-S (S = max(survivors, k)),
 * exact refinement and top-k (ranking PREFIX or HIGH), or the exact scan with
 * top-k (FULL). d_queries is nq x dim; d_ids / d_dists are nq x k, nearest
 * first, padded with UINT32_MAX / FLT_MAX. Queries are processed max_batch at
 * a time through the workspace (d_ws, ws_bytes from
 * katoann_gpu_search_workspace). Selection is by (distance, id), which is the
 * reference's Selection::kLocal result and its kThreshold result wherever the
 * latter has no tie on the survivor boundary. */
int katoann_gpu_search(const katoann_gpu_index *index, const float *d_queries, uint32_t nq,
                       uint32_t k, uint32_t nprobe, int ranking, uint32_t survivors,
                       uint32_t max_batch, void *d_ws, size_t ws_bytes, uint32_t *d_ids,
                       float *d_dists, katoann_stream_t stream);

/* Phase timer: CUDA events recorded on the search stream at the boundaries of
 * the pipeline's phases, so the duration of every phase of every pass in a
 * timed region is measured where it runs. Phases: 0 rotation+quantization of
 * the queries, 1 coarse product, 2 top-nprobe selection, 3 per-query probe
 * budget (empty without one), 4 inversion, 5 seed bounds of the tensor-core
 * ranking pass (empty on the CUDA-core pass), 6 ranking pass, 7 survivor
 * merge, 8 refinement. */
#define KATO_PHASES 9
void *katoann_gpu_timer_create(uint32_t max_passes);
void katoann_gpu_timer_destroy(void *timer);
/* Sums the phase durations (ms) of all passes recorded since the last read
 * into h_ms[0..KATO_PHASES) and their count into *passes; synchronous. */
int katoann_gpu_timer_read(void *timer, float *h_ms, uint32_t *passes);
/* The timer also brackets single kernels with events: 0 the query rotation
 * (its transposes and rotate_lanes_kernel), 1 coarse_tc_kernel, 2
 * rank_tc_kernel. Their summed ms and launch counts over the passes of the
 * last katoann_gpu_timer_read (a kernel a pass did not run is not counted). */
#define KATO_TIMED_KERNELS 3
void katoann_gpu_timer_kernels(void *timer, float *h_ms, uint32_t *h_launches);

/* Tensor-core form of a plane pair: d_hi16 / d_lo16 = (byte - 128) as fp16
 * bits, rows x dc each, and d_term[r] = norm[r] - 256 (65792 s_h + 257 s_l)
 * - 16384 dc 66049, s = the row's sum of (byte - 128) per plane. With these
 * for centroids and queries the coarse product is exact on fp16 tensor cores
 * for dc <= 1024. */
int katoann_gpu_centre_planes(const uint8_t *d_hi, const uint8_t *d_lo, const int64_t *d_norm,
                              uint32_t rows, uint32_t dc, uint16_t *d_hi16, uint16_t *d_lo16,
                              int64_t *d_term, katoann_stream_t stream);

/* Kernel launches of this thread's last katoann_gpu_search call (all passes). */
uint32_t katoann_gpu_last_launches(void);

/* Entries per query of the tensor-core ranking pass's candidate buffer
 * (default 32768, range [16, 2^20]; process-wide, read when a workspace is
 * sized and at each search). Queries with more candidates than this are
 * rescanned exactly; searches with survivors above it use the CUDA-core pass.
 * Results do not depend on it. */
int katoann_gpu_set_candidate_cap(uint32_t cap);

/* Rows of each query's nearest lists that give it a bound before the
 * tensor-core ranking pass (0 = the default, max(2048, 16 x survivors); at
 * most 4096; process-wide). Beyond 3 x survivors rows, a sketch over their
 * first 32 head bytes picks the 3 x survivors that are scored in full. More
 * rows mean a tighter bound (fewer candidates to merge) for more work up
 * front. Results do not depend on it. */
int katoann_gpu_set_seed_rows(uint32_t rows);

/* Knobs of the tensor-core ranking pass (process-wide; results never depend
 * on them): the largest work-item width (0 = by the prefix width, else 16,
 * 32 or 64 queries) and the cost weight of the split of tiles over the
 * persistent CTAs (0 = equal tile counts; 1 to 8 = a tile of an item of MMA
 * width w costs 64 + beta w, and the CTAs take equal cost). */
int katoann_gpu_set_rank_width(uint32_t width);
int katoann_gpu_set_rank_schedule(uint32_t beta);
/* The current knobs: h_out[3] = {seed rows (0 = default), split weight, item width}. */
void katoann_gpu_rank_knobs(uint32_t *h_out);
/* Every mbarrier wait of the tensor-core ranking pass gives up after this
 * many SM cycles (0 = the default, 4e9, about 2 s at 2 GHz); a CTA that gives
 * up sets its error flag, lets its copies and MMAs in flight finish, frees
 * its tensor memory and returns, and is counted in workspace statistic 3.
 * Process-wide. A limit far below a pipeline step makes searches fail with
 * KATO_ETIMEOUT (the host library checks the count after each pass); that is
 * its only use besides the default. */
int katoann_gpu_set_wait_limit(uint64_t cycles);

/* katoann_gpu_search that also records phase events into `timer` (may be
 * NULL, then identical to katoann_gpu_search). */
int katoann_gpu_search_timed(const katoann_gpu_index *index, const float *d_queries, uint32_t nq,
                             uint32_t k, uint32_t nprobe, int ranking, uint32_t survivors,
                             uint32_t max_batch, void *d_ws, size_t ws_bytes, uint32_t *d_ids,
                             float *d_dists, katoann_stream_t stream, void *timer);

/* Diagnostics that katoann_gpu_search left in its workspace, copied to the
 * host (synchronous on `stream`): [0] queries whose nprobe-th coarse distance
 * was tied with a list outside the probe set, [1] queries whose survivor
 * boundary (S-th ranking distance) was tied, [2] unused, [3] persistent
 * ranking CTAs whose bounded tensor-core wait ran out (their remaining work
 * is lost; never expected, reported so that it cannot pass silently), [4]
 * 128-row tiles the tensor-core ranking pass scored, [5] candidates it
 * appended (rows within their query's seed bound), [6] queries whose
 * candidate buffer overflowed and were rescanned exactly, [7] the largest
 * number of candidates one query had (last batch pass), [16..29] SM cycles
 * of the tensor-core ranking pass's warp roles, summed over CTAs (first
 * thread of each role): converters waiting for raw tiles, for free A stages,
 * total; MMA waiting for query tiles, free accumulators, converted tiles,
 * total; epilogue waiting for query tiles, accumulators, total; TMA waiting
 * for free stages, total; query staging waiting for free query tiles, total;
 * [30] cycles the ranking pass's MMA thread spent issuing MMAs and commits;
 * [31] cycles of the longest ranking CTA (the slowest SM's share);
 * [32..38] the same for the tensor-core coarse product: TMA waiting for free
 * stages, total; MMA waiting for accumulators, for stages, total; first
 * epilogue warp waiting for accumulators, total; [40..45] the ranking pass's
 * tiles by the number of queries of their work item: 1-2, 3-4, 5-8, 9-16,
 * 17-32, 33-64; [46] the distinct lists the batch probed (non-empty) and [47]
 * their rows (the rows the ranking pass reads once each). */
int katoann_gpu_workspace_stats(const void *d_ws, uint64_t *h_stats, uint32_t n,
                                katoann_stream_t stream);

/* Synchronous device-to-host copy of n bytes (exports the device index). */
int katoann_gpu_copy_to_host(void *h_dst, const void *d_src, size_t n);

/* float(double(l2) * step_sq) for n int64 values on the device (test hook of
 * the exact conversion every kernel uses). */
int katoann_gpu_dist_values(const int64_t *d_l2, uint32_t n, double step_sq, float *d_out,
                            katoann_stream_t stream);

/* ------------------------------------------------- learned probe budget
 * No counterpart in the reference, whose nprobe is one value for a whole
 * batch (SearchParams::nprobe, include/katoann/index.h:53). Here every query
 * may probe its own number of lists: the p_q nearest by (coarse distance,
 * list id), so a query's result is exactly the fixed-nprobe result at
 * nprobe = p_q. The budget comes either from the caller or from a small MLP
 * over the query's sorted coarse distances.
 *
 * Features: with d_r the r-th smallest coarse distance of the query (r from
 * 0), r_j the model's 64 ranks (r_0 = 0, ascending) and
 * e = 1e-4 d_{r_63} + 1e-30,
 *   z_0 = log(d_0 + e),   z_j = log(d_{r_j} + e) - log(d_0 + e)  (j >= 1),
 * standardized as x_j = (z_j - shift_j) * scale_j. The MLP is
 * 64 -> 256 (ReLU) -> 256 (ReLU) -> nclass: bf16 weights stored input-major
 * (w[i * outputs + o]), fp32 biases, fp32 accumulation. Its budget is
 * ladder[c] for the smallest class c whose cumulative softmax probability
 * reaches `threshold` (the last class if none does), capped at the search's
 * nprobe. */
#define KATO_PROBE_FEATURES 64
#define KATO_PROBE_HIDDEN 256
#define KATO_PROBE_MAX_CLASSES 32

typedef struct {
  uint32_t nclass;          /* 2 .. KATO_PROBE_MAX_CLASSES */
  uint32_t depth;           /* d_rank[63] + 1: how many coarse ranks the features read */
  float threshold;          /* cumulative probability the budget must reach */
  uint32_t reserved;
  const uint32_t *d_rank;   /* 64 */
  const float *d_shift;     /* 64 */
  const float *d_scale;     /* 64 */
  const uint16_t *d_w1;     /* 64 x 256 bf16, 16-byte aligned */
  const float *d_b1;        /* 256 */
  const uint16_t *d_w2;     /* 256 x 256 bf16 */
  const float *d_b2;        /* 256 */
  const uint16_t *d_w3;     /* 256 x nclass bf16 */
  const float *d_b3;        /* nclass */
  const uint32_t *d_ladder; /* nclass nprobe values, ascending */
} katoann_gpu_probe_model;

/* katoann_gpu_search_timed with a per-query nprobe. `nprobe` caps every
 * query's budget. The budget is d_nprobe_in[q] (device, nq values, each
 * clamped to [1, nprobe]) when given, else the model's choice when `model` is
 * given, else nprobe. The coarse selection takes P = max(nprobe,
 * model->depth) lists per query (P <= 4096 when a budget applies); size the
 * workspace with katoann_gpu_search_workspace(..., nprobe = P, ...).
 * d_nprobe_out (device, nq values, may be NULL) receives every query's
 * budget. */
int katoann_gpu_search_budget(const katoann_gpu_index *index, const float *d_queries,
                              uint32_t nq, uint32_t k, uint32_t nprobe, int ranking,
                              uint32_t survivors, uint32_t max_batch,
                              const uint32_t *d_nprobe_in, const katoann_gpu_probe_model *model,
                              void *d_ws, size_t ws_bytes, uint32_t *d_ids, float *d_dists,
                              uint32_t *d_nprobe_out, katoann_stream_t stream, void *timer);

/* A search captured as a CUDA graph (no counterpart in the reference): the
 * whole pipeline of one katoann_gpu_search_budget call - every kernel, memset
 * and copy of every batch pass - recorded on `stream` (a created stream, not
 * the legacy default one) and instantiated. Nothing runs at capture.
 * katoann_gpu_graph_launch replays it on any stream: the same pointers and
 * sizes, with whatever the buffers hold at replay, in one launch instead of
 * some thirty. The workspace, index, model and buffers must stay allocated
 * while the graph lives. */
int katoann_gpu_search_capture(const katoann_gpu_index *index, const float *d_queries,
                               uint32_t nq, uint32_t k, uint32_t nprobe, int ranking,
                               uint32_t survivors, uint32_t max_batch,
                               const uint32_t *d_nprobe_in, const katoann_gpu_probe_model *model,
                               void *d_ws, size_t ws_bytes, uint32_t *d_ids, float *d_dists,
                               uint32_t *d_nprobe_out, katoann_stream_t stream, void **graph);
int katoann_gpu_graph_launch(void *graph, katoann_stream_t stream);
/* Kernel launches one replay of the graph makes. */
uint32_t katoann_gpu_graph_launches(const void *graph);
void katoann_gpu_graph_destroy(void *graph);

/* The 64 raw features z (before standardization) of nq queries into d_z
 * (nq x 64, device): rotation, quantization, coarse product and selection of
 * the `depth` nearest lists, as in the search. The workspace is sized with
 * katoann_gpu_search_workspace(index, max_batch, 1, depth, KATO_RANK_FULL, 1). */
int katoann_gpu_probe_features(const katoann_gpu_index *index, const float *d_queries,
                               uint32_t nq, const uint32_t *d_rank, uint32_t depth,
                               uint32_t max_batch, void *d_ws, size_t ws_bytes, float *d_z,
                               katoann_stream_t stream);

/* The model on n raw feature rows d_z: class probabilities into d_probs
 * (n x nclass, may be NULL) and budgets, capped at `cap`, into d_nprobe (n,
 * may be NULL). */
int katoann_gpu_probe_predict(const katoann_gpu_probe_model *model, const float *d_z, uint32_t n,
                              uint32_t cap, float *d_probs, uint32_t *d_nprobe,
                              katoann_stream_t stream);

typedef struct {
  uint32_t epochs;     /* passes over the data */
  uint32_t batch;      /* rows per step */
  float lr;            /* Adam step size */
  float weight_decay;  /* decoupled, on the weights only */
  uint64_t seed;       /* initial weights and the order of the rows */
} katoann_gpu_probe_train_options;

/* Trains the MLP with softmax cross-entropy and Adam on n rows of raw
 * features d_z (n x 64) and classes d_label (n values < nclass), on the
 * device (synchronous; allocates its own device memory). The forward pass
 * uses bf16 copies of fp32 master weights. Outputs (host): the
 * standardization (h_shift, h_scale: the features' mean and 1 / standard
 * deviation), the trained weights in fp32 (h_w1 64 x 256, h_b1 256, h_w2
 * 256 x 256, h_b2 256, h_w3 256 x nclass, h_b3 nclass; round them to bf16 for
 * a model) and the mean loss of every epoch (h_loss, `epochs` values). */
int katoann_gpu_probe_train(const float *d_z, const uint8_t *d_label, uint32_t n,
                            uint32_t nclass, const katoann_gpu_probe_train_options *options,
                            float *h_shift, float *h_scale, float *h_w1, float *h_b1, float *h_w2,
                            float *h_b2, float *h_w3, float *h_b3, float *h_loss);

/* Mean cross-entropy loss of the model on n rows and its gradients with
 * respect to the weights (as fp32; test hook of the training kernels):
 * d_g = {w1, b1, w2, b2, w3, b3}, each sized like the parameter (device).
 * Synchronous. */
int katoann_gpu_probe_grads(const katoann_gpu_probe_model *model, const float *d_z,
                            const uint8_t *d_label, uint32_t n, float *h_loss, float *d_gw1,
                            float *d_gb1, float *d_gw2, float *d_gb2, float *d_gw3, float *d_gb3);

/* The autotuner: times one search of these queries (the workspace sized for
 * it) under every candidate setting - seed rows {1024, 2048, 4096}, split
 * weight {0, 1, 2, 4}, item width {default, 32} - and keeps the fastest
 * (settings that need a larger workspace are skipped). h_out[4] = {seed
 * rows, split weight, item width, microseconds per search}. Synchronous. */
int katoann_gpu_autotune(const katoann_gpu_index *index, const float *d_queries, uint32_t nq,
                         uint32_t k, uint32_t nprobe, int ranking, uint32_t survivors,
                         uint32_t max_batch, const uint32_t *d_nprobe_in,
                         const katoann_gpu_probe_model *model, void *d_ws, size_t ws_bytes,
                         katoann_stream_t stream, uint32_t *h_out);

/* ---- Index build on the device (replaces the host k-means of
 * src/kmeans.cpp and the covariance of pca_rotation, src/index.cpp:276-312).
 * Row arrays are fp32, row-major with a stride of ld floats: ld a multiple
 * of 32, at least the dimension, the padding zero; bases 16-byte aligned. */

/* The nearest centroid of each of n rows (replaces closest_centers,
 * src/kmeans.cpp:191-237): d_assign[i] = argmin_c |c|^2 - 2 x_i.c over the L
 * rows of d_cen (ties to the smaller c), on the tensor cores in TF32 with an
 * fp32 accumulator. d_cnorm[c] = |c|^2 (katoann_gpu_row_norms). d_best (may be
 * NULL) gets the minimum. d_timeouts (one zeroed word) counts CTAs whose
 * bounded pipeline wait ran out. */
int katoann_gpu_kmeans_assign(const float *d_x, uint32_t n, uint32_t ld, const float *d_cen,
                              const float *d_cnorm, uint32_t L, uint32_t *d_assign, float *d_best,
                              uint32_t *d_timeouts, katoann_stream_t stream);
/* d_out[i] = |x_i|^2 over ld floats. */
int katoann_gpu_row_norms(const float *d_x, uint32_t n, uint32_t ld, float *d_out,
                          katoann_stream_t stream);
/* One Lloyd update (the centre step of src/kmeans.cpp:73-187): each centroid
 * with members becomes their mean (summed in double); an empty one keeps its
 * value. Scratch: d_sums (L x ld doubles), d_counts (L). Also refreshes
 * d_cnorm. */
int katoann_gpu_kmeans_update(const float *d_x, uint32_t n, uint32_t ld, const uint32_t *d_assign,
                              uint32_t L, double *d_sums, uint32_t *d_counts, float *d_cen,
                              float *d_cnorm, katoann_stream_t stream);
/* k-means++ seeding (src/kmeans.cpp:280-321): centre 0 is row `first`; centre
 * m + 1 is drawn with probability proportional to the squared distance to
 * the nearest of centres 0..m, with d_u[m] (L - 1 uniforms in [0, 1), the
 * caller's seeded stream) as the draw. Writes L rows of d_cen and their row
 * indices to d_chosen. Scratch: d_dist (n floats) and
 * katoann_gpu_kmeanspp_scratch(n) bytes at d_part. */
size_t katoann_gpu_kmeanspp_scratch(uint32_t n);
int katoann_gpu_kmeanspp(const float *d_x, uint32_t n, uint32_t ld, uint32_t L, uint32_t first,
                         const double *d_u, float *d_cen, float *d_dist, void *d_part,
                         uint32_t *d_chosen, katoann_stream_t stream);
/* d_dst row i (stride ld, zero past d) = d_src row d_rows[i] (stride d). */
int katoann_gpu_gather_rows(const float *d_src, uint32_t d, const uint32_t *d_rows, uint32_t m,
                            uint32_t ld, float *d_dst, katoann_stream_t stream);
/* Mean-centred covariance of n rows over their first d columns, in double
 * (src/index.cpp:276-312): d_mean (d), d_cov (d x d, symmetric). */
int katoann_gpu_covariance(const float *d_x, uint32_t n, uint32_t ld, uint32_t d, double *d_mean,
                           double *d_cov, katoann_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* KATOANN_GPU_H_ */
