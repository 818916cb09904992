// extern "C" entry points of libkatoann_gpu.so (declared in
// include/katoann_gpu.h). Argument checks mirror the reference's exceptions
// (src/index.cpp:882-892) as status codes; nothing throws across the ABI.
#include <atomic>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <utility>

#include <cuda_fp16.h>

#include "kcommon.cuh"
#include "probe.cuh"
#include "rank_tc.cuh"

namespace kato {

namespace {
thread_local std::string g_error;
}

void set_error(const std::string &msg) { g_error = msg; }

int cuda_status(cudaError_t e, const char *what) {
  g_error = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? KATO_ENOMEM : KATO_ERUNTIME;
}

namespace {
std::mutex g_device_mu;
std::map<int, int> g_sms;                              // device -> SM count
std::map<std::pair<int, const void *>, int> g_smem;    // (device, kernel) -> bytes allowed
}  // namespace

int current_sms(int *sms) {
  int dev = 0;
  KATO_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_device_mu);
  auto it = g_sms.find(dev);
  if (it == g_sms.end()) {
    int n = 0;
    KATO_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    it = g_sms.emplace(dev, n).first;
  }
  *sms = it->second;
  return KATO_OK;
}

int smem_limit(const void *kernel, int bytes, const char *what) {
  int dev = 0;
  KATO_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_device_mu);
  int &have = g_smem[{dev, kernel}];
  if (have < bytes) {
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return cuda_status(e, what);
    have = bytes;
  }
  return KATO_OK;
}

int rotate_rows(const float *in, uint32_t nrows, uint32_t d, const float *rot, float *out,
                cudaStream_t st);
size_t rotation_kmajor_bytes(uint32_t d);
int rotation_kmajor(const float *rot, uint32_t d, float *out, cudaStream_t st);
int minmax(const float *x, size_t n, uint32_t *d_keys, float *h_out, cudaStream_t st);
int quantize_rows(const float *x, uint32_t nrows, uint32_t d, uint32_t dc, float lo,
                  double inv_step, uint32_t head, uint8_t *hi, uint8_t *lop, int64_t *norm,
                  int64_t *hinorm, int64_t *headnorm, cudaStream_t st);
int sq16_tiles(const uint8_t *qhi, const uint8_t *qlo, const uint8_t *xhi, const uint8_t *xlo,
               const int64_t *qn, const int64_t *xn, double step_sq, uint32_t m, uint32_t n,
               uint32_t dims, uint32_t qstride, uint32_t xstride, float *out, bool full,
               cudaStream_t st);
int select_topp(const float *dists, uint32_t nq, uint32_t n, uint32_t p, uint32_t *probed,
                unsigned long long *tie_count, cudaStream_t st);
int dist_values(const int64_t *l2, uint32_t n, double step_sq, float *out, cudaStream_t st);
int search(const katoann_gpu_index *ix, const float *queries, uint32_t nq, uint32_t k, uint32_t p,
           int ranking, uint32_t survivors, uint32_t max_batch, void *ws, size_t ws_bytes,
           uint32_t *out_ids, float *out_dists, const Budget &budget, cudaStream_t st,
           void *timer);
int probe_features_search(const katoann_gpu_index *ix, const float *queries, uint32_t nq,
                          const uint32_t *rank, uint32_t depth, uint32_t max_batch, void *ws,
                          size_t ws_bytes, float *z, cudaStream_t st);
int autotune(const katoann_gpu_index *ix, const float *queries, uint32_t nq, uint32_t k, uint32_t p,
             int ranking, uint32_t survivors, uint32_t max_batch, const Budget &budget, void *ws,
             size_t ws_bytes, cudaStream_t st, uint32_t *out);
int search_capture(const katoann_gpu_index *ix, const float *queries, uint32_t nq, uint32_t k,
                   uint32_t p, int ranking, uint32_t survivors, uint32_t max_batch, void *ws,
                   size_t ws_bytes, uint32_t *out_ids, float *out_dists, const Budget &budget,
                   cudaStream_t st, void **out);
int graph_launch(void *h, cudaStream_t st);
uint32_t graph_launches(const void *h);
void graph_destroy(void *h);
void *timer_create(uint32_t max_passes);
uint32_t last_launches();
int centre_planes(const uint8_t *hi, const uint8_t *lo, const int64_t *norm, uint32_t rows,
                  uint32_t dc, __half *hi16, __half *lo16, int64_t *term, cudaStream_t st);
bool coarse_tc_ok(uint32_t dc);
int kmeans_assign(const float *x, uint32_t n, uint32_t ld, const float *cen, const float *cnorm,
                  uint32_t L, uint32_t *assign, float *best, uint32_t *timeouts, cudaStream_t st);
int row_norms(const float *x, uint32_t n, uint32_t ld, float *out, cudaStream_t st);
int kmeans_update(const float *x, uint32_t n, uint32_t ld, const uint32_t *assign, uint32_t L,
                  double *sums, uint32_t *counts, float *cen, float *cnorm, cudaStream_t st);
size_t kmeanspp_scratch(uint32_t n);
int gather_rows(const float *src, uint32_t d, const uint32_t *rows, uint32_t m, uint32_t ld,
                float *dst, cudaStream_t st);
int kmeanspp(const float *x, uint32_t n, uint32_t ld, uint32_t L, uint32_t first, const double *u,
             float *cen, float *dist, double *part, uint32_t *chosen, cudaStream_t st);
int covariance(const float *x, uint32_t n, uint32_t ld, uint32_t d, double *mean, double *cov,
               cudaStream_t st);
int coarse_tc(const __half *ch, const __half *cl, const int64_t *cterm, uint32_t n, const __half *qh,
              const __half *ql, const int64_t *qterm, uint32_t m, uint32_t dc, double step_sq,
              float *out, uint32_t *timeouts, unsigned long long *prof, cudaStream_t st);
extern std::atomic<uint32_t> g_candidate_cap;
extern std::atomic<uint32_t> g_seed_rows;
void timer_destroy(void *t);
int timer_read(void *t, float *ms, uint32_t *passes);
void timer_kernels(void *t, float *ms, uint32_t *launches);
size_t search_workspace(const katoann_gpu_index *ix, uint32_t max_batch, uint32_t k, uint32_t p,
                        int ranking, uint32_t survivors);

}  // namespace kato

using kato::as_stream;

extern "C" {

const char *katoann_gpu_last_error(void) { return kato::g_error.c_str(); }

int katoann_gpu_version(void) { return 1; }

int katoann_gpu_rotate_rows(const float *d_in, uint32_t nrows, uint32_t d, const float *d_rot,
                            float *d_out, katoann_stream_t stream) {
  if (d == 0 || d > 4096) return kato::invalid("dimension must be 1 to 4096");
  return kato::rotate_rows(d_in, nrows, d, d_rot, d_out, as_stream(stream));
}

size_t katoann_gpu_rotation_kmajor_bytes(uint32_t d) { return kato::rotation_kmajor_bytes(d); }

int katoann_gpu_rotation_kmajor(const float *d_rot, uint32_t d, float *d_out,
                                katoann_stream_t stream) {
  if (d == 0 || d > 4096) return kato::invalid("dimension must be 1 to 4096");
  return kato::rotation_kmajor(d_rot, d, d_out, as_stream(stream));
}

int katoann_gpu_minmax(const float *d_x, size_t n, uint32_t *d_scratch, float *h_out,
                       katoann_stream_t stream) {
  return kato::minmax(d_x, n, d_scratch, h_out, as_stream(stream));
}

int katoann_gpu_quantize_rows(const float *d_x, uint32_t nrows, uint32_t d, uint32_t dc, float lo,
                              double inv_step, uint32_t head_dims, uint8_t *d_hi, uint8_t *d_lo,
                              int64_t *d_norm, int64_t *d_hinorm, int64_t *d_headnorm,
                              katoann_stream_t stream) {
  if (dc < d || dc % 64) return kato::invalid("padded dimension must be a multiple of 64 >= dim");
  if (head_dims > dc) return kato::invalid("prefix_dims must be a multiple of 64 within the dimension");
  return kato::quantize_rows(d_x, nrows, d, dc, lo, inv_step, d_headnorm ? head_dims : 0, d_hi,
                             d_lo, d_norm, d_hinorm, d_headnorm, as_stream(stream));
}

int katoann_gpu_sq16_l2(const uint8_t *d_qhi, const uint8_t *d_qlo, const uint8_t *d_xhi,
                        const uint8_t *d_xlo, const int64_t *d_qnorm, const int64_t *d_xnorm,
                        double step_sq, uint32_t m, uint32_t n, uint32_t dims, float *d_out,
                        katoann_stream_t stream) {
  return kato::sq16_tiles(d_qhi, d_qlo, d_xhi, d_xlo, d_qnorm, d_xnorm, step_sq, m, n, dims, dims,
                          dims, d_out, true, as_stream(stream));
}

int katoann_gpu_sq16_high_l2(const uint8_t *d_qhi, const uint8_t *d_xhi, const int64_t *d_qnorm,
                             const int64_t *d_xnorm, double step_sq, uint32_t m, uint32_t n,
                             uint32_t dims, uint32_t plane_dim, float *d_out,
                             katoann_stream_t stream) {
  if (plane_dim == 0) plane_dim = dims;
  if (plane_dim < dims || plane_dim % 64)  // src/kernels.cpp:301-303
    return kato::invalid("plane_dim must be a multiple of 64 and at least padded_dim");
  return kato::sq16_tiles(d_qhi, nullptr, d_xhi, nullptr, d_qnorm, d_xnorm, step_sq, m, n, dims,
                          dims, plane_dim, d_out, false, as_stream(stream));
}

int katoann_gpu_coarse(const katoann_gpu_index *ix, const uint8_t *d_qhi, const uint8_t *d_qlo,
                       const int64_t *d_qnorm, uint32_t nq, uint32_t nprobe, float *d_dists,
                       uint32_t *d_probed, katoann_stream_t stream) {
  if (!ix) return kato::invalid("null index");
  if (nprobe == 0 || nprobe > ix->nlist) return kato::invalid("need k >= 1 and 1 <= nprobe <= nlist");
  const cudaStream_t st = as_stream(stream);
  int rc;
  if (ix->d_chi16 && ix->d_clo16 && ix->d_cterm && kato::coarse_tc_ok(ix->dc) && nq) {
    // tensor cores: the queries' centred planes in stream-ordered scratch
    const size_t plane = static_cast<size_t>(nq) * ix->dc * 2;
    void *scratch = nullptr;
    KATO_CUDA(cudaMallocAsync(&scratch, 2 * plane + static_cast<size_t>(nq) * 8 + 256, st));
    auto *qh16 = static_cast<__half *>(scratch);
    auto *ql16 = reinterpret_cast<__half *>(static_cast<unsigned char *>(scratch) + plane);
    auto *qterm = reinterpret_cast<int64_t *>(static_cast<unsigned char *>(scratch) + 2 * plane);
    auto *flag = reinterpret_cast<uint32_t *>(qterm + nq);
    rc = cudaMemsetAsync(flag, 0, 4, st) != cudaSuccess ? KATO_ERUNTIME : KATO_OK;
    if (!rc) rc = kato::centre_planes(d_qhi, d_qlo, d_qnorm, nq, ix->dc, qh16, ql16, qterm, st);
    if (!rc)
      rc = kato::coarse_tc(reinterpret_cast<const __half *>(ix->d_chi16),
                           reinterpret_cast<const __half *>(ix->d_clo16), ix->d_cterm, ix->nlist,
                           qh16, ql16, qterm, nq, ix->dc, ix->step_sq, d_dists, flag, nullptr, st);
    uint32_t timeouts = 0;
    if (!rc && cudaMemcpyAsync(&timeouts, flag, 4, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
        cudaStreamSynchronize(st) == cudaSuccess && timeouts)
      rc = kato::invalid("tensor-core coarse product: a bounded pipeline wait ran out");
    cudaFreeAsync(scratch, st);
  } else {
    rc = kato::sq16_tiles(d_qhi, d_qlo, ix->d_chi, ix->d_clo, d_qnorm, ix->d_cnorm, ix->step_sq, nq,
                          ix->nlist, ix->dc, ix->dc, ix->dc, d_dists, true, st);
  }
  if (rc) return rc;
  return kato::select_topp(d_dists, nq, ix->nlist, nprobe, d_probed, nullptr, st);
}

size_t katoann_gpu_search_workspace(const katoann_gpu_index *ix, uint32_t max_batch, uint32_t k,
                                    uint32_t nprobe, int ranking, uint32_t survivors) {
  if (!ix) return 0;
  return kato::search_workspace(ix, max_batch, k, nprobe, ranking, survivors);
}

int katoann_gpu_search(const katoann_gpu_index *ix, const float *d_queries, uint32_t nq,
                       uint32_t k, uint32_t nprobe, int ranking, uint32_t survivors,
                       uint32_t max_batch, void *d_ws, size_t ws_bytes, uint32_t *d_ids,
                       float *d_dists, katoann_stream_t stream) {
  if (!ix) return kato::invalid("null index");
  if (ix->nlist == 0) {
    kato::set_error("search before load");
    return KATO_ELOGIC;
  }
  return kato::search(ix, d_queries, nq, k, nprobe, ranking, survivors, max_batch, d_ws, ws_bytes,
                      d_ids, d_dists, kato::Budget{}, as_stream(stream), nullptr);
}

int katoann_gpu_search_timed(const katoann_gpu_index *ix, const float *d_queries, uint32_t nq,
                             uint32_t k, uint32_t nprobe, int ranking, uint32_t survivors,
                             uint32_t max_batch, void *d_ws, size_t ws_bytes, uint32_t *d_ids,
                             float *d_dists, katoann_stream_t stream, void *timer) {
  if (!ix) return kato::invalid("null index");
  if (ix->nlist == 0) {
    kato::set_error("search before load");
    return KATO_ELOGIC;
  }
  return kato::search(ix, d_queries, nq, k, nprobe, ranking, survivors, max_batch, d_ws, ws_bytes,
                      d_ids, d_dists, kato::Budget{}, as_stream(stream), timer);
}

int katoann_gpu_search_budget(const katoann_gpu_index *ix, const float *d_queries, uint32_t nq,
                              uint32_t k, uint32_t nprobe, int ranking, uint32_t survivors,
                              uint32_t max_batch, const uint32_t *d_nprobe_in,
                              const katoann_gpu_probe_model *model, void *d_ws, size_t ws_bytes,
                              uint32_t *d_ids, float *d_dists, uint32_t *d_nprobe_out,
                              katoann_stream_t stream, void *timer) {
  if (!ix) return kato::invalid("null index");
  if (ix->nlist == 0) {
    kato::set_error("search before load");
    return KATO_ELOGIC;
  }
  kato::Budget b;
  b.nprobe_in = d_nprobe_in;
  b.model = d_nprobe_in ? nullptr : model;
  b.nprobe_out = d_nprobe_out;
  return kato::search(ix, d_queries, nq, k, nprobe, ranking, survivors, max_batch, d_ws, ws_bytes,
                      d_ids, d_dists, b, as_stream(stream), timer);
}

int katoann_gpu_set_rank_width(uint32_t width) {
  if (width != 0 && width != 16 && width != 32 && width != 64)
    return kato::invalid("rank width must be 0, 16, 32 or 64");
  kato::g_tc_width = width;
  return KATO_OK;
}

void katoann_gpu_rank_knobs(uint32_t *h_out) {
  h_out[0] = kato::g_seed_rows.load();
  h_out[1] = kato::g_tc_beta.load();
  h_out[2] = kato::g_tc_width.load();
}

int katoann_gpu_set_wait_limit(uint64_t cycles) {
  if (cycles > (1ull << 40)) return kato::invalid("wait limit must be at most 2^40 cycles");
  kato::g_tc_wait = cycles;
  return KATO_OK;
}

int katoann_gpu_set_rank_schedule(uint32_t beta) {
  if (beta > 8) return kato::invalid("rank schedule weight must be at most 8");
  kato::g_tc_beta = beta;
  return KATO_OK;
}

int katoann_gpu_autotune(const katoann_gpu_index *ix, const float *d_queries, uint32_t nq,
                         uint32_t k, uint32_t nprobe, int ranking, uint32_t survivors,
                         uint32_t max_batch, const uint32_t *d_nprobe_in,
                         const katoann_gpu_probe_model *model, void *d_ws, size_t ws_bytes,
                         katoann_stream_t stream, uint32_t *h_out) {
  if (!ix || !h_out) return kato::invalid("null index or output");
  if (ix->nlist == 0) {
    kato::set_error("autotune before load");
    return KATO_ELOGIC;
  }
  kato::Budget b;
  b.nprobe_in = d_nprobe_in;
  b.model = d_nprobe_in ? nullptr : model;
  return kato::autotune(ix, d_queries, nq, k, nprobe, ranking, survivors, max_batch, b, d_ws,
                        ws_bytes, as_stream(stream), h_out);
}

int katoann_gpu_search_capture(const katoann_gpu_index *ix, const float *d_queries, uint32_t nq,
                               uint32_t k, uint32_t nprobe, int ranking, uint32_t survivors,
                               uint32_t max_batch, const uint32_t *d_nprobe_in,
                               const katoann_gpu_probe_model *model, void *d_ws, size_t ws_bytes,
                               uint32_t *d_ids, float *d_dists, uint32_t *d_nprobe_out,
                               katoann_stream_t stream, void **graph) {
  if (!graph) return kato::invalid("null graph handle");
  *graph = nullptr;
  if (!ix) return kato::invalid("null index");
  if (ix->nlist == 0) {
    kato::set_error("search before load");
    return KATO_ELOGIC;
  }
  kato::Budget b;
  b.nprobe_in = d_nprobe_in;
  b.model = d_nprobe_in ? nullptr : model;
  b.nprobe_out = d_nprobe_out;
  return kato::search_capture(ix, d_queries, nq, k, nprobe, ranking, survivors, max_batch, d_ws,
                              ws_bytes, d_ids, d_dists, b, as_stream(stream), graph);
}

int katoann_gpu_graph_launch(void *graph, katoann_stream_t stream) {
  return kato::graph_launch(graph, as_stream(stream));
}

uint32_t katoann_gpu_graph_launches(const void *graph) { return kato::graph_launches(graph); }

void katoann_gpu_graph_destroy(void *graph) { kato::graph_destroy(graph); }

int katoann_gpu_probe_features(const katoann_gpu_index *ix, const float *d_queries, uint32_t nq,
                               const uint32_t *d_rank, uint32_t depth, uint32_t max_batch,
                               void *d_ws, size_t ws_bytes, float *d_z, katoann_stream_t stream) {
  if (!ix) return kato::invalid("null index");
  if (ix->nlist == 0) {
    kato::set_error("features before load");
    return KATO_ELOGIC;
  }
  return kato::probe_features_search(ix, d_queries, nq, d_rank, depth, max_batch, d_ws, ws_bytes,
                                     d_z, as_stream(stream));
}

void *katoann_gpu_timer_create(uint32_t max_passes) { return kato::timer_create(max_passes); }

uint32_t katoann_gpu_last_launches(void) { return kato::last_launches(); }

int katoann_gpu_centre_planes(const uint8_t *d_hi, const uint8_t *d_lo, const int64_t *d_norm,
                              uint32_t rows, uint32_t dc, uint16_t *d_hi16, uint16_t *d_lo16,
                              int64_t *d_term, katoann_stream_t stream) {
  return kato::centre_planes(d_hi, d_lo, d_norm, rows, dc, reinterpret_cast<__half *>(d_hi16),
                             reinterpret_cast<__half *>(d_lo16), d_term, as_stream(stream));
}

int katoann_gpu_set_seed_rows(uint32_t rows) {
  if (rows > 4096) return kato::invalid("seed rows must be at most 4096");
  kato::g_seed_rows.store(rows);
  return KATO_OK;
}

int katoann_gpu_set_candidate_cap(uint32_t cap) {
  if (cap < 16 || cap > (1u << 20)) return kato::invalid("candidate buffer size must be in [16, 2^20]");
  kato::g_candidate_cap.store(cap);
  return KATO_OK;
}

void katoann_gpu_timer_destroy(void *timer) { kato::timer_destroy(timer); }

void katoann_gpu_timer_kernels(void *timer, float *h_ms, uint32_t *h_launches) {
  kato::timer_kernels(timer, h_ms, h_launches);
}

int katoann_gpu_timer_read(void *timer, float *h_ms, uint32_t *passes) {
  if (!timer) return kato::invalid("null timer");
  return kato::timer_read(timer, h_ms, passes);
}

int katoann_gpu_workspace_stats(const void *d_ws, uint64_t *h_stats, uint32_t n,
                                katoann_stream_t stream) {
  if (n > 48) return kato::invalid("at most 48 statistics");
  KATO_CUDA(cudaMemcpyAsync(h_stats, d_ws, n * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                            as_stream(stream)));
  KATO_CUDA(cudaStreamSynchronize(as_stream(stream)));
  return KATO_OK;
}

int katoann_gpu_copy_to_host(void *h_dst, const void *d_src, size_t n) {
  KATO_CUDA(cudaMemcpy(h_dst, d_src, n, cudaMemcpyDeviceToHost));
  return KATO_OK;
}

int katoann_gpu_dist_values(const int64_t *d_l2, uint32_t n, double step_sq, float *d_out,
                            katoann_stream_t stream) {
  return kato::dist_values(d_l2, n, step_sq, d_out, as_stream(stream));
}


// ---- index build on the device
int katoann_gpu_kmeans_assign(const float *d_x, uint32_t n, uint32_t ld, const float *d_cen,
                              const float *d_cnorm, uint32_t L, uint32_t *d_assign, float *d_best,
                              uint32_t *d_timeouts, katoann_stream_t stream) {
  return kato::kmeans_assign(d_x, n, ld, d_cen, d_cnorm, L, d_assign, d_best, d_timeouts,
                             as_stream(stream));
}

int katoann_gpu_row_norms(const float *d_x, uint32_t n, uint32_t ld, float *d_out,
                          katoann_stream_t stream) {
  if (n && (!d_x || !d_out || ld == 0)) return kato::invalid("row norms: bad arguments");
  return kato::row_norms(d_x, n, ld, d_out, as_stream(stream));
}

int katoann_gpu_kmeans_update(const float *d_x, uint32_t n, uint32_t ld, const uint32_t *d_assign,
                              uint32_t L, double *d_sums, uint32_t *d_counts, float *d_cen,
                              float *d_cnorm, katoann_stream_t stream) {
  if (L == 0 || ld == 0 || !d_sums || !d_counts || !d_cen || !d_cnorm || (n && (!d_x || !d_assign)))
    return kato::invalid("k-means update: bad arguments");
  return kato::kmeans_update(d_x, n, ld, d_assign, L, d_sums, d_counts, d_cen, d_cnorm,
                             as_stream(stream));
}

size_t katoann_gpu_kmeanspp_scratch(uint32_t n) { return kato::kmeanspp_scratch(n); }

int katoann_gpu_kmeanspp(const float *d_x, uint32_t n, uint32_t ld, uint32_t L, uint32_t first,
                         const double *d_u, float *d_cen, float *d_dist, void *d_part,
                         uint32_t *d_chosen, katoann_stream_t stream) {
  if (!d_x || !d_u || !d_cen || !d_dist || !d_part || !d_chosen || ld == 0)
    return kato::invalid("k-means++: bad arguments");
  return kato::kmeanspp(d_x, n, ld, L, first, d_u, d_cen, d_dist, static_cast<double *>(d_part),
                        d_chosen, as_stream(stream));
}

int katoann_gpu_gather_rows(const float *d_src, uint32_t d, const uint32_t *d_rows, uint32_t m,
                            uint32_t ld, float *d_dst, katoann_stream_t stream) {
  if (m && (!d_src || !d_rows || !d_dst || ld < d)) return kato::invalid("gather rows: bad arguments");
  return kato::gather_rows(d_src, d, d_rows, m, ld, d_dst, as_stream(stream));
}

int katoann_gpu_covariance(const float *d_x, uint32_t n, uint32_t ld, uint32_t d, double *d_mean,
                           double *d_cov, katoann_stream_t stream) {
  if (!d_x || !d_mean || !d_cov || ld < d) return kato::invalid("covariance: bad arguments");
  return kato::covariance(d_x, n, ld, d, d_mean, d_cov, as_stream(stream));
}

}  // extern "C"
