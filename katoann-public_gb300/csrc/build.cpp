// Index::build on the GPU: the k-means partition, the assignment of every
// vector, and the PCA rotation, written in the reference's file format.
//
// Follows Index::build (src/index.cpp:419-514): a strided training sample
// (:430-443), k-means++ seeding (src/kmeans.cpp:280-321), Lloyd iterations
// (the reference's Elkan iteration, :73-187, reaches the same fixed point
// with fewer distance evaluations), the nearest centroid of every vector
// (closest_centers, :191-237), lists in ascending id order (:464-480), the
// files (:482-505), and the rotation of a list-order sample (:516-533) by
// cyclic Jacobi on its covariance (pca_rotation, :276-380) with the default
// head dims (:512) in .dimc (:535-545). The distance work runs on the device
// (libkatoann_gpu.so: katoann_gpu_kmeans*, katoann_gpu_covariance); the
// Jacobi sweeps run on the host cores, their pairs ordered as rounds of
// disjoint rotations so that a round runs in parallel.
//
// The partition need not match the reference's bit for bit: search parity is
// defined over the index files, whoever wrote them.
#include <cuda_runtime.h>
#include <omp.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <random>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "katoann/index.h"
#include "katoann_gpu.h"

namespace katoann {

namespace {

constexpr uint32_t kDimcMagic = 0x434D4944u;

void cuda_ok(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

void gpu_ok(int rc) {
  if (rc == KATO_EINVAL) throw std::invalid_argument(katoann_gpu_last_error());
  if (rc != KATO_OK) throw std::runtime_error(katoann_gpu_last_error());
}

// Device memory owned for the length of one build.
struct Dev {
  void *p = nullptr;
  Dev() = default;
  explicit Dev(size_t bytes) { cuda_ok(cudaMalloc(&p, std::max<size_t>(bytes, 16)), "cudaMalloc"); }
  ~Dev() {
    if (p) cudaFree(p);
  }
  Dev(const Dev &) = delete;
  Dev &operator=(const Dev &) = delete;
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
  }
  template <typename T>
  T *as() const {
    return static_cast<T *>(p);
  }
};

// Rows `rows` of data (host or device, n x dim) into a device buffer of
// stride ld (zero-padded), in order.
void stage_rows(const float *data, bool on_device, uint32_t dim, const std::vector<uint32_t> &rows,
                uint32_t ld, float *d_out, cudaStream_t st) {
  const uint32_t m = static_cast<uint32_t>(rows.size());
  if (m == 0) return;
  if (on_device) {
    Dev idx(rows.size() * sizeof(uint32_t));
    cuda_ok(cudaMemcpyAsync(idx.p, rows.data(), rows.size() * 4, cudaMemcpyHostToDevice, st), "upload");
    gpu_ok(katoann_gpu_gather_rows(data, dim, idx.as<uint32_t>(), m, ld, d_out,
                                   reinterpret_cast<katoann_stream_t>(st)));
    cuda_ok(cudaStreamSynchronize(st), "gather");
    return;
  }
  std::vector<float> host(static_cast<size_t>(m) * ld, 0.0f);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < static_cast<int64_t>(m); ++i)
    std::memcpy(host.data() + static_cast<size_t>(i) * ld, data + static_cast<size_t>(rows[i]) * dim,
                dim * sizeof(float));
  cuda_ok(cudaMemcpyAsync(d_out, host.data(), host.size() * 4, cudaMemcpyHostToDevice, st), "upload");
  cuda_ok(cudaStreamSynchronize(st), "upload");
}

// Contiguous rows [r0, r0 + m) of data into a device buffer of stride ld.
void stage_range(const float *data, bool on_device, uint32_t dim, uint32_t r0, uint32_t m,
                 uint32_t ld, float *d_out, cudaStream_t st) {
  if (ld != dim) cuda_ok(cudaMemsetAsync(d_out, 0, static_cast<size_t>(m) * ld * 4, st), "memset");
  cuda_ok(cudaMemcpy2DAsync(d_out, ld * sizeof(float), data + static_cast<size_t>(r0) * dim,
                            dim * sizeof(float), dim * sizeof(float), m,
                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st),
          "upload rows");
}

// Cyclic Jacobi on the symmetric d x d matrix A (destroyed); rot row j = the
// eigenvector of the j-th largest eigenvalue. Each sweep visits every pair
// once, in d - 1 rounds of d / 2 disjoint pairs (round-robin order); the
// angles of a round come from the matrix as the round begins, so its
// rotations commute and are applied together: rows, then columns, then V.
void jacobi_rotation(std::vector<double> &A, uint32_t d, uint32_t sweeps, std::vector<float> &rot) {
  const uint32_t m = d + (d & 1);  // even number of players (the last one idle when d is odd)
  std::vector<double> V(static_cast<size_t>(d) * d, 0.0);
  for (uint32_t i = 0; i < d; ++i) V[static_cast<size_t>(i) * d + i] = 1.0;
  double diag = 0;
  for (uint32_t i = 0; i < d; ++i) diag += A[static_cast<size_t>(i) * d + i] * A[static_cast<size_t>(i) * d + i];
  std::vector<uint32_t> ring(m);
  for (uint32_t i = 0; i < m; ++i) ring[i] = i;
  std::vector<std::pair<uint32_t, uint32_t>> pairs(m / 2);
  std::vector<double> cs(m / 2), sn(m / 2);
  sweeps = std::clamp<uint32_t>(sweeps, 1u, 64u);
  for (uint32_t sw = 0; sw < sweeps; ++sw) {
    double offd = 0;
#pragma omp parallel for reduction(+ : offd) schedule(static)
    for (int64_t i = 0; i < static_cast<int64_t>(d); ++i)
      for (uint32_t j = static_cast<uint32_t>(i) + 1; j < d; ++j)
        offd += 2.0 * A[static_cast<size_t>(i) * d + j] * A[static_cast<size_t>(i) * d + j];
    std::fprintf(stderr, "rotation: Jacobi sweep %u/%u, off-diagonal %.3e\n", sw + 1, sweeps, offd);
    if (offd <= 1e-18 * std::max(diag, 1e-300)) break;
    for (uint32_t round = 0; round + 1 < m; ++round) {
      // the circle method: player 0 stays, the others rotate
      for (uint32_t k = 0; k < m / 2; ++k) {
        uint32_t p = ring[k], q = ring[m - 1 - k];
        if (p > q) std::swap(p, q);
        pairs[k] = {p, q};
      }
      std::rotate(ring.begin() + 1, ring.end() - 1, ring.end());
      for (uint32_t k = 0; k < m / 2; ++k) {
        const auto [p, q] = pairs[k];
        cs[k] = 1.0, sn[k] = 0.0;
        if (q >= d) continue;  // the idle player
        const double apq = A[static_cast<size_t>(p) * d + q];
        const double app = A[static_cast<size_t>(p) * d + p], aqq = A[static_cast<size_t>(q) * d + q];
        if (std::fabs(apq) <= 1e-14 * std::sqrt(std::fabs(app * aqq)) + 1e-300) continue;
        const double theta = 0.5 * (aqq - app) / apq;
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(1.0 + theta * theta));
        cs[k] = 1.0 / std::sqrt(1.0 + t * t);
        sn[k] = t * cs[k];
      }
      // rows p and q of every rotated pair
#pragma omp parallel for schedule(static)
      for (int64_t k = 0; k < static_cast<int64_t>(m / 2); ++k) {
        const auto [p, q] = pairs[k];
        if (q >= d || sn[k] == 0.0) continue;
        double *rp = A.data() + static_cast<size_t>(p) * d, *rq = A.data() + static_cast<size_t>(q) * d;
        for (uint32_t c = 0; c < d; ++c) {
          const double xp = rp[c], xq = rq[c];
          rp[c] = cs[k] * xp - sn[k] * xq;
          rq[c] = sn[k] * xp + cs[k] * xq;
        }
      }
      // columns p and q of every row of A and V
#pragma omp parallel for schedule(static)
      for (int64_t r = 0; r < static_cast<int64_t>(d); ++r) {
        double *ra = A.data() + static_cast<size_t>(r) * d, *rv = V.data() + static_cast<size_t>(r) * d;
        for (uint32_t k = 0; k < m / 2; ++k) {
          const auto [p, q] = pairs[k];
          if (q >= d || sn[k] == 0.0) continue;
          const double ap = ra[p], aq = ra[q], vp = rv[p], vq = rv[q];
          ra[p] = cs[k] * ap - sn[k] * aq;
          ra[q] = sn[k] * ap + cs[k] * aq;
          rv[p] = cs[k] * vp - sn[k] * vq;
          rv[q] = sn[k] * vp + cs[k] * vq;
        }
      }
    }
  }
  std::vector<std::pair<double, uint32_t>> ev(d);
  for (uint32_t i = 0; i < d; ++i) ev[i] = {A[static_cast<size_t>(i) * d + i], i};
  std::stable_sort(ev.begin(), ev.end(), [](const auto &a, const auto &b) { return a.first > b.first; });
  rot.resize(static_cast<size_t>(d) * d);
  for (uint32_t j = 0; j < d; ++j)
    for (uint32_t k = 0; k < d; ++k)
      rot[static_cast<size_t>(j) * d + k] = static_cast<float>(V[static_cast<size_t>(k) * d + ev[j].second]);
}

}  // namespace

uint32_t default_head_dims(uint32_t dim) {
  const uint32_t dc = (dim + 63) / 64 * 64;
  return std::min(std::max(64u, (dim / 4 + 63) / 64 * 64), dc);  // src/index.cpp:512
}

BuildResult Index::partition(const float *data, uint32_t n, uint32_t dim, const BuildOptions &opt,
                             bool on_device) {
  if (dim == 0 || dim > kMaxDim) throw std::invalid_argument("dimension must be 1 to 4096");
  if (n == 0 || opt.nlist == 0 || opt.nlist > n) throw std::invalid_argument("need at least nlist vectors");
  const uint32_t L = opt.nlist, ld = (dim + 31) / 32 * 32;
  const uint32_t ts = std::min(opt.train_size, n);
  if (ts < L) throw std::invalid_argument("train_size must be at least nlist");
  cudaStream_t st = nullptr;
  cuda_ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } guard{st};
  const katoann_stream_t ks = reinterpret_cast<katoann_stream_t>(st);
  BuildResult out;

  // 1. the strided training sample (src/index.cpp:430-443), on the device
  std::vector<uint32_t> rows(ts);
  const uint64_t stride = static_cast<uint64_t>(n) * (1ull << 32) / ts;
  for (uint32_t i = 0; i < ts; ++i)
    rows[i] = ts == n ? i : std::min<uint32_t>(n - 1, static_cast<uint32_t>((i * stride) >> 32));
  Dev train(static_cast<size_t>(ts) * ld * 4);
  stage_rows(data, on_device, dim, rows, ld, train.as<float>(), st);

  // 2. k-means++ seeding from the seeded stream (src/kmeans.cpp:280-321)
  std::mt19937_64 gen(opt.seed ? opt.seed : std::random_device{}());
  std::uniform_real_distribution<double> uni(0.0, 1.0);
  const uint32_t first = static_cast<uint32_t>(gen() % ts);
  std::vector<double> u(std::max<uint32_t>(L, 2));
  for (double &v : u) v = uni(gen);
  Dev du(u.size() * 8), cen(static_cast<size_t>(L) * ld * 4), cnorm(static_cast<size_t>(L) * 4);
  Dev dist(static_cast<size_t>(ts) * 4), part(katoann_gpu_kmeanspp_scratch(ts)), chosen(L * 4ull);
  cuda_ok(cudaMemcpyAsync(du.p, u.data(), u.size() * 8, cudaMemcpyHostToDevice, st), "upload");
  gpu_ok(katoann_gpu_kmeanspp(train.as<float>(), ts, ld, L, first, du.as<double>(), cen.as<float>(),
                              dist.as<float>(), part.p, chosen.as<uint32_t>(), ks));

  // 3. Lloyd iterations on the sample; the residual is reported as the
  // reference's elkan reports it
  Dev assign(static_cast<size_t>(ts) * 4), best(static_cast<size_t>(ts) * 4), xn(static_cast<size_t>(ts) * 4);
  Dev sums(static_cast<size_t>(L) * ld * 8), counts(static_cast<size_t>(L) * 4), tmo(16);
  cuda_ok(cudaMemsetAsync(tmo.p, 0, 16, st), "memset");
  gpu_ok(katoann_gpu_row_norms(train.as<float>(), ts, ld, xn.as<float>(), ks));
  gpu_ok(katoann_gpu_row_norms(cen.as<float>(), L, ld, cnorm.as<float>(), ks));
  std::vector<float> hb(ts), hx(ts);
  cuda_ok(cudaMemcpyAsync(hx.data(), xn.p, ts * 4ull, cudaMemcpyDeviceToHost, st), "download");
  double prev = -1;
  for (uint32_t it = 0; it < opt.kmeans_iters; ++it) {
    gpu_ok(katoann_gpu_kmeans_assign(train.as<float>(), ts, ld, cen.as<float>(), cnorm.as<float>(), L,
                                     assign.as<uint32_t>(), best.as<float>(), tmo.as<uint32_t>(), ks));
    gpu_ok(katoann_gpu_kmeans_update(train.as<float>(), ts, ld, assign.as<uint32_t>(), L,
                                     sums.as<double>(), counts.as<uint32_t>(), cen.as<float>(),
                                     cnorm.as<float>(), ks));
    cuda_ok(cudaMemcpyAsync(hb.data(), best.p, ts * 4ull, cudaMemcpyDeviceToHost, st), "download");
    cuda_ok(cudaStreamSynchronize(st), "k-means");
    double res = 0;
    for (uint32_t i = 0; i < ts; ++i) res += std::max(0.0, static_cast<double>(hx[i]) + hb[i]);
    std::fprintf(stderr, "build: k-means iteration %u, residual %.6e\n", it + 1, res);
    if (prev > 0 && std::fabs(prev - res) / std::max(res, 1e-30) < 1e-5) break;
    prev = res;
  }
  uint32_t timeouts = 0;
  cuda_ok(cudaMemcpyAsync(&timeouts, tmo.p, 4, cudaMemcpyDeviceToHost, st), "download");
  cuda_ok(cudaStreamSynchronize(st), "k-means");
  if (timeouts) throw std::runtime_error("k-means assignment: a bounded pipeline wait ran out");
  train.reset();
  out.centroids.assign(static_cast<size_t>(L) * dim, 0.0f);
  cuda_ok(cudaMemcpy2D(out.centroids.data(), dim * 4, cen.p, ld * 4, dim * 4, L, cudaMemcpyDeviceToHost),
          "download centroids");

  // 4. every vector's nearest centroid, in chunks
  out.assign.resize(n);
  const uint32_t chunk = std::max<uint32_t>(1, std::min<uint32_t>(n, (1u << 30) / (ld * 4)));
  const bool direct = on_device && ld == dim && reinterpret_cast<uintptr_t>(data) % 16 == 0;
  Dev rowbuf(direct ? 16 : static_cast<size_t>(chunk) * ld * 4), ca(static_cast<size_t>(chunk) * 4);
  for (uint32_t r0 = 0; r0 < n; r0 += chunk) {
    const uint32_t m = std::min(chunk, n - r0);
    const float *x = data + static_cast<size_t>(r0) * dim;
    if (!direct) {
      stage_range(data, on_device, dim, r0, m, ld, rowbuf.as<float>(), st);
      x = rowbuf.as<float>();
    }
    gpu_ok(katoann_gpu_kmeans_assign(x, m, ld, cen.as<float>(), cnorm.as<float>(), L, ca.as<uint32_t>(),
                                     nullptr, tmo.as<uint32_t>(), ks));
    cuda_ok(cudaMemcpyAsync(out.assign.data() + r0, ca.p, m * 4ull, cudaMemcpyDeviceToHost, st), "download");
    cuda_ok(cudaStreamSynchronize(st), "assignment");
  }
  cuda_ok(cudaMemcpyAsync(&timeouts, tmo.p, 4, cudaMemcpyDeviceToHost, st), "download");
  cuda_ok(cudaStreamSynchronize(st), "assignment");
  if (timeouts) throw std::runtime_error("k-means assignment: a bounded pipeline wait ran out");

  // 5. the rotation: a list-order sample (src/index.cpp:516-533), its
  // covariance on the device, Jacobi on the host
  std::vector<uint32_t> sizes(L, 0);
  for (uint32_t a : out.assign) ++sizes[a];
  std::vector<uint64_t> start(L + 1, 0);
  for (uint32_t c = 0; c < L; ++c) start[c + 1] = start[c] + sizes[c];
  std::vector<uint32_t> by_list(n);
  {
    std::vector<uint64_t> at(start.begin(), start.end() - 1);
    for (uint32_t i = 0; i < n; ++i) by_list[at[out.assign[i]]++] = i;  // ids ascend in each list
  }
  const size_t target = std::min<size_t>(std::max<uint32_t>(opt.rotation_sample, 1024u), n);
  const size_t step = std::max<size_t>(1, n / target);
  std::vector<uint32_t> srows;
  srows.reserve(target);
  for (size_t g = 0; g < n && srows.size() < target; g += step) srows.push_back(by_list[g]);
  const uint32_t ns = static_cast<uint32_t>(srows.size());
  out.head_dims = default_head_dims(dim);
  if (ns >= 2 && dim >= 2) {
    Dev sample(static_cast<size_t>(ns) * ld * 4), mean(dim * 8ull), cov(static_cast<size_t>(dim) * dim * 8);
    stage_rows(data, on_device, dim, srows, ld, sample.as<float>(), st);
    gpu_ok(katoann_gpu_covariance(sample.as<float>(), ns, ld, dim, mean.as<double>(), cov.as<double>(), ks));
    std::vector<double> A(static_cast<size_t>(dim) * dim);
    cuda_ok(cudaMemcpyAsync(A.data(), cov.p, A.size() * 8, cudaMemcpyDeviceToHost, st), "download");
    cuda_ok(cudaStreamSynchronize(st), "covariance");
    jacobi_rotation(A, dim, opt.jacobi_sweeps, out.rotation);
  }
  return out;
}

void Index::build(const float *data, uint32_t n, uint32_t dim, const BuildOptions &opt,
                  const std::string &prefix) {
  const BuildResult b = partition(data, n, dim, opt, false);
  const uint32_t k = opt.nlist;
  std::vector<std::vector<uint32_t>> lists(k);
  for (uint32_t i = 0; i < n; ++i) lists[b.assign[i]].push_back(i);
  {
    std::ofstream f(prefix + ".meta", std::ios::binary);
    if (!f) throw std::runtime_error("cannot write " + prefix + ".meta");
    const uint32_t meta[5] = {dim, k, n, 0u, opt.normalized ? 1u : 0u};
    f.write(reinterpret_cast<const char *>(meta), sizeof(meta));
  }
  {
    std::ofstream f(prefix + ".centroids", std::ios::binary);
    f.write(reinterpret_cast<const char *>(b.centroids.data()), b.centroids.size() * sizeof(float));
    if (!f) throw std::runtime_error("cannot write " + prefix + ".centroids");
  }
  {
    std::ofstream f(prefix + ".invlist", std::ios::binary), g(prefix + ".norms", std::ios::binary);
    for (uint32_t c = 0; c < k; ++c) {
      const uint32_t sz = static_cast<uint32_t>(lists[c].size());
      f.write(reinterpret_cast<const char *>(&sz), 4);
      f.write(reinterpret_cast<const char *>(lists[c].data()), static_cast<std::streamsize>(sz) * 4);
      for (uint32_t id : lists[c])
        f.write(reinterpret_cast<const char *>(data + static_cast<size_t>(id) * dim), dim * sizeof(float));
      g.write(reinterpret_cast<const char *>(&sz), 4);
    }
    if (!f || !g) throw std::runtime_error("cannot write " + prefix + ".invlist");
  }
  const bool rotated = !b.rotation.empty();
  std::ofstream f(prefix + ".dimc", std::ios::binary);
  if (!f) throw std::runtime_error("cannot write " + prefix + ".dimc");
  const uint32_t hdr[8] = {kDimcMagic, 2u, dim, k, n, b.head_dims, rotated ? 1u : 0u, 0u};
  f.write(reinterpret_cast<const char *>(hdr), sizeof(hdr));
  if (rotated)
    f.write(reinterpret_cast<const char *>(b.rotation.data()), static_cast<std::streamsize>(b.rotation.size() * 4));
  if (!f) throw std::runtime_error("cannot write " + prefix + ".dimc");
}

}  // namespace katoann
