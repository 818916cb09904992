// Index::build on the host: k-means++ seeding and Lloyd iterations on a
// training sample, assignment of every vector to its nearest centroid, the
// reference's file format, and the PCA rotation by cyclic Jacobi.
//
// Follows Index::build (src/index.cpp:419-514), compute_rotation_ (:516-533),
// pca_rotation (:276-380) and write_dimc_ (:535-545), with k-means from
// src/kmeans.cpp (k-means++ :280-321; the reference's Elkan iteration
// :73-187 reaches the same Lloyd fixed point with fewer distance
// evaluations). The partition need not match the reference's bit for bit:
// search parity is defined over the index files, whoever wrote them.
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
#include <vector>

#include "katoann/index.h"

namespace katoann {

namespace {

constexpr uint32_t kDimcMagic = 0x434D4944u;

inline float l2sq(const float *a, const float *b, uint32_t d) {
  float s = 0.0f;
  for (uint32_t k = 0; k < d; ++k) {
    const float t = a[k] - b[k];
    s += t * t;
  }
  return s;
}

void nearest_centers(const float *x, size_t n, uint32_t d, const float *c, uint32_t k,
                     uint32_t *out) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < static_cast<int64_t>(n); ++i) {
    const float *xi = x + static_cast<size_t>(i) * d;
    float best = FLT_MAX;
    uint32_t bi = 0;
    for (uint32_t j = 0; j < k; ++j) {
      const float v = l2sq(xi, c + static_cast<size_t>(j) * d, d);
      if (v < best) {
        best = v;
        bi = j;
      }
    }
    out[i] = bi;
  }
}

// D^2 seeding (src/kmeans.cpp:280-321).
void kmeanspp(const float *x, size_t n, uint32_t d, float *centers, uint32_t k, uint64_t seed) {
  std::mt19937_64 gen(seed ? seed : std::random_device{}());
  std::uniform_real_distribution<double> uni(0.0, 1.0);
  const size_t first = static_cast<size_t>(gen() % n);
  std::memcpy(centers, x + first * d, d * sizeof(float));
  std::vector<float> dist(n);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < static_cast<int64_t>(n); ++i)
    dist[i] = l2sq(x + static_cast<size_t>(i) * d, centers, d);
  std::vector<char> taken(n, 0);
  taken[first] = 1;
  for (uint32_t m = 1; m < k; ++m) {
    double sum = 0;
    for (size_t i = 0; i < n; ++i) sum += dist[i];
    size_t next = 0;
    if (sum > 0) {
      const double dart = uni(gen) * sum;
      double acc = 0;
      next = n - 1;
      for (size_t i = 0; i < n; ++i) {
        acc += dist[i];
        if (dart < acc) {
          next = i;
          break;
        }
      }
    } else {
      next = static_cast<size_t>(gen() % n);
    }
    if (taken[next] && sum > 0) {
      --m;
      continue;
    }
    taken[next] = 1;
    float *cm = centers + static_cast<size_t>(m) * d;
    std::memcpy(cm, x + next * d, d * sizeof(float));
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < static_cast<int64_t>(n); ++i)
      dist[i] = std::min(dist[i], l2sq(x + static_cast<size_t>(i) * d, cm, d));
  }
}

void lloyd(const float *x, size_t n, uint32_t d, float *centers, uint32_t k, uint32_t iters) {
  std::vector<uint32_t> a(n);
  std::vector<double> sums(static_cast<size_t>(k) * d);
  std::vector<uint64_t> cnt(k);
  double prev = -1;
  for (uint32_t it = 0; it < iters; ++it) {
    nearest_centers(x, n, d, centers, k, a.data());
    std::fill(sums.begin(), sums.end(), 0.0);
    std::fill(cnt.begin(), cnt.end(), 0);
    for (size_t i = 0; i < n; ++i) {
      const float *xi = x + i * d;
      double *s = sums.data() + static_cast<size_t>(a[i]) * d;
      for (uint32_t t = 0; t < d; ++t) s[t] += xi[t];
      ++cnt[a[i]];
    }
    for (uint32_t c = 0; c < k; ++c)
      if (cnt[c])
        for (uint32_t t = 0; t < d; ++t)
          centers[static_cast<size_t>(c) * d + t] =
              static_cast<float>(sums[static_cast<size_t>(c) * d + t] / static_cast<double>(cnt[c]));
    double res = 0;
#pragma omp parallel for reduction(+ : res)
    for (int64_t i = 0; i < static_cast<int64_t>(n); ++i)
      res += l2sq(x + static_cast<size_t>(i) * d, centers + static_cast<size_t>(a[i]) * d, d);
    std::fprintf(stderr, "build: k-means iteration %u, residual %.6e\n", it + 1, res);
    if (prev > 0 && std::fabs(prev - res) / std::max(res, 1e-30) < 1e-5) break;
    prev = res;
  }
}

// Principal axes of a sample by cyclic Jacobi on its covariance
// (src/index.cpp:276-380). Row j of rot is the axis of j-th largest variance.
bool pca_rotation(std::vector<float> &sample, size_t n, uint32_t d, uint32_t sweeps,
                  std::vector<float> &rot) {
  if (n < 2 || d < 2) return false;
  std::vector<double> mean(d, 0.0);
  for (size_t s = 0; s < n; ++s)
    for (uint32_t t = 0; t < d; ++t) mean[t] += sample[s * d + t];
  for (uint32_t t = 0; t < d; ++t) mean[t] /= static_cast<double>(n);
  std::vector<double> A(static_cast<size_t>(d) * d, 0.0);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t i = 0; i < static_cast<int64_t>(d); ++i)
    for (size_t s = 0; s < n; ++s) {
      const float *x = sample.data() + s * d;
      const double xi = x[i] - mean[i];
      double *row = A.data() + static_cast<size_t>(i) * d;
      for (uint32_t j = static_cast<uint32_t>(i); j < d; ++j) row[j] += xi * (x[j] - mean[j]);
    }
  for (uint32_t i = 0; i < d; ++i)
    for (uint32_t j = i; j < d; ++j) {
      const double v = A[static_cast<size_t>(i) * d + j] / static_cast<double>(n);
      A[static_cast<size_t>(i) * d + j] = v;
      A[static_cast<size_t>(j) * d + i] = v;
    }
  std::vector<double> V(static_cast<size_t>(d) * d, 0.0);
  for (uint32_t i = 0; i < d; ++i) V[static_cast<size_t>(i) * d + i] = 1.0;
  double diag = 0;
  for (uint32_t i = 0; i < d; ++i) diag += A[static_cast<size_t>(i) * d + i] * A[static_cast<size_t>(i) * d + i];
  sweeps = std::clamp<uint32_t>(sweeps, 1u, 64u);
  for (uint32_t sw = 0; sw < sweeps; ++sw) {
    double offd = 0;
    for (uint32_t i = 0; i < d; ++i)
      for (uint32_t j = i + 1; j < d; ++j) offd += 2.0 * A[static_cast<size_t>(i) * d + j] * A[static_cast<size_t>(i) * d + j];
    std::fprintf(stderr, "rotation: Jacobi sweep %u/%u, off-diagonal %.3e\n", sw + 1, sweeps, offd);
    if (offd <= 1e-18 * std::max(diag, 1e-300)) break;
    for (uint32_t p = 0; p + 1 < d; ++p)
      for (uint32_t q = p + 1; q < d; ++q) {
        const double apq = A[static_cast<size_t>(p) * d + q];
        const double app = A[static_cast<size_t>(p) * d + p], aqq = A[static_cast<size_t>(q) * d + q];
        if (std::fabs(apq) <= 1e-14 * std::sqrt(std::fabs(app * aqq)) + 1e-300) continue;
        const double theta = 0.5 * (aqq - app) / apq;
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(1.0 + theta * theta));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        double *rp = A.data() + static_cast<size_t>(p) * d, *rq = A.data() + static_cast<size_t>(q) * d;
        for (uint32_t k = 0; k < d; ++k) {
          const double xp = rp[k], xq = rq[k];
          rp[k] = c * xp - s * xq;
          rq[k] = s * xp + c * xq;
        }
        for (uint32_t k = 0; k < d; ++k) {
          double *row = A.data() + static_cast<size_t>(k) * d;
          const double xp = row[p], xq = row[q];
          row[p] = c * xp - s * xq;
          row[q] = s * xp + c * xq;
        }
        for (uint32_t k = 0; k < d; ++k) {
          double *row = V.data() + static_cast<size_t>(k) * d;
          const double xp = row[p], xq = row[q];
          row[p] = c * xp - s * xq;
          row[q] = s * xp + c * xq;
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
  return true;
}

}  // namespace

void Index::build(const float *data, uint32_t n, uint32_t dim, const BuildOptions &opt,
                  const std::string &prefix) {
  if (dim == 0 || dim > kMaxDim) throw std::invalid_argument("dimension must be 1 to 4096");
  if (n == 0 || opt.nlist == 0 || opt.nlist > n) throw std::invalid_argument("need at least nlist vectors");
  const uint32_t k = opt.nlist;
  const uint32_t ts = std::min(opt.train_size, n);
  if (ts > (1u << 23)) throw std::invalid_argument("train_size is limited to 8388608");
  // Strided training sample (src/index.cpp:430-443).
  std::vector<float> train(static_cast<size_t>(ts) * dim);
  const uint64_t stride = static_cast<uint64_t>(n) * (1ull << 32) / ts;
  for (uint32_t i = 0; i < ts; ++i) {
    uint32_t src = ts == n ? i : static_cast<uint32_t>((static_cast<uint64_t>(i) * stride) >> 32);
    if (src >= n) src = n - 1;
    std::memcpy(train.data() + static_cast<size_t>(i) * dim, data + static_cast<size_t>(src) * dim,
                dim * sizeof(float));
  }
  std::vector<float> centroids(static_cast<size_t>(k) * dim);
  kmeanspp(train.data(), ts, dim, centroids.data(), k, opt.seed);
  lloyd(train.data(), ts, dim, centroids.data(), k, opt.kmeans_iters);
  train.clear();
  train.shrink_to_fit();
  std::vector<uint32_t> assign(n);
  nearest_centers(data, n, dim, centroids.data(), k, assign.data());
  std::vector<std::vector<uint32_t>> lists(k);
  for (uint32_t i = 0; i < n; ++i) lists[assign[i]].push_back(i);
  {
    std::ofstream f(prefix + ".meta", std::ios::binary);
    if (!f) throw std::runtime_error("cannot write " + prefix + ".meta");
    const uint32_t meta[5] = {dim, k, n, 0u, opt.normalized ? 1u : 0u};
    f.write(reinterpret_cast<const char *>(meta), sizeof(meta));
  }
  {
    std::ofstream f(prefix + ".centroids", std::ios::binary);
    f.write(reinterpret_cast<const char *>(centroids.data()), centroids.size() * sizeof(float));
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
  // Rotation sample in list order (src/index.cpp:516-533).
  const size_t target = std::min<size_t>(std::max<uint32_t>(opt.rotation_sample, 1024u), n);
  const size_t step = std::max<size_t>(1, n / target);
  std::vector<float> sample;
  sample.reserve(target * dim);
  size_t taken = 0, gi = 0;
  for (uint32_t c = 0; c < k && taken < target; ++c)
    for (size_t i = 0; i < lists[c].size() && taken < target; ++i, ++gi) {
      if (gi % step) continue;
      const float *v = data + static_cast<size_t>(lists[c][i]) * dim;
      sample.insert(sample.end(), v, v + dim);
      ++taken;
    }
  std::vector<float> rot;
  const bool rotated = taken >= 2 && pca_rotation(sample, taken, dim, opt.jacobi_sweeps, rot);
  const uint32_t dc = (dim + 63) / 64 * 64;
  const uint32_t head = std::min(std::max(64u, (dim / 4 + 63) / 64 * 64), dc);
  std::ofstream f(prefix + ".dimc", std::ios::binary);
  if (!f) throw std::runtime_error("cannot write " + prefix + ".dimc");
  const uint32_t hdr[8] = {kDimcMagic, 2u, dim, k, n, head, rotated ? 1u : 0u, 0u};
  f.write(reinterpret_cast<const char *>(hdr), sizeof(hdr));
  if (rotated) f.write(reinterpret_cast<const char *>(rot.data()), static_cast<std::streamsize>(rot.size() * 4));
  if (!f) throw std::runtime_error("cannot write " + prefix + ".dimc");
}

}  // namespace katoann
