// CPU restatement of the reference's batched IVF search over 16-bit
// split-byte codes. TEST INFRASTRUCTURE, not the product: tests, the smoke
// check and the CPU-baseline leg of bench.py call it as the checker; the GPU
// library never links it.
//
// Portable C++17 (no intrinsics; built with -ffp-contract=off and explicit
// fmaf where the reference's AVX-512 code fuses), so it runs and gives the
// same bits on x86-64 and aarch64. It is pinned against the reference itself
// by the golden fixtures in tests/golden (made by tests/golden/make_golden.py
// from a build of the reference's own sources).
//
// Selection rule (the reference's, made deterministic): candidates are ranked
// by (distance, id) lexicographically. That is exactly the reference's
// Selection::kLocal result for lists whose ids ascend (every index written by
// Index::build), and equals Selection::kThreshold wherever the reference's
// threshold pass has no distance tie on the survivor boundary (there it depends
// on the OpenMP schedule). Final top-k follows the reference's heap exactly.
#include <omp.h>

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <numeric>
#include <queue>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace oracle {

using PFI = std::pair<float, uint32_t>;

constexpr uint32_t kMaxDim = 4096;            // include/katoann/kernels.h:177
constexpr uint32_t kDimcMagic = 0x434D4944u;  // src/index.cpp:27

uint32_t round_up(uint32_t x, uint32_t m) { return (x + m - 1) / m * m; }

// Sum of 16 lane accumulators in the order of GCC's _mm512_reduce_add_ps:
// lanes (l, l+8), then (l, l+4), then (l, l+2), then lanes 0 and 1.
inline float reduce16(const float *a) {
  float t3[8], t6[4];
  for (int l = 0; l < 8; ++l) t3[l] = a[l + 8] + a[l];
  for (int l = 0; l < 4; ++l) t6[l] = t3[l + 4] + t3[l];
  const float t8_0 = t6[0] + t6[2], t8_1 = t6[1] + t6[3];
  return t8_0 + t8_1;
}

// s + x * r with the product rounded first (no fusion).
inline float mul_add(float s, float x, float r) {
  volatile float p = x * r;
  return s + p;
}

// One output of the reference's rotation, <x, r> over d floats, with the
// arithmetic of rotate_rows_serial / rotate_tile4x4 (src/index.cpp:139-208):
// output columns j < (d & ~3) use 16 lane accumulators over 16-float chunks
// (fused multiply-add), the reduction above, then the scalar tail over the
// last d % 16 dimensions; the last d % 4 columns are one chain over all d
// (src/index.cpp:171-179, :247-257). The scalar chains follow the reference as
// GCC 13 compiles it (-O3 -march=native): the loop is vectorised four
// elements at a time with the products rounded before each in-order add, and
// the remaining (length % 4) elements are fused. Dimensions that are a
// multiple of 16 never reach either chain.
// The scalar chain over dimensions [k, d) after the lanes: products rounded
// before each add for the first (d - k) & ~3 of them, fused for the rest.
inline float dot_tail(const float *x, const float *r, uint32_t k, uint32_t d, float s) {
  const uint32_t m = k + ((d - k) & ~3u);
  for (; k < m; ++k) s = mul_add(s, x[k], r[k]);
  for (; k < d; ++k) s = std::fmaf(x[k], r[k], s);
  return s;
}

inline float rotate_dot(const float *x, const float *r, uint32_t d, bool lanes) {
  if (!lanes) return dot_tail(x, r, 0, d, 0.0f);
  float acc[16] = {0};
  uint32_t k = 0;
  for (; k + 16 <= d; k += 16)
    for (int l = 0; l < 16; ++l) acc[l] = std::fmaf(x[k + l], r[k + l], acc[l]);
  return dot_tail(x, r, k, d, reduce16(acc));
}

// Every output is rotate_dot's arithmetic. For speed (a 10M-row index is
// coded here), four rows share each pass over a rotation row, and a thread
// walks 32 rows against all columns so that their values stay in cache.
void rotate_rows(const float *in, float *out, size_t nrows, uint32_t d, const float *rot) {
  const uint32_t d4 = d & ~3u, d16 = d & ~15u;
  constexpr size_t kTile = 32, kSub = 4;
  const int64_t tiles = static_cast<int64_t>((nrows + kTile - 1) / kTile);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t t = 0; t < tiles; ++t) {
    const size_t i0 = static_cast<size_t>(t) * kTile, i1 = std::min(nrows, i0 + kTile);
    for (uint32_t j = 0; j < d; ++j) {
      const float *r = rot + static_cast<size_t>(j) * d;
      size_t i = i0;
      for (; j < d4 && i + kSub <= i1; i += kSub) {
        const float *x[kSub];
        for (size_t u = 0; u < kSub; ++u) x[u] = in + (i + u) * d;
        float acc[kSub][16] = {};
        for (uint32_t k = 0; k < d16; k += 16)
          for (size_t u = 0; u < kSub; ++u)
            for (int l = 0; l < 16; ++l) acc[u][l] = std::fmaf(x[u][k + l], r[k + l], acc[u][l]);
        for (size_t u = 0; u < kSub; ++u)
          out[(i + u) * d + j] = dot_tail(x[u], r, d16, d, reduce16(acc[u]));
      }
      for (; i < i1; ++i) out[i * d + j] = rotate_dot(in + i * d, r, d, j < d4);
    }
  }
}

// Quantization of one value, src/index.cpp:669-670 (also :735-736, :925-926).
inline uint32_t quantize1(float v, float lo, double inv_step) {
  long r = std::lround((static_cast<double>(v) - lo) * inv_step);
  if (r < 0) r = 0;
  else if (r > 65535) r = 65535;
  return static_cast<uint32_t>(r);
}

// Distance value, src/kernels.cpp:166-168 / :208-210.
inline float to_dist(int64_t l2, double step_sq) {
  return static_cast<float>(static_cast<double>(l2) * step_sq);
}

struct Index {
  uint32_t dim = 0, nlist = 0, npts = 0, dc = 0, head = 0;
  bool normalized = false, rotated = false, has_dimc = false;
  float lo = 0;
  double inv_step = 0, step = 0, step_sq = 0;
  std::vector<float> centroids, rotation;
  std::vector<uint32_t> list_off;  // nlist + 1, rows of list c: [off[c], off[c+1])
  std::vector<uint32_t> ids;       // per row
  std::vector<uint8_t> hi, lo_plane;  // rows x dc, row-major
  std::vector<int64_t> norm, hinorm, headnorm;
  std::vector<uint8_t> chi, clo;
  std::vector<int64_t> cnorm;
  std::vector<uint32_t> id_row;  // id -> row (UINT32_MAX if absent)
};

// src/index.cpp:550-611
void read_files(Index &x, const std::string &prefix, std::vector<float> &raw, uint32_t *stored) {
  {
    std::ifstream f(prefix + ".meta", std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + prefix + ".meta");
    uint32_t meta[3] = {0, 0, 0};
    f.read(reinterpret_cast<char *>(meta), sizeof(meta));
    if (!f) throw std::runtime_error("truncated " + prefix + ".meta");
    x.dim = meta[0];
    x.nlist = meta[1];
    x.npts = meta[2];
    uint32_t extra[2] = {0, 0};
    f.read(reinterpret_cast<char *>(extra), sizeof(extra));
    if (f.gcount() == static_cast<std::streamsize>(sizeof(extra))) {
      if (extra[0] != 0) throw std::runtime_error("only the L2 metric is supported");
      x.normalized = extra[1] != 0;
    }
  }
  if (x.dim == 0 || x.dim > kMaxDim || x.nlist == 0)
    throw std::runtime_error("bad header in " + prefix + ".meta");
  x.centroids.assign(static_cast<size_t>(x.nlist) * x.dim, 0.0f);
  {
    std::ifstream f(prefix + ".centroids", std::ios::binary);
    f.read(reinterpret_cast<char *>(x.centroids.data()), x.centroids.size() * sizeof(float));
    if (!f) throw std::runtime_error("cannot read " + prefix + ".centroids");
  }
  std::ifstream f(prefix + ".invlist", std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + prefix + ".invlist");
  x.list_off.assign(x.nlist + 1, 0);
  uint64_t total = 0;
  for (uint32_t c = 0; c < x.nlist; ++c) {
    uint32_t sz = 0;
    f.read(reinterpret_cast<char *>(&sz), sizeof(sz));
    if (!f) break;
    const size_t r0 = x.ids.size();
    x.ids.resize(r0 + sz);
    f.read(reinterpret_cast<char *>(x.ids.data() + r0), sz * sizeof(uint32_t));
    raw.resize((r0 + sz) * static_cast<size_t>(x.dim));
    f.read(reinterpret_cast<char *>(raw.data() + r0 * x.dim),
           static_cast<size_t>(sz) * x.dim * sizeof(float));
    total += sz;
    x.list_off[c + 1] = static_cast<uint32_t>(total);
  }
  if (!f || total != x.npts) throw std::runtime_error("truncated " + prefix + ".invlist");
  std::ifstream g(prefix + ".dimc", std::ios::binary);
  x.has_dimc = static_cast<bool>(g);
  if (x.has_dimc) {
    uint32_t hdr[8] = {0};
    g.read(reinterpret_cast<char *>(hdr), sizeof(hdr));
    if (!g || hdr[0] != kDimcMagic || (hdr[1] != 1u && hdr[1] != 2u))
      throw std::runtime_error("bad header in " + prefix + ".dimc");
    if (hdr[2] != x.dim || hdr[3] != x.nlist || hdr[4] != x.npts)
      throw std::runtime_error(prefix + ".dimc does not match the index");
    *stored = hdr[5];
    x.rotated = hdr[6] == 1u;
    if (x.rotated) {
      x.rotation.resize(static_cast<size_t>(x.dim) * x.dim);
      g.read(reinterpret_cast<char *>(x.rotation.data()),
             static_cast<std::streamsize>(x.rotation.size() * sizeof(float)));
      if (!g) throw std::runtime_error("truncated rotation in " + prefix + ".dimc");
    }
  }
}

// Coding of an index whose files have been read (src/index.cpp:613-750,
// :777-807): raw holds the unrotated vectors in list order.
void code_index(Index *x, std::vector<float> &raw, uint32_t dims, bool raw_rotated = false) {
  const uint32_t d = x->dim;
  const size_t n = x->npts;
  if (x->rotated && n && !raw_rotated) {
    std::vector<float> tmp(raw.size());
    rotate_rows(raw.data(), tmp.data(), n, d, x->rotation.data());
    raw.swap(tmp);
  }
  x->dc = round_up(d, 64u);
  const uint32_t Dc = x->dc;
  float glo = FLT_MAX, ghi = -FLT_MAX;
#pragma omp parallel for reduction(min : glo) reduction(max : ghi)
  for (int64_t i = 0; i < static_cast<int64_t>(raw.size()); ++i) {
    glo = std::min(glo, raw[i]);
    ghi = std::max(ghi, raw[i]);
  }
  x->lo = glo;
  const double rng = static_cast<double>(ghi) - glo;
  x->inv_step = 65535.0 / rng;
  x->step = rng / 65535.0;
  x->step_sq = x->step * x->step;
  x->hi.assign(n * Dc, 0);
  x->lo_plane.assign(n * Dc, 0);
  x->norm.assign(n, 0);
  x->hinorm.assign(n, 0);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < static_cast<int64_t>(n); ++i) {
    int64_t nrm = 0, nh = 0;
    for (uint32_t k = 0; k < d; ++k) {
      const uint32_t q = quantize1(raw[static_cast<size_t>(i) * d + k], x->lo, x->inv_step);
      const uint8_t qh = static_cast<uint8_t>(q >> 8);
      x->hi[static_cast<size_t>(i) * Dc + k] = qh;
      x->lo_plane[static_cast<size_t>(i) * Dc + k] = static_cast<uint8_t>(q & 0xFF);
      nrm += static_cast<int64_t>(q) * q;
      nh += static_cast<int64_t>(qh) * qh;
    }
    x->norm[i] = nrm;
    x->hinorm[i] = nh;
  }
  if (x->has_dimc && dims) {
    if (dims % 64 || dims > Dc)  // src/index.cpp:695-696
      throw std::invalid_argument("prefix_dims must be a multiple of 64 within the dimension");
    x->headnorm.assign(n, 0);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < static_cast<int64_t>(n); ++i) {
      int64_t s = 0;
      for (uint32_t k = 0; k < dims; ++k) {
        const int64_t v = x->hi[static_cast<size_t>(i) * Dc + k];
        s += v * v;
      }
      x->headnorm[i] = s;
    }
    x->head = dims;
  }
  // Centroid planes with the database scale (src/index.cpp:718-750).
  std::vector<float> cen = x->centroids;
  if (x->rotated) rotate_rows(x->centroids.data(), cen.data(), x->nlist, d, x->rotation.data());
  x->chi.assign(static_cast<size_t>(x->nlist) * Dc, 0);
  x->clo.assign(static_cast<size_t>(x->nlist) * Dc, 0);
  x->cnorm.assign(x->nlist, 0);
  for (uint32_t c = 0; c < x->nlist; ++c) {
    int64_t nrm = 0;
    for (uint32_t k = 0; k < d; ++k) {
      const uint32_t q = quantize1(cen[static_cast<size_t>(c) * d + k], x->lo, x->inv_step);
      x->chi[static_cast<size_t>(c) * Dc + k] = static_cast<uint8_t>(q >> 8);
      x->clo[static_cast<size_t>(c) * Dc + k] = static_cast<uint8_t>(q & 0xFF);
      nrm += static_cast<int64_t>(q) * q;
    }
    x->cnorm[c] = nrm;
  }
  // id -> row (src/index.cpp:795-806); ids >= npts are not mapped.
  x->id_row.assign(n, UINT32_MAX);
  for (uint32_t r = 0; r < n; ++r)
    if (x->ids[r] < n) x->id_row[x->ids[r]] = r;
}

Index *load(const std::string &prefix, uint32_t prefix_dims) {
  auto x = std::make_unique<Index>();
  std::vector<float> raw;
  uint32_t stored = 0;
  read_files(*x, prefix, raw, &stored);
  code_index(x.get(), raw, prefix_dims ? prefix_dims : stored);
  return x.release();
}

// Exact squared L2 from full codes (hi, lo) or from high bytes over `dims`.
inline int64_t dot_full(const uint8_t *qh, const uint8_t *ql, const uint8_t *xh, const uint8_t *xl,
                        uint32_t dims) {
  int64_t hh = 0, mx = 0, ll = 0;
  for (uint32_t k = 0; k < dims; ++k) {
    hh += static_cast<int32_t>(qh[k]) * xh[k];
    mx += static_cast<int32_t>(qh[k]) * xl[k] + static_cast<int32_t>(ql[k]) * xh[k];
    ll += static_cast<int32_t>(ql[k]) * xl[k];
  }
  return (hh << 16) + (mx << 8) + ll;
}
inline int64_t dot_high(const uint8_t *qh, const uint8_t *xh, uint32_t dims) {
  int64_t s = 0;
  for (uint32_t k = 0; k < dims; ++k) s += static_cast<int32_t>(qh[k]) * xh[k];
  return s;
}

struct Quantized {
  std::vector<uint8_t> hi, lo;
  std::vector<int64_t> norm, hinorm, h0norm;
};

// src/index.cpp:917-943
void quantize_queries(const Index &x, const float *fq, uint32_t B, Quantized &q) {
  const uint32_t d = x.dim, Dc = x.dc;
  q.hi.assign(static_cast<size_t>(B) * Dc, 0);
  q.lo.assign(static_cast<size_t>(B) * Dc, 0);
  q.norm.assign(B, 0);
  q.hinorm.assign(B, 0);
  q.h0norm.assign(B, 0);
  const uint32_t dh = std::min(x.head, d);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < static_cast<int64_t>(B); ++i) {
    int64_t nrm = 0, nh = 0, n0 = 0;
    for (uint32_t k = 0; k < d; ++k) {
      const uint32_t v = quantize1(fq[static_cast<size_t>(i) * d + k], x.lo, x.inv_step);
      const uint8_t vh = static_cast<uint8_t>(v >> 8);
      q.hi[static_cast<size_t>(i) * Dc + k] = vh;
      q.lo[static_cast<size_t>(i) * Dc + k] = static_cast<uint8_t>(v & 0xFF);
      nrm += static_cast<int64_t>(v) * v;
      nh += static_cast<int64_t>(vh) * vh;
      if (k < dh) n0 += static_cast<int64_t>(vh) * vh;
    }
    q.norm[i] = nrm;
    q.hinorm[i] = nh;
    q.h0norm[i] = n0;
  }
}

// src/index.cpp:846-877, with the same standard-library calls, so ties on the
// nprobe boundary resolve as in the reference.
void coarse(const Index &x, const Quantized &q, uint32_t B, uint32_t nprobe, uint32_t *probed) {
  const uint32_t Dc = x.dc, L = x.nlist;
  const uint32_t np = std::min(nprobe, L);
#pragma omp parallel
  {
    std::vector<float> dq(L);
    std::vector<uint32_t> ord(L);
#pragma omp for schedule(dynamic, 1)
    for (int64_t i = 0; i < static_cast<int64_t>(B); ++i) {
      const uint8_t *qh = q.hi.data() + static_cast<size_t>(i) * Dc;
      const uint8_t *ql = q.lo.data() + static_cast<size_t>(i) * Dc;
      for (uint32_t c = 0; c < L; ++c) {
        const int64_t dot = dot_full(qh, ql, x.chi.data() + static_cast<size_t>(c) * Dc,
                                     x.clo.data() + static_cast<size_t>(c) * Dc, Dc);
        dq[c] = to_dist(q.norm[i] + x.cnorm[c] - 2 * dot, x.step_sq);
      }
      std::iota(ord.begin(), ord.end(), 0u);
      if (np < L)
        std::nth_element(ord.begin(), ord.begin() + np, ord.end(),
                         [&](uint32_t a, uint32_t b) { return dq[a] < dq[b]; });
      std::sort(ord.begin(), ord.begin() + np,
                [&](uint32_t a, uint32_t b) { return dq[a] < dq[b]; });
      uint32_t *pr = probed + static_cast<size_t>(i) * nprobe;
      for (uint32_t p = 0; p < np; ++p) pr[p] = ord[p];
      for (uint32_t p = np; p < nprobe; ++p) pr[p] = ord[np - 1];
    }
  }
}

// Lexicographic (distance, id) bounded max-heap.
struct TopS {
  std::priority_queue<PFI> h;
  uint32_t cap = 0;
  void push(float dd, uint32_t id) {
    if (h.size() < cap) h.emplace(dd, id);
    else if (PFI(dd, id) < h.top()) {
      h.pop();
      h.emplace(dd, id);
    }
  }
};

// src/index.cpp:384-398
void emit_topk(std::priority_queue<PFI> &h, uint32_t K, uint32_t *ids, float *dists) {
  std::vector<PFI> tmp;
  while (!h.empty()) {
    tmp.push_back(h.top());
    h.pop();
  }
  std::reverse(tmp.begin(), tmp.end());
  for (uint32_t i = 0; i < K; ++i) {
    dists[i] = i < tmp.size() ? tmp[i].first : FLT_MAX;
    ids[i] = i < tmp.size() ? tmp[i].second : UINT32_MAX;
  }
}

// ranking: 0 full, 1 high bytes, 2 prefix (include/katoann/index.h:45-49).
void search(const Index &x, const float *queries, uint32_t B, uint32_t K, uint32_t nprobe,
            int ranking, uint32_t survivors, uint32_t *out_ids, float *out_dists) {
  if (B == 0) return;  // src/index.cpp:879-904
  if (x.nlist == 0) throw std::logic_error("search before load");
  if (K == 0 || nprobe == 0 || nprobe > x.nlist)
    throw std::invalid_argument("need k >= 1 and 1 <= nprobe <= nlist");
  if (ranking == 2 && x.head == 0)
    throw std::invalid_argument("prefix ranking needs the rotation file (.dimc)");
  const uint32_t d = x.dim, Dc = x.dc;
  std::vector<float> fq(queries, queries + static_cast<size_t>(B) * d);
  if (x.rotated) rotate_rows(queries, fq.data(), B, d, x.rotation.data());
  Quantized q;
  quantize_queries(x, fq.data(), B, q);
  std::vector<uint32_t> probed(static_cast<size_t>(B) * nprobe);
  coarse(x, q, B, nprobe, probed.data());
  // Inversion, src/index.cpp:403-412 (list order does not affect the result).
  std::vector<std::vector<uint32_t>> c2q(x.nlist);
  for (uint32_t i = 0; i < B; ++i)
    for (uint32_t p = 0; p < nprobe; ++p) c2q[probed[static_cast<size_t>(i) * nprobe + p]].push_back(i);
  const bool full = ranking == 0;
  const uint32_t S = full ? K : std::max(survivors, K);
  const uint32_t scan = ranking == 2 ? x.head : Dc;
  const int Tn = omp_get_max_threads();
  std::vector<std::vector<TopS>> th(Tn, std::vector<TopS>(B));
  for (auto &v : th)
    for (auto &t : v) t.cap = S;
#pragma omp parallel
  {
    std::vector<TopS> &mine = th[omp_get_thread_num()];
#pragma omp for schedule(dynamic, 1)
    for (int64_t c = 0; c < static_cast<int64_t>(x.nlist); ++c) {
      for (uint32_t i : c2q[c]) {
        const uint8_t *qh = q.hi.data() + static_cast<size_t>(i) * Dc;
        const uint8_t *ql = q.lo.data() + static_cast<size_t>(i) * Dc;
        for (uint32_t r = x.list_off[c]; r < x.list_off[c + 1]; ++r) {
          const uint8_t *xh = x.hi.data() + static_cast<size_t>(r) * Dc;
          float dd;
          if (full) {
            const int64_t dot = dot_full(qh, ql, xh, x.lo_plane.data() + static_cast<size_t>(r) * Dc, Dc);
            dd = to_dist(q.norm[i] + x.norm[r] - 2 * dot, x.step_sq);
          } else if (ranking == 2) {
            dd = to_dist(q.h0norm[i] + x.headnorm[r] - 2 * dot_high(qh, xh, scan), x.step_sq);
          } else {
            dd = to_dist(q.hinorm[i] + x.hinorm[r] - 2 * dot_high(qh, xh, scan), x.step_sq);
          }
          mine[i].push(dd, x.ids[r]);
        }
      }
    }
  }
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < static_cast<int64_t>(B); ++i) {
    TopS merged;
    merged.cap = S;
    for (int t = 0; t < Tn; ++t) {
      auto &h = th[t][i].h;
      while (!h.empty()) {
        merged.push(h.top().first, h.top().second);
        h.pop();
      }
    }
    uint32_t *ids = out_ids + static_cast<size_t>(i) * K;
    float *dists = out_dists + static_cast<size_t>(i) * K;
    if (full) {
      emit_topk(merged.h, K, ids, dists);
      continue;
    }
    // Refinement, src/index.cpp:1081-1125: survivors in descending (rank
    // distance, id) order, exact distance, heap with a strict < on distance.
    const uint8_t *qh = q.hi.data() + static_cast<size_t>(i) * Dc;
    const uint8_t *ql = q.lo.data() + static_cast<size_t>(i) * Dc;
    std::priority_queue<PFI> fin;
    while (!merged.h.empty()) {
      const uint32_t id = merged.h.top().second;
      merged.h.pop();
      if (id >= x.npts) continue;
      const uint32_t r = x.id_row[id];
      if (r == UINT32_MAX) continue;
      const int64_t dot = dot_full(qh, ql, x.hi.data() + static_cast<size_t>(r) * Dc,
                                   x.lo_plane.data() + static_cast<size_t>(r) * Dc, Dc);
      const float dd = to_dist(q.norm[i] + x.norm[r] - 2 * dot, x.step_sq);
      if (fin.size() < K) fin.emplace(dd, id);
      else if (dd < fin.top().first) {
        fin.pop();
        fin.emplace(dd, id);
      }
    }
    emit_topk(fin, K, ids, dists);
  }
}

thread_local std::string g_err;

template <class F>
int guarded(F &&f) {
  try {
    f();
    return 0;
  } catch (const std::invalid_argument &e) {
    g_err = e.what();
    return -1;
  } catch (const std::logic_error &e) {
    g_err = e.what();
    return -3;
  } catch (const std::exception &e) {
    g_err = e.what();
    return -2;
  }
}

}  // namespace oracle

using oracle::Index;

extern "C" {

const char *oracle_last_error() { return oracle::g_err.c_str(); }

void *oracle_load(const char *prefix, uint32_t prefix_dims) {
  Index *x = nullptr;
  if (oracle::guarded([&] { x = oracle::load(prefix, prefix_dims); })) return nullptr;
  return x;
}

void oracle_free(void *h) { delete static_cast<Index *>(h); }

// An oracle index from in-memory arrays in the layout of the index files
// (lists concatenated in list order, unrotated vectors), coded on the CPU.
void *oracle_load_arrays(uint32_t dim, uint32_t nlist, uint32_t npts, const float *centroids,
                         const uint32_t *list_sizes, const uint32_t *ids, const float *vectors,
                         const float *rotation, uint32_t head_dims) {
  Index *out = nullptr;
  if (oracle::guarded([&] {
        auto x = std::make_unique<Index>();
        x->dim = dim;
        x->nlist = nlist;
        x->npts = npts;
        x->centroids.assign(centroids, centroids + static_cast<size_t>(nlist) * dim);
        x->list_off.assign(nlist + 1, 0);
        for (uint32_t c = 0; c < nlist; ++c) x->list_off[c + 1] = x->list_off[c] + list_sizes[c];
        x->ids.assign(ids, ids + npts);
        x->has_dimc = true;
        x->rotated = rotation != nullptr;
        if (x->rotated) x->rotation.assign(rotation, rotation + static_cast<size_t>(dim) * dim);
        std::vector<float> raw(vectors, vectors + static_cast<size_t>(npts) * dim);
        oracle::code_index(x.get(), raw, head_dims);
        out = x.release();
      }))
    return nullptr;
  return out;
}

// An oracle index coded from rows handed over in pieces, so that a large
// index never needs a second full copy of its unrotated vectors:
// oracle_code_begin takes the index's shape, oracle_code_rows rotates rows
// [row0, row0 + nrows) into place, oracle_code_finish codes them all.
struct PendingIndex {
  std::unique_ptr<Index> x;
  std::vector<float> raw;  // rotated (or copied) rows
  uint32_t head_dims = 0;
};

void *oracle_code_begin(uint32_t dim, uint32_t nlist, uint32_t npts, const float *centroids,
                        const uint32_t *list_sizes, const uint32_t *ids, const float *rotation,
                        uint32_t head_dims) {
  PendingIndex *out = nullptr;
  if (oracle::guarded([&] {
        auto p = std::make_unique<PendingIndex>();
        p->x = std::make_unique<Index>();
        Index *x = p->x.get();
        x->dim = dim;
        x->nlist = nlist;
        x->npts = npts;
        x->centroids.assign(centroids, centroids + static_cast<size_t>(nlist) * dim);
        x->list_off.assign(nlist + 1, 0);
        for (uint32_t c = 0; c < nlist; ++c) x->list_off[c + 1] = x->list_off[c] + list_sizes[c];
        x->ids.assign(ids, ids + npts);
        x->has_dimc = true;
        x->rotated = rotation != nullptr;
        if (x->rotated) x->rotation.assign(rotation, rotation + static_cast<size_t>(dim) * dim);
        p->raw.resize(static_cast<size_t>(npts) * dim);
        p->head_dims = head_dims;
        out = p.release();
      }))
    return nullptr;
  return out;
}

int oracle_code_rows(void *h, uint32_t row0, uint32_t nrows, const float *vectors) {
  auto *p = static_cast<PendingIndex *>(h);
  return oracle::guarded([&] {
    const uint32_t d = p->x->dim;
    if (static_cast<uint64_t>(row0) + nrows > p->x->npts) throw std::invalid_argument("rows out of range");
    float *dst = p->raw.data() + static_cast<size_t>(row0) * d;
    if (p->x->rotated) oracle::rotate_rows(vectors, dst, nrows, d, p->x->rotation.data());
    else std::copy(vectors, vectors + static_cast<size_t>(nrows) * d, dst);
  });
}

void *oracle_code_finish(void *h) {
  std::unique_ptr<PendingIndex> p(static_cast<PendingIndex *>(h));
  Index *out = nullptr;
  if (oracle::guarded([&] {
        oracle::code_index(p->x.get(), p->raw, p->head_dims, true);
        out = p->x.release();
      }))
    return nullptr;
  return out;
}

// An oracle index from already coded arrays (row-major planes in list order),
// so that a large index coded elsewhere can be searched on the CPU. info:
// {dim, nlist, npts, dc, head, rotated}; scale: {lo, inv_step, step, step_sq}.
void *oracle_load_codes(const uint32_t *info, const double *scale, const float *rotation,
                        const uint32_t *list_off, const uint32_t *ids, const uint8_t *hi,
                        const uint8_t *lo, const int64_t *norm, const int64_t *hinorm,
                        const int64_t *headnorm, const uint8_t *chi, const uint8_t *clo,
                        const int64_t *cnorm) {
  auto *x = new Index();
  x->dim = info[0];
  x->nlist = info[1];
  x->npts = info[2];
  x->dc = info[3];
  x->head = info[4];
  x->rotated = info[5] != 0;
  x->has_dimc = x->head != 0 || x->rotated;
  x->lo = static_cast<float>(scale[0]);
  x->inv_step = scale[1];
  x->step = scale[2];
  x->step_sq = scale[3];
  const size_t n = x->npts, L = x->nlist, dc = x->dc;
  if (x->rotated) x->rotation.assign(rotation, rotation + static_cast<size_t>(x->dim) * x->dim);
  x->list_off.assign(list_off, list_off + L + 1);
  x->ids.assign(ids, ids + n);
  x->hi.assign(hi, hi + n * dc);
  x->lo_plane.assign(lo, lo + n * dc);
  x->norm.assign(norm, norm + n);
  x->hinorm.assign(hinorm, hinorm + n);
  if (x->head) x->headnorm.assign(headnorm, headnorm + n);
  x->chi.assign(chi, chi + L * dc);
  x->clo.assign(clo, clo + L * dc);
  x->cnorm.assign(cnorm, cnorm + L);
  x->id_row.assign(n, UINT32_MAX);
  for (uint32_t r = 0; r < n; ++r)
    if (x->ids[r] < n) x->id_row[x->ids[r]] = r;
  return x;
}

int oracle_search(void *h, const float *q, uint32_t nq, uint32_t k, uint32_t nprobe, int ranking,
                  uint32_t survivors, uint32_t *ids, float *dists) {
  return oracle::guarded([&] {
    oracle::search(*static_cast<Index *>(h), q, nq, k, nprobe, ranking, survivors, ids, dists);
  });
}

// u32 info[8] = {dim, nlist, npts, dc, head, rotated, normalized, has_dimc}
// double scale[4] = {lo, inv_step, step, step_sq}
void oracle_info(void *h, uint32_t *info, double *scale) {
  const Index &x = *static_cast<Index *>(h);
  const uint32_t v[8] = {x.dim, x.nlist, x.npts, x.dc, x.head, x.rotated, x.normalized, x.has_dimc};
  std::memcpy(info, v, sizeof(v));
  scale[0] = x.lo;
  scale[1] = x.inv_step;
  scale[2] = x.step;
  scale[3] = x.step_sq;
}

void oracle_list_offsets(void *h, uint32_t *off) {
  const Index &x = *static_cast<Index *>(h);
  std::memcpy(off, x.list_off.data(), x.list_off.size() * sizeof(uint32_t));
}

void oracle_codes(void *h, uint8_t *hi, uint8_t *lo, int64_t *norm, int64_t *hinorm,
                  int64_t *headnorm, uint32_t *ids) {
  const Index &x = *static_cast<Index *>(h);
  std::memcpy(hi, x.hi.data(), x.hi.size());
  std::memcpy(lo, x.lo_plane.data(), x.lo_plane.size());
  std::memcpy(norm, x.norm.data(), x.norm.size() * 8);
  std::memcpy(hinorm, x.hinorm.data(), x.hinorm.size() * 8);
  if (!x.headnorm.empty()) std::memcpy(headnorm, x.headnorm.data(), x.headnorm.size() * 8);
  std::memcpy(ids, x.ids.data(), x.ids.size() * 4);
}

void oracle_centroid_codes(void *h, uint8_t *hi, uint8_t *lo, int64_t *norm) {
  const Index &x = *static_cast<Index *>(h);
  std::memcpy(hi, x.chi.data(), x.chi.size());
  std::memcpy(lo, x.clo.data(), x.clo.size());
  std::memcpy(norm, x.cnorm.data(), x.cnorm.size() * 8);
}

void oracle_rotate(void *h, const float *in, uint32_t nrows, float *out) {
  const Index &x = *static_cast<Index *>(h);
  if (x.rotated) oracle::rotate_rows(in, out, nrows, x.dim, x.rotation.data());
  else std::memcpy(out, in, static_cast<size_t>(nrows) * x.dim * 4);
}

// A rotation of nrows x d rows by an explicit d x d basis (row j = basis j).
void oracle_rotate_with(const float *in, uint32_t nrows, uint32_t d, const float *rot,
                        float *out) {
  oracle::rotate_rows(in, out, nrows, d, rot);
}

void oracle_quantize(void *h, const float *fq, uint32_t nq, uint8_t *qhi, uint8_t *qlo,
                     int64_t *qnorm, int64_t *qhinorm, int64_t *qh0norm) {
  const Index &x = *static_cast<Index *>(h);
  oracle::Quantized q;
  oracle::quantize_queries(x, fq, nq, q);
  std::memcpy(qhi, q.hi.data(), q.hi.size());
  std::memcpy(qlo, q.lo.data(), q.lo.size());
  std::memcpy(qnorm, q.norm.data(), nq * 8);
  std::memcpy(qhinorm, q.hinorm.data(), nq * 8);
  std::memcpy(qh0norm, q.h0norm.data(), nq * 8);
}

int oracle_coarse(void *h, const uint8_t *qhi, const uint8_t *qlo, const int64_t *qnorm,
                  uint32_t nq, uint32_t nprobe, uint32_t *probed) {
  return oracle::guarded([&] {
    const Index &x = *static_cast<Index *>(h);
    oracle::Quantized q;
    q.hi.assign(qhi, qhi + static_cast<size_t>(nq) * x.dc);
    q.lo.assign(qlo, qlo + static_cast<size_t>(nq) * x.dc);
    q.norm.assign(qnorm, qnorm + nq);
    oracle::coarse(x, q, nq, nprobe, probed);
  });
}

// The sq16_l2 / sq16_high_l2 contract (include/katoann/kernels.h:187-205) on
// row-major planes: out[m][n]; plane_dim is the row stride of x (>= dims).
void oracle_sq16_l2(const uint8_t *qhi, const uint8_t *qlo, const uint8_t *xhi, const uint8_t *xlo,
                    const int64_t *qn, const int64_t *xn, double step_sq, uint32_t m, uint32_t n,
                    uint32_t dims, float *out) {
  for (uint32_t i = 0; i < m; ++i)
    for (uint32_t j = 0; j < n; ++j) {
      const int64_t dot = oracle::dot_full(qhi + static_cast<size_t>(i) * dims,
                                           qlo + static_cast<size_t>(i) * dims,
                                           xhi + static_cast<size_t>(j) * dims,
                                           xlo + static_cast<size_t>(j) * dims, dims);
      out[static_cast<size_t>(i) * n + j] = oracle::to_dist(qn[i] + xn[j] - 2 * dot, step_sq);
    }
}

void oracle_sq16_high_l2(const uint8_t *qhi, const uint8_t *xhi, const int64_t *qn,
                         const int64_t *xn, double step_sq, uint32_t m, uint32_t n, uint32_t dims,
                         uint32_t plane_dim, float *out) {
  for (uint32_t i = 0; i < m; ++i)
    for (uint32_t j = 0; j < n; ++j) {
      const int64_t dot = oracle::dot_high(qhi + static_cast<size_t>(i) * dims,
                                           xhi + static_cast<size_t>(j) * plane_dim, dims);
      out[static_cast<size_t>(i) * n + j] = oracle::to_dist(qn[i] + xn[j] - 2 * dot, step_sq);
    }
}

float oracle_to_dist(int64_t l2, double step_sq) { return oracle::to_dist(l2, step_sq); }

void oracle_set_threads(int t) {
  if (t > 0) omp_set_num_threads(t);
}
int oracle_max_threads() { return omp_get_max_threads(); }

}  // extern "C"
