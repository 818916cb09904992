// katoann::ProbeModel: the learned per-query probe budget (host side).
// Labels come from searches of the index (Index::search at every ladder
// value and the exact Ranking::kFull search); features, training and
// inference run on the device through libkatoann_gpu.so.
#include "katoann/probe.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "katoann_gpu.h"

namespace katoann {

namespace {

constexpr uint32_t kF = KATO_PROBE_FEATURES;
constexpr uint32_t kH = KATO_PROBE_HIDDEN;
constexpr uint32_t kMagic = 0x4252504Bu;  // "KPRB"
constexpr uint32_t kVersion = 1;

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

struct Dev {
  void *p = nullptr;
  Dev() = default;
  explicit Dev(size_t bytes) { cuda_check(cudaMalloc(&p, bytes ? bytes : 16), "cudaMalloc"); }
  Dev(const Dev &) = delete;
  Dev &operator=(const Dev &) = delete;
  ~Dev() {
    if (p) cudaFree(p);
  }
  template <class T>
  T *as() const {
    return static_cast<T *>(p);
  }
};

uint16_t to_bf16(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return static_cast<uint16_t>(u >> 16);
}

void check_ladder(const std::vector<uint32_t> &ladder) {
  if (ladder.size() < 2 || ladder.size() > KATO_PROBE_MAX_CLASSES)
    throw std::invalid_argument("probe model: the ladder needs 2 to 32 nprobe values");
  for (size_t i = 0; i < ladder.size(); ++i)
    if (ladder[i] == 0 || ladder[i] > 4096 || (i && ladder[i] <= ladder[i - 1]))
      throw std::invalid_argument("probe model: ladder values must ascend within 1..4096");
}

}  // namespace

std::vector<uint32_t> probe_feature_ranks(uint32_t depth) {
  if (depth == 0) throw std::invalid_argument("probe features: depth must be positive");
  std::vector<uint32_t> r(kF);
  if (depth <= kF) {
    for (uint32_t j = 0; j < kF; ++j) r[j] = static_cast<uint32_t>(uint64_t(j) * (depth - 1) / (kF - 1));
    return r;
  }
  for (uint32_t j = 0; j < 16; ++j) r[j] = j;
  const double top = depth - 1, ratio = top / 16.0;
  for (uint32_t j = 16; j < kF; ++j) {
    const double v = 16.0 * std::pow(ratio, (j - 16) / 47.0);
    r[j] = std::min<uint32_t>(static_cast<uint32_t>(std::lround(v)), depth - 1);
  }
  r[kF - 1] = depth - 1;
  for (uint32_t j = 1; j < kF; ++j) r[j] = std::max(r[j], r[j - 1]);
  return r;
}

struct ProbeModel::Impl {
  uint32_t C = 0, depth = 0;
  std::vector<uint32_t> ladder, rank;
  std::vector<float> shift, scale, b1, b2, b3;
  std::vector<uint16_t> w1, w2, w3;  // bf16, input-major
  std::vector<uint8_t> labels;
  std::vector<float> loss;
  // device copies, made on first use
  std::mutex mu;
  std::unique_ptr<Dev> dev;
  katoann_gpu_probe_model view{};

  void check() const {
    check_ladder(ladder);
    if (C != ladder.size() || rank.size() != kF || shift.size() != kF || scale.size() != kF ||
        w1.size() != size_t(kF) * kH || b1.size() != kH || w2.size() != size_t(kH) * kH ||
        b2.size() != kH || w3.size() != size_t(kH) * C || b3.size() != C || depth == 0 ||
        depth > 4096 || rank[0] != 0 || rank[kF - 1] + 1 != depth)
      throw std::invalid_argument("probe model: inconsistent arrays");
  }

  const katoann_gpu_probe_model &device() {
    std::lock_guard<std::mutex> lock(mu);
    if (dev) return view;
    size_t o = 0;
    auto take = [&](size_t bytes) {
      const size_t at = o;
      o += (bytes + 255) / 256 * 256;
      return at;
    };
    const size_t o_rank = take(kF * 4), o_shift = take(kF * 4), o_scale = take(kF * 4),
                 o_w1 = take(w1.size() * 2), o_b1 = take(kH * 4), o_w2 = take(w2.size() * 2),
                 o_b2 = take(kH * 4), o_w3 = take(w3.size() * 2), o_b3 = take(C * 4),
                 o_ladder = take(C * 4);
    std::vector<unsigned char> blob(o, 0);
    auto put = [&](size_t at, const void *src, size_t bytes) { std::memcpy(blob.data() + at, src, bytes); };
    put(o_rank, rank.data(), kF * 4);
    put(o_shift, shift.data(), kF * 4);
    put(o_scale, scale.data(), kF * 4);
    put(o_w1, w1.data(), w1.size() * 2);
    put(o_b1, b1.data(), kH * 4);
    put(o_w2, w2.data(), w2.size() * 2);
    put(o_b2, b2.data(), kH * 4);
    put(o_w3, w3.data(), w3.size() * 2);
    put(o_b3, b3.data(), C * 4);
    put(o_ladder, ladder.data(), C * 4);
    auto d = std::make_unique<Dev>(o);
    cuda_check(cudaMemcpy(d->p, blob.data(), o, cudaMemcpyHostToDevice), "upload probe model");
    unsigned char *base = d->as<unsigned char>();
    view = katoann_gpu_probe_model{};
    view.nclass = C;
    view.depth = depth;
    view.d_rank = reinterpret_cast<const uint32_t *>(base + o_rank);
    view.d_shift = reinterpret_cast<const float *>(base + o_shift);
    view.d_scale = reinterpret_cast<const float *>(base + o_scale);
    view.d_w1 = reinterpret_cast<const uint16_t *>(base + o_w1);
    view.d_b1 = reinterpret_cast<const float *>(base + o_b1);
    view.d_w2 = reinterpret_cast<const uint16_t *>(base + o_w2);
    view.d_b2 = reinterpret_cast<const float *>(base + o_b2);
    view.d_w3 = reinterpret_cast<const uint16_t *>(base + o_w3);
    view.d_b3 = reinterpret_cast<const float *>(base + o_b3);
    view.d_ladder = reinterpret_cast<const uint32_t *>(base + o_ladder);
    dev = std::move(d);
    return view;
  }
};

ProbeModel::ProbeModel() = default;
ProbeModel::~ProbeModel() = default;
ProbeModel::ProbeModel(ProbeModel &&) noexcept = default;
ProbeModel &ProbeModel::operator=(ProbeModel &&) noexcept = default;

namespace {
const ProbeModel::Impl &need(const std::shared_ptr<ProbeModel::Impl> &m) {
  if (!m) throw std::logic_error("empty probe model");
  return *m;
}
}  // namespace

uint32_t ProbeModel::classes() const { return need(m_).C; }
uint32_t ProbeModel::depth() const { return need(m_).depth; }
const std::vector<uint32_t> &ProbeModel::ladder() const { return need(m_).ladder; }
const std::vector<uint32_t> &ProbeModel::feature_ranks() const { return need(m_).rank; }
const std::vector<uint8_t> &ProbeModel::labels() const { return need(m_).labels; }
const std::vector<float> &ProbeModel::loss() const { return need(m_).loss; }

void ProbeModel::weights(float *shift, float *scale, uint16_t *w1, float *b1, uint16_t *w2,
                         float *b2, uint16_t *w3, float *b3) const {
  const Impl &m = need(m_);
  auto cp = [](auto *dst, const auto &v) {
    if (dst) std::copy(v.begin(), v.end(), dst);
  };
  cp(shift, m.shift);
  cp(scale, m.scale);
  cp(w1, m.w1);
  cp(b1, m.b1);
  cp(w2, m.w2);
  cp(b2, m.b2);
  cp(w3, m.w3);
  cp(b3, m.b3);
}

void ProbeModel::device_model(float threshold, void *out) const {
  if (!m_) throw std::logic_error("empty probe model");
  katoann_gpu_probe_model v = m_->device();
  v.threshold = threshold;
  *static_cast<katoann_gpu_probe_model *>(out) = v;
}

void ProbeModel::features(const Index &index, const float *queries, uint32_t nq, uint32_t depth,
                          float *z) {
  if (nq == 0) return;
  if (index.nlist() == 0) throw std::logic_error("features before load");
  if (depth == 0 || depth > index.nlist() || depth > 4096)
    throw std::invalid_argument("probe features: depth must be 1 to min(nlist, 4096)");
  const auto *view = static_cast<const katoann_gpu_index *>(index.device_view());
  const std::vector<uint32_t> rank = probe_feature_ranks(depth);
  const uint32_t mb = std::min<uint32_t>(nq, 4096);
  const size_t wsb = katoann_gpu_search_workspace(view, mb, 1, depth, KATO_RANK_FULL, 1);
  if (wsb == 0) gpu_check(KATO_EINVAL);
  const float *src = queries;  // normalized by the caller, as for Index::search
  Dev ws(wsb), dr(kF * 4), dq(static_cast<size_t>(mb) * index.dim() * 4),
      dz(static_cast<size_t>(mb) * kF * 4);
  cuda_check(cudaMemcpy(dr.p, rank.data(), kF * 4, cudaMemcpyHostToDevice), "upload ranks");
  for (uint32_t q0 = 0; q0 < nq; q0 += mb) {
    const uint32_t b = std::min(mb, nq - q0);
    cuda_check(cudaMemcpy(dq.p, src + static_cast<size_t>(q0) * index.dim(),
                          static_cast<size_t>(b) * index.dim() * 4, cudaMemcpyHostToDevice),
               "copy queries");
    gpu_check(katoann_gpu_probe_features(view, dq.as<float>(), b, dr.as<uint32_t>(), depth, mb,
                                         ws.p, wsb, dz.as<float>(), nullptr));
    cuda_check(cudaMemcpy(z + static_cast<size_t>(q0) * kF, dz.p, static_cast<size_t>(b) * kF * 4,
                          cudaMemcpyDeviceToHost),
               "copy features");
  }
}

ProbeModel ProbeModel::fit(const float *z, const uint8_t *labels, uint32_t n,
                           const ProbeTrainOptions &opt) {
  check_ladder(opt.ladder);
  if (n == 0) throw std::invalid_argument("probe model: no training rows");
  const uint32_t C = static_cast<uint32_t>(opt.ladder.size());
  for (uint32_t i = 0; i < n; ++i)
    if (labels[i] >= C) throw std::invalid_argument("probe model: a label is not a ladder class");
  auto m = std::make_shared<Impl>();
  m->C = C;
  m->depth = opt.depth;
  m->ladder = opt.ladder;
  m->rank = probe_feature_ranks(opt.depth);
  m->shift.resize(kF);
  m->scale.resize(kF);
  std::vector<float> w1(size_t(kF) * kH), w2(size_t(kH) * kH), w3(size_t(kH) * C);
  m->b1.resize(kH);
  m->b2.resize(kH);
  m->b3.resize(C);
  m->loss.resize(opt.epochs);
  Dev dz(static_cast<size_t>(n) * kF * 4), dl(n);
  cuda_check(cudaMemcpy(dz.p, z, static_cast<size_t>(n) * kF * 4, cudaMemcpyHostToDevice), "copy features");
  cuda_check(cudaMemcpy(dl.p, labels, n, cudaMemcpyHostToDevice), "copy labels");
  katoann_gpu_probe_train_options o{opt.epochs, opt.batch, opt.lr, opt.weight_decay, opt.seed};
  gpu_check(katoann_gpu_probe_train(dz.as<float>(), dl.as<uint8_t>(), n, C, &o, m->shift.data(),
                                    m->scale.data(), w1.data(), m->b1.data(), w2.data(),
                                    m->b2.data(), w3.data(), m->b3.data(), m->loss.data()));
  auto half = [](const std::vector<float> &w) {
    std::vector<uint16_t> h(w.size());
    for (size_t i = 0; i < w.size(); ++i) h[i] = to_bf16(w[i]);
    return h;
  };
  m->w1 = half(w1);
  m->w2 = half(w2);
  m->w3 = half(w3);
  m->labels.assign(labels, labels + n);
  m->check();
  ProbeModel out;
  out.m_ = std::move(m);
  return out;
}

ProbeModel ProbeModel::train(const Index &index, const float *queries, uint32_t nq,
                             const ProbeTrainOptions &opt) {
  check_ladder(opt.ladder);
  const uint32_t L = index.nlist();
  if (L == 0) throw std::logic_error("training before load");
  if (nq == 0) throw std::invalid_argument("probe model: no training queries");
  if (opt.ladder.back() > L) throw std::invalid_argument("probe model: ladder values must be <= nlist");
  if (opt.depth == 0 || opt.depth > L || opt.depth > 4096)
    throw std::invalid_argument("probe model: depth must be 1 to min(nlist, 4096)");
  const uint32_t k = opt.k;
  if (k == 0) throw std::invalid_argument("probe model: k must be positive");
  const uint32_t ref_p =
      opt.label_nprobe ? std::min(opt.label_nprobe, L) : std::min(L, 2 * opt.ladder.back());
  // the exact top-k within the ref_p nearest lists
  std::vector<uint32_t> ref(static_cast<size_t>(nq) * k), ids(static_cast<size_t>(nq) * k);
  std::vector<float> dd(static_cast<size_t>(nq) * k);
  SearchParams sp;
  sp.k = k;
  sp.nprobe = ref_p;
  sp.ranking = opt.label_ranking;
  sp.survivors = std::max(opt.label_survivors, k);
  index.search(queries, nq, sp, ref.data(), dd.data());
  // per query: how much of it each ladder value's search recovers
  const uint32_t C = static_cast<uint32_t>(opt.ladder.size());
  std::vector<uint8_t> hits(static_cast<size_t>(nq) * C);
  sp.ranking = opt.ranking;
  sp.survivors = opt.survivors;
  for (uint32_t c = 0; c < C; ++c) {
    sp.nprobe = opt.ladder[c];
    index.search(queries, nq, sp, ids.data(), dd.data());
    for (uint32_t q = 0; q < nq; ++q) {
      const uint32_t *a = ref.data() + static_cast<size_t>(q) * k;
      const uint32_t *b = ids.data() + static_cast<size_t>(q) * k;
      uint32_t h = 0;
      for (uint32_t i = 0; i < k; ++i)
        if (a[i] != 0xFFFFFFFFu && std::find(b, b + k, a[i]) != b + k) ++h;
      hits[static_cast<size_t>(q) * C + c] = static_cast<uint8_t>(std::min(h, 255u));
    }
  }
  std::vector<uint8_t> labels(nq);
  for (uint32_t q = 0; q < nq; ++q) {
    const uint8_t *h = hits.data() + static_cast<size_t>(q) * C;
    const uint8_t best = *std::max_element(h, h + C);
    labels[q] = static_cast<uint8_t>(std::find(h, h + C, best) - h);
  }
  std::vector<float> z(static_cast<size_t>(nq) * kF);
  features(index, queries, nq, opt.depth, z.data());
  return fit(z.data(), labels.data(), nq, opt);
}

void ProbeModel::predict(const float *z, uint32_t n, float threshold, uint32_t cap, float *probs,
                         uint32_t *nprobe) const {
  if (!m_) throw std::logic_error("empty probe model");
  if (n == 0) return;
  if (cap == 0) throw std::invalid_argument("probe model: the cap must be positive");
  katoann_gpu_probe_model v = m_->device();
  v.threshold = threshold;
  Dev dz(static_cast<size_t>(n) * kF * 4), dp(static_cast<size_t>(n) * m_->C * 4), dn(size_t(n) * 4);
  cuda_check(cudaMemcpy(dz.p, z, static_cast<size_t>(n) * kF * 4, cudaMemcpyHostToDevice), "copy features");
  gpu_check(katoann_gpu_probe_predict(&v, dz.as<float>(), n, cap, dp.as<float>(),
                                      dn.as<uint32_t>(), nullptr));
  if (probs)
    cuda_check(cudaMemcpy(probs, dp.p, static_cast<size_t>(n) * m_->C * 4, cudaMemcpyDeviceToHost),
               "copy probabilities");
  if (nprobe)
    cuda_check(cudaMemcpy(nprobe, dn.p, static_cast<size_t>(n) * 4, cudaMemcpyDeviceToHost),
               "copy budgets");
}

// File: magic, version, classes, depth, then ladder, ranks, shift, scale, w1,
// b1, w2, b2, w3, b3 (little-endian; weights as bf16).
void ProbeModel::save(const std::string &path) const {
  const Impl &m = need(m_);
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f) throw std::runtime_error("cannot open " + path + " for writing");
  auto w = [&](const void *p, size_t bytes) { f.write(static_cast<const char *>(p), static_cast<std::streamsize>(bytes)); };
  const uint32_t head[4] = {kMagic, kVersion, m.C, m.depth};
  w(head, sizeof head);
  w(m.ladder.data(), m.C * 4);
  w(m.rank.data(), kF * 4);
  w(m.shift.data(), kF * 4);
  w(m.scale.data(), kF * 4);
  w(m.w1.data(), m.w1.size() * 2);
  w(m.b1.data(), kH * 4);
  w(m.w2.data(), m.w2.size() * 2);
  w(m.b2.data(), kH * 4);
  w(m.w3.data(), m.w3.size() * 2);
  w(m.b3.data(), m.C * 4);
  if (!f) throw std::runtime_error("write failed: " + path);
}

ProbeModel ProbeModel::load(const std::string &path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + path);
  auto r = [&](void *p, size_t bytes) {
    f.read(static_cast<char *>(p), static_cast<std::streamsize>(bytes));
    if (!f) throw std::runtime_error("truncated probe model: " + path);
  };
  uint32_t head[4];
  r(head, sizeof head);
  if (head[0] != kMagic || head[1] != kVersion) throw std::runtime_error("bad header: " + path);
  if (head[2] < 2 || head[2] > KATO_PROBE_MAX_CLASSES || head[3] == 0 || head[3] > 4096)
    throw std::runtime_error("bad header: " + path);
  auto m = std::make_shared<Impl>();
  m->C = head[2];
  m->depth = head[3];
  m->ladder.resize(m->C);
  m->rank.resize(kF);
  m->shift.resize(kF);
  m->scale.resize(kF);
  m->w1.resize(size_t(kF) * kH);
  m->b1.resize(kH);
  m->w2.resize(size_t(kH) * kH);
  m->b2.resize(kH);
  m->w3.resize(size_t(kH) * m->C);
  m->b3.resize(m->C);
  r(m->ladder.data(), m->C * 4);
  r(m->rank.data(), kF * 4);
  r(m->shift.data(), kF * 4);
  r(m->scale.data(), kF * 4);
  r(m->w1.data(), m->w1.size() * 2);
  r(m->b1.data(), kH * 4);
  r(m->w2.data(), m->w2.size() * 2);
  r(m->b2.data(), kH * 4);
  r(m->w3.data(), m->w3.size() * 2);
  r(m->b3.data(), m->C * 4);
  try {
    m->check();
  } catch (const std::invalid_argument &e) {
    throw std::runtime_error(std::string("bad probe model ") + path + ": " + e.what());
  }
  ProbeModel out;
  out.m_ = std::move(m);
  return out;
}

}  // namespace katoann
