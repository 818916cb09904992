// Learned per-query probe budget for katoann::Index (no counterpart in the
// reference, whose nprobe is one value per batch: SearchParams::nprobe,
// include/katoann/index.h:53).
//
// A ProbeModel is a 64 -> 256 -> 256 -> C MLP (bf16 weights, fp32
// accumulation) over 64 features of a query's sorted coarse distances. It
// gives a distribution over a ladder of nprobe values; a search with
// SearchParams::budget set probes, per query, the smallest ladder value whose
// cumulative probability reaches SearchParams::budget_threshold (at most
// SearchParams::nprobe). A query's result is then exactly the fixed-nprobe
// result at its own nprobe, which the plain search (and the reference)
// reproduce.
//
// ProbeModel::train labels training queries by searching the index itself:
// a query's label is the smallest ladder value whose fixed-nprobe search
// (the ranking and survivors the budget is for) recovers as much of the
// query's exact top-k as any ladder value does. The exact top-k comes from
// the exact-distance search (Ranking::kFull) at label_nprobe lists, or, to
// label many queries faster, from a search with label_ranking and
// label_survivors (its refinement gives exact distances of the survivors, so
// it equals the exact top-k whenever those rank within the survivors).
// Training runs on the device (softmax cross-entropy, Adam).
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "katoann/index.h"

namespace katoann {

struct ProbeTrainOptions {
  // nprobe values the model chooses from, ascending, each <= min(nlist, 4096)
  std::vector<uint32_t> ladder = {8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512};
  uint32_t depth = 256;          // coarse ranks the features read (<= nlist, <= 4096)
  uint32_t k = 10;               // the exact top-k the labels recover
  uint32_t label_nprobe = 0;     // lists of the exact search; 0: min(nlist, 2 x the top of the ladder)
  Ranking label_ranking = Ranking::kFull;  // the search that gives the exact top-k
  uint32_t label_survivors = 0;  // its survivors (0: k)
  Ranking ranking = Ranking::kPrefix;  // the search the budget is for
  uint32_t survivors = 64;
  uint32_t epochs = 24;
  uint32_t batch = 1024;
  float lr = 1e-3f;
  float weight_decay = 1e-4f;
  uint64_t seed = 0;
};

class ProbeModel {
 public:
  ProbeModel();
  ~ProbeModel();
  ProbeModel(ProbeModel &&) noexcept;
  ProbeModel &operator=(ProbeModel &&) noexcept;
  ProbeModel(const ProbeModel &) = delete;
  ProbeModel &operator=(const ProbeModel &) = delete;

  // Labels nq training queries (host, nq x dim) by searches of `index` and
  // trains the model on the device.
  static ProbeModel train(const Index &index, const float *queries, uint32_t nq,
                          const ProbeTrainOptions &opt = {});
  // Trains on given raw features (n x 64, from features()) and labels (class
  // indices into opt.ladder); opt.depth must be the depth the features used.
  static ProbeModel fit(const float *z, const uint8_t *labels, uint32_t n,
                        const ProbeTrainOptions &opt);

  void save(const std::string &path) const;
  static ProbeModel load(const std::string &path);

  // The 64 raw features of nq queries (host in, host nq x 64 out) at `depth`.
  static void features(const Index &index, const float *queries, uint32_t nq, uint32_t depth,
                       float *z);
  // Class probabilities (n x classes, may be null) and budgets capped at
  // `cap` (n, may be null) of n raw feature rows (host).
  void predict(const float *z, uint32_t n, float threshold, uint32_t cap, float *probs,
               uint32_t *nprobe) const;

  bool empty() const { return !m_; }
  uint32_t classes() const;
  uint32_t depth() const;
  const std::vector<uint32_t> &ladder() const;
  const std::vector<uint32_t> &feature_ranks() const;
  // Training record: the labels of the training queries (class indices) and
  // the mean loss of every epoch (empty for a loaded model).
  const std::vector<uint8_t> &labels() const;
  const std::vector<float> &loss() const;

  // The device model (a katoann_gpu_probe_model) with this threshold into *out.
  void device_model(float threshold, void *out) const;
  // The weights as the device uses them (any pointer may be null): shift,
  // scale (64), w1 (64 x 256 bf16, input-major), b1 (256), w2 (256 x 256),
  // b2 (256), w3 (256 x classes), b3 (classes).
  void weights(float *shift, float *scale, uint16_t *w1, float *b1, uint16_t *w2, float *b2,
               uint16_t *w3, float *b3) const;

  struct Impl;

 private:
  std::shared_ptr<Impl> m_;
};

// The 64 feature ranks of a depth: ranks 0..15, then 48 ranks spaced
// geometrically up to depth - 1 (all 64 evenly spread when depth <= 64).
std::vector<uint32_t> probe_feature_ranks(uint32_t depth);

}  // namespace katoann
