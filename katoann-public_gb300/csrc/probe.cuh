// Learned per-query probe budget: device functions shared by the search
// pipeline and the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "katoann_gpu.h"

namespace kato {

// Per-query nprobe of one search: from the caller (nprobe_in), from the
// model, or none (every query probes the search's nprobe).
struct Budget {
  const uint32_t *nprobe_in = nullptr;           // device, one per query
  const katoann_gpu_probe_model *model = nullptr;
  uint32_t *nprobe_out = nullptr;                // device, one per query
  uint32_t cap = 0;                              // the search's nprobe
  bool active() const { return nprobe_in || model; }
};

// The 64 raw features of B queries from their coarse distance rows (cd,
// B x L) and their P nearest lists in order (probed, B x P) into z (B x 64).
int probe_features(const float *cd, uint32_t L, const uint32_t *probed, uint32_t P,
                   const uint32_t *rank, uint32_t B, float *z, cudaStream_t st);

// The MLP on B feature rows: class probabilities (may be null) and budgets
// capped at `cap` (may be null).
int probe_budget(const katoann_gpu_probe_model &m, const float *z, uint32_t B, uint32_t cap,
                 float *probs, uint32_t *nprobe, cudaStream_t st);

// Caller-given budgets, clamped to [1, cap] (in == null: every one is cap).
int clamp_budget(const uint32_t *in, uint32_t B, uint32_t cap, uint32_t *out, cudaStream_t st);

// Host checks of a model (sizes, pointers).
int check_probe_model(const katoann_gpu_probe_model &m);

}  // namespace kato
