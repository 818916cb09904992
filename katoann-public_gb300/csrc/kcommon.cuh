// Shared pieces of the sm_103a kernels: status handling and small helpers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <algorithm>
#include <string>

#include "dist_value.h"
#include "katoann_gpu.h"

namespace kato {

void set_error(const std::string &msg);
int cuda_status(cudaError_t e, const char *what);

#define KATO_CUDA(call)                                        \
  do {                                                         \
    cudaError_t e_ = (call);                                   \
    if (e_ != cudaSuccess) return ::kato::cuda_status(e_, #call); \
  } while (0)

#define KATO_LAUNCHED(what)                                            \
  do {                                                                 \
    cudaError_t e_ = cudaGetLastError();                               \
    if (e_ != cudaSuccess) return ::kato::cuda_status(e_, what);       \
  } while (0)

// One-time device settings, kept per device and safe from any thread (a
// server's dispatcher and the callers' threads may make first calls at once,
// and one process may drive several GPUs).
// The SM count of the current device.
int current_sms(int *sms);
// Raises `kernel`'s dynamic shared-memory limit on the current device to at
// least `bytes` (once per device and kernel).
int smem_limit(const void *kernel, int bytes, const char *what);

inline int invalid(const std::string &msg) {
  set_error(msg);
  return KATO_EINVAL;
}

inline cudaStream_t as_stream(katoann_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

__host__ __device__ __forceinline__ uint32_t div_up(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

// Order-preserving map of a float onto uint32 (for min/max with atomics).
__device__ __forceinline__ uint32_t float_order_key(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__host__ __device__ __forceinline__ float float_from_order_key(uint32_t k) {
  const uint32_t b = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
  return bits_to_float(b);
}

// Quantization of one value (src/index.cpp:669-670): lround in double of
// (x - lo) * inv_step, clamped to [0, 65535].
__device__ __forceinline__ uint32_t quantize1(float x, float lo, double inv_step) {
  const double t = __dmul_rn(__dsub_rn(static_cast<double>(x), static_cast<double>(lo)), inv_step);
  long long r = llround(t);
  r = r < 0 ? 0 : (r > 65535 ? 65535 : r);
  return static_cast<uint32_t>(r);
}

// Packed unsigned byte dot product of two 32-bit words (4 lanes).
__device__ __forceinline__ uint32_t dp4(uint32_t a, uint32_t b, uint32_t c) {
  return __dp4a(a, b, c);
}

}  // namespace kato
