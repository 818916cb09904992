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
// The reference's quantization (src/index.cpp:669-670, :735-736, :925-926):
// (double(x) - lo) * inv_step in double, rounded half away from zero
// (lround), clamped to [0, 65535].
__device__ __forceinline__ uint32_t quantize_double(float x, float lo, double inv_step) {
  const double t = __dmul_rn(__dsub_rn(static_cast<double>(x), static_cast<double>(lo)), inv_step);
  long long r = llround(t);
  r = r < 0 ? 0 : (r > 65535 ? 65535 : r);
  return static_cast<uint32_t>(r);
}

// inv_step as ih + il (two floats, within 2^-48 of it), made once per thread.
struct QuantScale {
  float lo, ih, il;
  double inv_step;
};

__device__ __forceinline__ QuantScale quant_scale(float lo, double inv_step) {
  const float ih = __double2float_rn(inv_step);
  return QuantScale{lo, ih, __double2float_rn(__dsub_rn(inv_step, static_cast<double>(ih))), inv_step};
}

// quantize_double's value from single-precision arithmetic (GB300's FP64 rate
// is a small fraction of its FP32 rate). Knuth's TwoSum gives x - lo exactly
// as s + e; Dekker's product with an FMA gives s * ih exactly as p + pe; with
// the small terms added, p + q is within 2^-45 |t| of the exact product
// t = (x - lo) * inv_step, and the reference's double result within 2^-52 |t|.
// For |t| < 2^17 both are within 2^-27 of t, so where the fraction of p + q
// lies more than 2^-20 from one half they round to the same integer; nearer
// (about one value in 2^19), or for values that are not finite, the double
// arithmetic runs.
__device__ __forceinline__ uint32_t quantize1(float x, const QuantScale &k) {
  const float nlo = -k.lo;
  const float s = __fadd_rn(x, nlo);
  const float bv = __fadd_rn(s, -x), av = __fadd_rn(s, -bv);
  const float e = __fadd_rn(__fadd_rn(x, -av), __fadd_rn(nlo, -bv));
  const float p = __fmul_rn(s, k.ih);
  const float pe = __fmaf_rn(s, k.ih, -p);
  const float q = __fadd_rn(pe, __fmaf_rn(s, k.il, __fmul_rn(e, k.ih)));
  if (!(fabsf(p) < 131072.0f)) {  // far outside the range (or not finite)
    if (p >= 131072.0f) return 65535u;
    if (p <= -131072.0f) return 0u;
    return quantize_double(x, k.lo, k.inv_step);
  }
  const float fp = floorf(p);
  const float r = __fadd_rn(__fadd_rn(p, -fp), q);  // the fraction, near [0, 1)
  if (!(fabsf(__fadd_rn(r, -0.5f)) > 0x1p-20f)) return quantize_double(x, k.lo, k.inv_step);
  const float n = __fadd_rn(fp, r >= 0.5f ? 1.0f : 0.0f);
  return static_cast<uint32_t>(fminf(fmaxf(n, 0.0f), 65535.0f));
}

// Packed unsigned byte dot product of two 32-bit words (4 lanes).
__device__ __forceinline__ uint32_t dp4(uint32_t a, uint32_t b, uint32_t c) {
  return __dp4a(a, b, c);
}

}  // namespace kato
