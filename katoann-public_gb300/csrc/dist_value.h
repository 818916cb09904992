// Exact distance value of the reference, float(double(l2) * step_sq), without
// double-precision arithmetic (GB300's FP64 rate is a small fraction of its
// integer rate, and every candidate distance goes through this conversion).
//
// The reference converts an exact int64 squared L2 between 16-bit codes to a
// double (exact: l2 < 2^53), multiplies by step_sq in double (one rounding to
// 53 bits, nearest-even) and narrows to float (a second rounding to 24 bits,
// nearest-even) (src/kernels.cpp:166-168, :208-210). With step_sq = m * 2^e
// (m a 53-bit integer), l2 * step_sq = (l2 * m) * 2^e exactly, so both
// roundings can be replayed on the 128-bit integer product l2 * m. This is
// IEEE 754 round-to-nearest-even done by hand, from its definition.
//
// Shared by the CUDA kernels and by host code (tests call the host build).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define KATO_HD __host__ __device__ __forceinline__
#else
#define KATO_HD inline
#endif

namespace kato {

struct DistScale {
  uint64_t m;      // 53-bit integer mantissa of step_sq
  int32_t e;       // step_sq = m * 2^e
  int32_t pad;
  double step_sq;  // for the out-of-range fallback
};

inline DistScale make_dist_scale(double step_sq) {
  DistScale s{};
  int ex = 0;
  const double f = std::frexp(step_sq, &ex);  // step_sq = f * 2^ex, f in [0.5, 1)
  s.m = static_cast<uint64_t>(std::ldexp(f, 53));
  s.e = ex - 53;
  s.step_sq = step_sq;
  return s;
}

KATO_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return static_cast<uint64_t>((static_cast<unsigned __int128>(a) * b) >> 64);
#endif
}

KATO_HD int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll(static_cast<long long>(x));
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

KATO_HD float bits_to_float(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float f;
  std::memcpy(&f, &b, 4);
  return f;
#endif
}

// The double-precision path, for the rare values outside the fast path's
// range. Kept out of line on the GPU so that callers never evaluate it
// speculatively (GB300's FP64 pipe is narrow).
#if defined(__CUDACC__)
static __host__ __device__ __noinline__ float dist_value_slow(int64_t l2, DistScale s) {
#else
static inline float dist_value_slow(int64_t l2, DistScale s) {
#endif
  return static_cast<float>(static_cast<double>(l2) * s.step_sq);
}

// float(double(l2) * step_sq), bit for bit.
KATO_HD float dist_value(int64_t l2, const DistScale &s) {
  if (l2 <= 0) return l2 == 0 ? 0.0f : dist_value_slow(l2, s);
  const uint64_t a = static_cast<uint64_t>(l2);
  const uint64_t lo = a * s.m, hi = mulhi64(a, s.m);
  const int nb = hi ? 128 - clz64(hi) : 64 - clz64(lo);  // bits of l2 * m
  const int sh = nb - 53;
  uint64_t q;
  int e = s.e;
  if (sh <= 0) {  // the product fits in 53 bits: the double is exact
    q = lo << (-sh);
    e += sh;
  } else if (sh < 64) {  // round to 53 bits, nearest-even
    q = (hi << (64 - sh)) | (lo >> sh);
    const uint64_t rem = lo & ((1ull << sh) - 1);
    const uint64_t half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (q & 1))) {
      ++q;
      if (q == (1ull << 53)) {
        q >>= 1;
        ++e;
      }
    }
    e += sh;
  } else {
    return dist_value_slow(l2, s);
  }
  // q in [2^52, 2^53): the double is q * 2^e. Round to 24 bits, nearest-even.
  uint64_t q24 = q >> 29;
  const uint64_t rem2 = q & ((1ull << 29) - 1);
  if (rem2 > (1ull << 28) || (rem2 == (1ull << 28) && (q24 & 1))) {
    ++q24;
    if (q24 == (1ull << 24)) {
      q24 >>= 1;
      ++e;
    }
  }
  const int biased = e + 29 + 23 + 127;  // value = q24 * 2^(e+29) = 1.f * 2^(e+29+23)
  if (biased < 1 || biased > 254) return dist_value_slow(l2, s);
  return bits_to_float((static_cast<uint32_t>(biased) << 23) |
                       static_cast<uint32_t>(q24 & 0x7FFFFFu));
}

}  // namespace kato
