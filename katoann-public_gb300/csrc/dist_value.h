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
  int32_t single;  // the single-precision path of the device applies
  double step_sq;  // for the out-of-range fallback
  // step_sq = s1 + s2 + r with s1, s2 floats and |r| <= 2^-48 step_sq;
  // a1, a2 = s1, s2 scaled by 2^23 (exact)
  float s1, s2, a1, a2;
};

inline DistScale make_dist_scale(double step_sq) {
  DistScale s{};
  int ex = 0;
  const double f = std::frexp(step_sq, &ex);  // step_sq = f * 2^ex, f in [0.5, 1)
  s.m = static_cast<uint64_t>(std::ldexp(f, 53));
  s.e = ex - 53;
  s.step_sq = step_sq;
  // the split needs normal floats with room below them: step_sq in [2^-80, 2^80]
  s.single = step_sq >= std::ldexp(1.0, -80) && step_sq <= std::ldexp(1.0, 80);
  if (s.single) {
    s.s1 = static_cast<float>(step_sq);
    s.s2 = static_cast<float>(step_sq - static_cast<double>(s.s1));  // the difference is exact
    s.a1 = std::ldexp(s.s1, 23);
    s.a2 = std::ldexp(s.s2, 23);
  }
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
static __host__ __device__ __noinline__ float dist_value_slow(int64_t l2, double step_sq) {
#else
static inline float dist_value_slow(int64_t l2, double step_sq) {
#endif
  return static_cast<float>(static_cast<double>(l2) * step_sq);
}

// float(double(l2) * step_sq), bit for bit, from the 128-bit integer product
// l2 * m (step_sq = m * 2^e0). Out of line on the GPU, where the
// single-precision path below settles all but about 2^-14 of the values.
#if defined(__CUDACC__)
static __host__ __device__ __noinline__ float dist_value_exact(int64_t l2, uint64_t m, int e0,
                                                               double step_sq) {
#else
static inline float dist_value_exact(int64_t l2, uint64_t m, int e0, double step_sq) {
#endif
  if (l2 <= 0) return l2 == 0 ? 0.0f : dist_value_slow(l2, step_sq);
  const uint64_t a = static_cast<uint64_t>(l2);
  const uint64_t lo = a * m, hi = mulhi64(a, m);
  const int nb = hi ? 128 - clz64(hi) : 64 - clz64(lo);  // bits of l2 * m
  const int sh = nb - 53;
  uint64_t q;
  int e = e0;
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
    return dist_value_slow(l2, step_sq);
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
  if (biased < 1 || biased > 254) return dist_value_slow(l2, step_sq);
  return bits_to_float((static_cast<uint32_t>(biased) << 23) |
                       static_cast<uint32_t>(q24 & 0x7FFFFFu));
}

#if defined(__CUDA_ARCH__)
// The same value from single-precision arithmetic, where that is provably
// exact (out = the result, true), else false. Classic error-free
// transformations (Dekker's product through fma, Fast2Sum):
//   l2 = xh 2^23 + xl with xh, xl < 2^23 (exact floats), so
//   S = l2 step_sq = xh a1 + xl s1 + [xh a2 + xl s2] + l2 r,
//   xh a1 = p1 + e1 and xl s1 = p3 + e3 exactly, p1 + p3 = s0 + e0 exactly,
//   S ~ s0 + tail, tail = e0 + e1 + e3 + p2 + p4 (p2, p4: the rounded
//   bracket), |S - (s0 + tail)| <= 16 2^-48 S.
// r = round(s0 + tail) and d ~ S - r (s0 - r is exact: Sterbenz). The double
// product rounds S to 53 bits (a move of at most 2^-53 S) and then to a
// float. If d lies inside r's rounding interval by more than twice
// M = 2^(E-166) (E: r's biased exponent; M exceeds the error terms above 16
// times over), both roundings end at r.
__device__ __forceinline__ bool dist_value_single(int64_t l2, const DistScale &s, float &out) {
  if (!s.single || l2 <= 0 || l2 >= (1ll << 46)) return false;
  const uint32_t xh = static_cast<uint32_t>(l2 >> 23), xl = static_cast<uint32_t>(l2) & 0x7FFFFFu;
  // v < 2^23 as a float: 2^23 + v has v in its mantissa, exactly
  const float fh = __fsub_rn(__uint_as_float(0x4B000000u | xh), 8388608.0f);
  const float fl = __fsub_rn(__uint_as_float(0x4B000000u | xl), 8388608.0f);
  const float p1 = __fmul_rn(fh, s.a1), e1 = __fmaf_rn(fh, s.a1, -p1);
  const float p3 = __fmul_rn(fl, s.s1), e3 = __fmaf_rn(fl, s.s1, -p3);
  const float p2 = __fmul_rn(fh, s.a2), p4 = __fmul_rn(fl, s.s2);
  // Fast2Sum: |p1| >= |p3| (xh >= 1 gives p1 >= a1 >= p3), or p1 = 0
  const float s0 = __fadd_rn(p1, p3);
  const float e0 = __fsub_rn(p3, __fsub_rn(s0, p1));
  const float tail = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(e0, e1), e3), p2), p4);
  const float r = __fadd_rn(s0, tail);
  const float d = __fadd_rn(__fsub_rn(s0, r), tail);
  const uint32_t rb = __float_as_uint(r), E = rb >> 23;
  if (E < 64 || E > 253) return false;
  // half the gaps to the next float up and down (down: a quarter ulp at a
  // power of two), less 2M; both differences are exact
  const float hup = __uint_as_float((E - 24) << 23);
  const float hdn = (rb & 0x7FFFFFu) ? hup : __uint_as_float((E - 25) << 23);
  const float m2 = __uint_as_float((E - 38) << 23);  // 2M = 2^(E-165)
  if (!(d < __fsub_rn(hup, m2) && -d < __fsub_rn(hdn, m2))) return false;
  out = r;
  return true;
}
#endif

// float(double(l2) * step_sq), bit for bit.
KATO_HD float dist_value(int64_t l2, const DistScale &s) {
#if defined(__CUDA_ARCH__)
  float r;
  if (dist_value_single(l2, s, r)) return r;
#endif
  return dist_value_exact(l2, s.m, s.e, s.step_sq);
}

}  // namespace kato
