// Exact SQ16 distance tiles (the reference's sq16_l2 / sq16_high_l2) and the
// coarse top-nprobe selection.
//
// A 16-bit code is h * 256 + l, so q.x = 65536 (qh.xh) + 256 (qh.xl + ql.xh)
// + ql.xl (include/katoann/kernels.h:163-170). Each of the three byte sums is
// accumulated in an exact 32-bit integer with packed 4-byte dot products
// (each sum is at most 2 * 4096 * 255^2 < 2^32), combined in 64 bits, and the
// squared L2 qn + xn - 2 q.x is mapped to the reference's float value by
// dist_value() (src/kernels.cpp:203-210).
#include "kcommon.cuh"

namespace kato {

namespace {

constexpr int kTile = 64;     // queries x database rows per CTA
constexpr int kKw = 16;       // 32-bit words (64 bytes) of each row per k-step
constexpr int kSw = kKw + 1;  // padded words per staged row

template <bool kFull>
__global__ void __launch_bounds__(256) sq16_tile_kernel(
    const uint8_t *__restrict__ qhi, const uint8_t *__restrict__ qlo,
    const uint8_t *__restrict__ xhi, const uint8_t *__restrict__ xlo,
    const int64_t *__restrict__ qn, const int64_t *__restrict__ xn, DistScale scale, uint32_t m,
    uint32_t n, uint32_t dims, uint32_t qstride, uint32_t xstride, float *__restrict__ out) {
  __shared__ uint32_t sqh[kTile * kSw], sxh[kTile * kSw];
  __shared__ uint32_t sql[kFull ? kTile * kSw : 1], sxl[kFull ? kTile * kSw : 1];
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  const uint32_t m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
  uint32_t hh[4][4], mx[4][4], ll[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) hh[a][b] = mx[a][b] = ll[a][b] = 0;

  // Staging: 64 rows x 64 bytes per array = 256 16-byte loads, one per thread.
  const int lr = t >> 2, lw = (t & 3) * 4;
  for (uint32_t k0 = 0; k0 < dims; k0 += kKw * 4) {
    {
      const uint32_t qi = m0 + lr, xi = n0 + lr;
      uint4 vqh = make_uint4(0, 0, 0, 0), vql = vqh, vxh = vqh, vxl = vqh;
      if (qi < m) {
        vqh = *reinterpret_cast<const uint4 *>(qhi + static_cast<size_t>(qi) * qstride + k0 + lw * 4);
        if (kFull) vql = *reinterpret_cast<const uint4 *>(qlo + static_cast<size_t>(qi) * qstride + k0 + lw * 4);
      }
      if (xi < n) {
        vxh = *reinterpret_cast<const uint4 *>(xhi + static_cast<size_t>(xi) * xstride + k0 + lw * 4);
        if (kFull) vxl = *reinterpret_cast<const uint4 *>(xlo + static_cast<size_t>(xi) * xstride + k0 + lw * 4);
      }
      uint32_t *dq = sqh + lr * kSw + lw, *dx = sxh + lr * kSw + lw;
      dq[0] = vqh.x; dq[1] = vqh.y; dq[2] = vqh.z; dq[3] = vqh.w;
      dx[0] = vxh.x; dx[1] = vxh.y; dx[2] = vxh.z; dx[3] = vxh.w;
      if (kFull) {
        uint32_t *eq = sql + lr * kSw + lw, *ex = sxl + lr * kSw + lw;
        eq[0] = vql.x; eq[1] = vql.y; eq[2] = vql.z; eq[3] = vql.w;
        ex[0] = vxl.x; ex[1] = vxl.y; ex[2] = vxl.z; ex[3] = vxl.w;
      }
    }
    __syncthreads();
#pragma unroll 4
    for (int w = 0; w < kKw; ++w) {
      uint32_t a_h[4], a_l[4], b_h[4], b_l[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        a_h[a] = sqh[(ty + 16 * a) * kSw + w];
        if (kFull) a_l[a] = sql[(ty + 16 * a) * kSw + w];
      }
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        b_h[b] = sxh[(tx + 16 * b) * kSw + w];
        if (kFull) b_l[b] = sxl[(tx + 16 * b) * kSw + w];
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          hh[a][b] = dp4(a_h[a], b_h[b], hh[a][b]);
          if (kFull) {
            mx[a][b] = dp4(a_h[a], b_l[b], mx[a][b]);
            mx[a][b] = dp4(a_l[a], b_h[b], mx[a][b]);
            ll[a][b] = dp4(a_l[a], b_l[b], ll[a][b]);
          }
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const uint32_t qi = m0 + ty + 16 * a;
    if (qi >= m) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const uint32_t xi = n0 + tx + 16 * b;
      if (xi >= n) continue;
      const int64_t dot = kFull ? static_cast<int64_t>((static_cast<uint64_t>(hh[a][b]) << 16) +
                                                       (static_cast<uint64_t>(mx[a][b]) << 8) +
                                                       ll[a][b])
                                : static_cast<int64_t>(hh[a][b]);
      out[static_cast<size_t>(qi) * n + xi] = dist_value(qn[qi] + xn[xi] - 2 * dot, scale);
    }
  }
}

// Smallest `p` of a row of `n` float distances (all >= 0, so their bit
// patterns order like the values) by (distance, list id), ascending.
// One CTA per query: radix selection of the p-th distance over 8-bit digits,
// then, among lists tied at that distance, of the smallest ids; the p chosen
// are then sorted (bitonic, in shared memory) when p <= kSortMax.
constexpr int kSelThreads = 256;
constexpr int kSortMax = 4096;

__device__ __forceinline__ uint32_t block_scan_bins(uint32_t *hist, uint32_t rank, uint32_t *sh_sel,
                                                    uint32_t *sh_below) {
  // Serial over 256 bins by warp 0 with a warp prefix sum.
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    uint32_t carry = 0;
    for (int base = 0; base < 256; base += 32) {
      const uint32_t v = hist[base + lane];
      uint32_t incl = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      const uint32_t excl = carry + incl - v;
      // the bin holding the rank-th element (0-based)
      const bool hit = excl <= rank && rank < excl + v;
      const uint32_t mask = __ballot_sync(0xffffffffu, hit);
      if (mask) {
        const int src = __ffs(mask) - 1;
        const uint32_t e = __shfl_sync(0xffffffffu, excl, src);
        if (lane == 0) {
          *sh_sel = base + src;
          *sh_below = e;
        }
        break;
      }
      carry += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
  __syncthreads();
  return *sh_sel;
}

// Smallest p keys of a row by (key, index) in up to six passes over the row
// (8-bit radix digits of the p-th key, then of the tied indices, then the
// gather). sel holds np2(p) 64-bit words, hist 256 counters, scal 4 words.
__device__ void select_passes(const uint32_t *__restrict__ keys, uint32_t n, uint32_t p,
                              uint32_t *__restrict__ outp, unsigned long long *__restrict__ tie_count,
                              unsigned long long *sel, uint32_t *hist, uint32_t *scal) {
  const uint32_t tid = threadIdx.x;
  // 1) the p-th smallest key (rank p-1), and how many keys are below it.
  uint32_t prefix = 0, rank = p - 1, below = 0;
  for (int shift = 24; shift >= 0; shift -= 8) {
    for (int i = tid; i < 256; i += kSelThreads) hist[i] = 0;
    __syncthreads();
    const uint32_t hmask = shift == 24 ? 0u : (0xFFFFFFFFu << (shift + 8));
    for (uint32_t i = tid; i < n; i += kSelThreads) {
      const uint32_t k = keys[i];
      if ((k & hmask) == prefix) atomicAdd(&hist[(k >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    const uint32_t bin = block_scan_bins(hist, rank, scal, scal + 1);
    rank -= scal[1];
    below += scal[1];
    prefix |= bin << shift;
    __syncthreads();
  }
  const uint32_t T = prefix;        // the p-th smallest key
  const uint32_t need = rank + 1;   // ids to take among keys == T
  // 2) among keys == T, the need-th smallest list id (only when ties exceed need).
  if (tid == 0) scal[3] = 0;
  __syncthreads();
  for (uint32_t i = tid; i < n; i += kSelThreads)
    if (keys[i] == T) atomicAdd(&scal[3], 1u);
  __syncthreads();
  const uint32_t neq = scal[3];
  uint32_t idmax = 0xFFFFFFFFu;
  if (neq > need) {
    if (tid == 0 && tie_count) atomicAdd(tie_count, 1ull);
    uint32_t ip = 0, ir = need - 1;
    for (int shift = 24; shift >= 0; shift -= 8) {
      for (int i = tid; i < 256; i += kSelThreads) hist[i] = 0;
      __syncthreads();
      const uint32_t hmask = shift == 24 ? 0u : (0xFFFFFFFFu << (shift + 8));
      for (uint32_t i = tid; i < n; i += kSelThreads)
        if (keys[i] == T && (i & hmask) == ip) atomicAdd(&hist[(i >> shift) & 0xFFu], 1u);
      __syncthreads();
      const uint32_t bin = block_scan_bins(hist, ir, scal, scal + 1);
      ir -= scal[1];
      ip |= bin << shift;
      __syncthreads();
    }
    idmax = ip;
  }
  // 3) gather the p selected.
  if (tid == 0) scal[2] = 0;
  __syncthreads();
  const bool sorted = p <= kSortMax;
  for (uint32_t i = tid; i < n; i += kSelThreads) {
    const uint32_t k = keys[i];
    if (k < T || (k == T && i <= idmax)) {
      const uint32_t pos = atomicAdd(&scal[2], 1u);
      if (sorted) sel[pos] = (static_cast<unsigned long long>(k) << 32) | i;
      else outp[pos] = i;
    }
  }
  __syncthreads();
  if (!sorted) return;
  // 4) bitonic sort of the p selected, padded to a power of two.
  uint32_t np2 = 1;
  while (np2 < p) np2 <<= 1;
  for (uint32_t i = p + tid; i < np2; i += kSelThreads) sel[i] = ~0ull;
  __syncthreads();
  for (uint32_t size = 2; size <= np2; size <<= 1) {
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t i = tid; i < np2; i += kSelThreads) {
        const uint32_t j = i ^ stride;
        if (j > i) {
          const bool up = (i & size) == 0;
          const unsigned long long a = sel[i], b = sel[j];
          if ((a > b) == up) {
            sel[i] = b;
            sel[j] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  for (uint32_t i = tid; i < p; i += kSelThreads) outp[i] = static_cast<uint32_t>(sel[i] & 0xFFFFFFFFu);
}

// Rows are written `stride` apart. With `only`, rows whose only[q] is at
// most only_above are skipped (a second, deeper selection for the queries
// that need it).
__global__ void __launch_bounds__(kSelThreads) select_topp_kernel(
    const float *__restrict__ dists, uint32_t n, uint32_t p, uint32_t stride,
    uint32_t *__restrict__ probed, unsigned long long *__restrict__ tie_count,
    const uint32_t *__restrict__ only, uint32_t only_above) {
  extern __shared__ unsigned long long sel[];  // up to kSortMax (key << 32 | id)
  __shared__ uint32_t hist[256], scal[4];
  const uint32_t q = blockIdx.x;
  if (only && only[q] <= only_above) return;
  select_passes(reinterpret_cast<const uint32_t *>(dists) + static_cast<size_t>(q) * n, n, p,
                probed + static_cast<size_t>(q) * stride, tie_count, sel, hist, scal);
}

// In-shared-memory bitonic sort of n 64-bit keys, ascending.
__device__ void sort_keys(unsigned long long *key, uint32_t n) {
  uint32_t np2 = 1;
  while (np2 < n) np2 <<= 1;
  for (uint32_t i = n + threadIdx.x; i < np2; i += blockDim.x) key[i] = ~0ull;
  __syncthreads();
  for (uint32_t size = 2; size <= np2; size <<= 1)
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t i = threadIdx.x; i < np2; i += blockDim.x) {
        const uint32_t j = i ^ stride;
        if (j > i) {
          const bool up = (i & size) == 0;
          const unsigned long long a = key[i], b = key[j];
          if ((a > b) == up) {
            key[i] = b;
            key[j] = a;
          }
        }
      }
      __syncthreads();
    }
}

// Smallest p of a row of n non-negative float distances by (distance, list),
// ascending, for p <= kSortMax, in two passes over the row: a histogram of
// the top 12 bits below the sign (distances cluster in a narrow range, so
// these bits still spread them), then a gather that takes every key of a bin
// below the boundary bin and collects the boundary bin's keys, of which the
// first (p - below) by (key, index) complete the selection. A boundary bin
// with more than kCand keys falls back to select_passes.
constexpr uint32_t kHistBins = 4096;
constexpr uint32_t kCand = 2048;

__global__ void __launch_bounds__(kSelThreads) select_topp_hist_kernel(
    const float *__restrict__ dists, uint32_t n, uint32_t p, uint32_t stride,
    uint32_t *__restrict__ probed, unsigned long long *__restrict__ tie_count,
    const uint32_t *__restrict__ only, uint32_t only_above) {
  extern __shared__ unsigned long long dyn[];
  unsigned long long *cand = dyn;          // kCand
  unsigned long long *sel = dyn + kCand;   // np2(p)
  __shared__ uint32_t hist[kHistBins];
  __shared__ uint32_t scal[8];
  __shared__ uint32_t wsum[kSelThreads / 32];
  const uint32_t q = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (only && only[q] <= only_above) return;
  const uint32_t *keys = reinterpret_cast<const uint32_t *>(dists) + static_cast<size_t>(q) * n;
  uint32_t *outp = probed + static_cast<size_t>(q) * stride;
  for (uint32_t i = tid; i < kHistBins; i += kSelThreads) hist[i] = 0;
  if (tid < 8) scal[tid] = 0;
  __syncthreads();
  const bool vec = (reinterpret_cast<uintptr_t>(keys) & 15) == 0;
  const uint32_t n4 = vec ? n / 4 : 0;
  auto bin_of = [](uint32_t k) { return (k >> 19) & (kHistBins - 1); };
  // 1) histogram
#pragma unroll 4
  for (uint32_t i = tid; i < n4; i += kSelThreads) {
    const uint4 v = reinterpret_cast<const uint4 *>(keys)[i];
    atomicAdd(&hist[bin_of(v.x)], 1u);
    atomicAdd(&hist[bin_of(v.y)], 1u);
    atomicAdd(&hist[bin_of(v.z)], 1u);
    atomicAdd(&hist[bin_of(v.w)], 1u);
  }
  for (uint32_t i = n4 * 4 + tid; i < n; i += kSelThreads) atomicAdd(&hist[bin_of(keys[i])], 1u);
  __syncthreads();
  // 2) the bin holding rank p - 1: each thread owns 16 consecutive bins
  constexpr uint32_t kPer = kHistBins / kSelThreads;
  uint32_t tsum = 0;
#pragma unroll
  for (uint32_t j = 0; j < kPer; ++j) tsum += hist[tid * kPer + j];
  uint32_t incl = tsum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= static_cast<uint32_t>(o)) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  uint32_t wbase = 0;
  for (uint32_t w = 0; w < warp; ++w) wbase += wsum[w];
  const uint32_t excl = wbase + incl - tsum, rank = p - 1;
  if (rank >= excl && rank < excl + tsum) {
    uint32_t acc = excl, j = 0;
    for (; j < kPer; ++j) {
      const uint32_t h = hist[tid * kPer + j];
      if (rank < acc + h) break;
      acc += h;
    }
    scal[0] = tid * kPer + j;  // boundary bin
    scal[1] = acc;             // keys below it
  }
  __syncthreads();
  const uint32_t bstar = scal[0], below = scal[1], c = hist[bstar];
  if (c > kCand) {  // a crowded boundary bin: the radix passes instead
    select_passes(keys, n, p, outp, tie_count, sel, hist, scal + 4);
    return;
  }
  // 3) gather: bins below the boundary are in; the boundary bin is a candidate
  auto take = [&](uint32_t k, uint32_t i) {
    const uint32_t b = bin_of(k);
    if (b < bstar) sel[atomicAdd(&scal[2], 1u)] = (static_cast<unsigned long long>(k) << 32) | i;
    else if (b == bstar) cand[atomicAdd(&scal[3], 1u)] = (static_cast<unsigned long long>(k) << 32) | i;
  };
#pragma unroll 4
  for (uint32_t i = tid; i < n4; i += kSelThreads) {
    const uint4 v = reinterpret_cast<const uint4 *>(keys)[i];
    take(v.x, 4 * i);
    take(v.y, 4 * i + 1);
    take(v.z, 4 * i + 2);
    take(v.w, 4 * i + 3);
  }
  for (uint32_t i = n4 * 4 + tid; i < n; i += kSelThreads) take(keys[i], i);
  __syncthreads();
  // 4) the boundary bin's keys in order; the first `need` complete the set
  sort_keys(cand, c);
  const uint32_t need = p - below;
  for (uint32_t i = tid; i < need; i += kSelThreads) sel[below + i] = cand[i];
  if (tid == 0 && tie_count && need < c && (cand[need] >> 32) == (cand[need - 1] >> 32))
    atomicAdd(tie_count, 1ull);
  __syncthreads();
  // 5) the p selected in order
  sort_keys(sel, p);
  for (uint32_t i = tid; i < p; i += kSelThreads) outp[i] = static_cast<uint32_t>(sel[i] & 0xFFFFFFFFu);
}

__global__ void dist_values_kernel(const int64_t *l2, uint32_t n, DistScale s, float *out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = dist_value(l2[i], s);
}

}  // namespace

int sq16_tiles(const uint8_t *qhi, const uint8_t *qlo, const uint8_t *xhi, const uint8_t *xlo,
               const int64_t *qn, const int64_t *xn, double step_sq, uint32_t m, uint32_t n,
               uint32_t dims, uint32_t qstride, uint32_t xstride, float *out, bool full,
               cudaStream_t st) {
  if (m == 0 || n == 0) return KATO_OK;
  if (dims % 64 || dims == 0) return invalid("dims must be a positive multiple of 64");
  if (qstride % 16 || xstride % 16) return invalid("row strides must be multiples of 16 bytes");
  const DistScale s = make_dist_scale(step_sq);
  dim3 grid(div_up(n, kTile), div_up(m, kTile));
  if (grid.y > 65535) return invalid("too many query rows for one call");
  if (full) sq16_tile_kernel<true><<<grid, 256, 0, st>>>(qhi, qlo, xhi, xlo, qn, xn, s, m, n, dims, qstride, xstride, out);
  else sq16_tile_kernel<false><<<grid, 256, 0, st>>>(qhi, qlo, xhi, xlo, qn, xn, s, m, n, dims, qstride, xstride, out);
  KATO_LAUNCHED("sq16_tile_kernel");
  return KATO_OK;
}

int select_topp_ex(const float *dists, uint32_t nq, uint32_t n, uint32_t p, uint32_t stride,
                   uint32_t *probed, unsigned long long *tie_count, const uint32_t *only,
                   uint32_t only_above, cudaStream_t st) {
  if (nq == 0) return KATO_OK;
  if (p == 0 || p > n || stride < p) return invalid("need 1 <= nprobe <= nlist");
  uint32_t np2 = 1;
  while (np2 < p) np2 <<= 1;
  int rc;
  if ((rc = smem_limit(reinterpret_cast<const void *>(select_topp_kernel), kSortMax * 8,
                       "select_topp_kernel shared memory")) ||
      (rc = smem_limit(reinterpret_cast<const void *>(select_topp_hist_kernel),
                       (kCand + kSortMax) * 8, "select_topp_hist_kernel shared memory")))
    return rc;
  if (p <= kSortMax) {
    // candidates and the sorted selection (the bitonic sort pads to a power of two)
    const size_t smem = (kCand + std::max<uint32_t>(np2, 2)) * sizeof(unsigned long long);
    select_topp_hist_kernel<<<nq, kSelThreads, smem, st>>>(dists, n, p, stride, probed, tie_count,
                                                            only, only_above);
    KATO_LAUNCHED("select_topp_hist_kernel");
    return KATO_OK;
  }
  select_topp_kernel<<<nq, kSelThreads, 0, st>>>(dists, n, p, stride, probed, tie_count, only,
                                                  only_above);
  KATO_LAUNCHED("select_topp_kernel");
  return KATO_OK;
}

int select_topp(const float *dists, uint32_t nq, uint32_t n, uint32_t p, uint32_t *probed,
                unsigned long long *tie_count, cudaStream_t st) {
  return select_topp_ex(dists, nq, n, p, p, probed, tie_count, nullptr, 0, st);
}

int dist_values(const int64_t *l2, uint32_t n, double step_sq, float *out, cudaStream_t st) {
  if (n == 0) return KATO_OK;
  dist_values_kernel<<<div_up(n, 256), 256, 0, st>>>(l2, n, make_dist_scale(step_sq), out);
  KATO_LAUNCHED("dist_values_kernel");
  return KATO_OK;
}

}  // namespace kato
