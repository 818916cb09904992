// Exclusive prefix sums of two sequences at once by one CTA of 1024 threads
// (the list-sized scans of the search: nlist is at most a few 10^5).
#pragma once

#include <cstdint>

namespace kato {

// val(i) gives the pair of values at i < n; out(i, a, b) receives the pair of
// exclusive prefix sums there. Tiles of 4096: each thread takes 4 consecutive
// values (coalesced across the CTA), warps scan with shuffles. Returns the
// totals; all threads of the CTA must call it.
template <typename Val, typename Out>
__device__ uint2 block_scan2(uint32_t n, Val val, Out out) {
  __shared__ uint2 wsum[32];
  const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
  uint2 carry = make_uint2(0, 0);
  for (uint32_t base = 0; base < n; base += 4096) {
    const uint32_t i0 = base + t * 4;
    uint2 v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = i0 + k < n ? val(i0 + k) : make_uint2(0, 0);
    const uint2 ts = make_uint2(v[0].x + v[1].x + v[2].x + v[3].x, v[0].y + v[1].y + v[2].y + v[3].y);
    uint2 x = ts;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t ya = __shfl_up_sync(0xffffffffu, x.x, o), yb = __shfl_up_sync(0xffffffffu, x.y, o);
      if (lane >= static_cast<uint32_t>(o)) x.x += ya, x.y += yb;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      const uint2 w = wsum[lane];
      uint2 z = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t ya = __shfl_up_sync(0xffffffffu, z.x, o), yb = __shfl_up_sync(0xffffffffu, z.y, o);
        if (lane >= static_cast<uint32_t>(o)) z.x += ya, z.y += yb;
      }
      wsum[lane] = make_uint2(z.x - w.x, z.y - w.y);  // exclusive over warps
    }
    __syncthreads();
    uint2 e = make_uint2(carry.x + wsum[warp].x + x.x - ts.x, carry.y + wsum[warp].y + x.y - ts.y);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (i0 + k < n) out(i0 + k, e.x, e.y);
      e.x += v[k].x;
      e.y += v[k].y;
    }
    // the tile's total: the last thread's inclusive sum
    __shared__ uint2 tile_total;
    if (t == blockDim.x - 1) tile_total = make_uint2(e.x - carry.x, e.y - carry.y);
    __syncthreads();
    carry.x += tile_total.x;
    carry.y += tile_total.y;
    __syncthreads();
  }
  return carry;
}

// Radix-selection step by a whole CTA (blockDim.x >= 256, whole warps): the
// bin of a 256-bin histogram that holds the rank-th smallest value (rank <
// the histogram's total), into sel[0], and the count below that bin, into
// sel[1]. Thread t owns bin t; warp scans and the 8 warp totals (wsum) give
// each bin's exclusive prefix, and the one bin whose range holds the rank
// writes. Contains barriers: every thread of the CTA calls it.
__device__ __forceinline__ void block_pick_digit(const uint32_t *hist, uint32_t rank, uint32_t *sel,
                                                 uint32_t *wsum) {
  const uint32_t t = threadIdx.x, lane = t & 31, w = t >> 5;
  const uint32_t h = t < 256 ? hist[t] : 0u;
  uint32_t incl = h;
#pragma unroll
  for (uint32_t o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (t < 256 && lane == 31) wsum[w] = incl;
  __syncthreads();
  if (t < 256) {
    uint32_t base = 0;
    for (uint32_t i = 0; i < w; ++i) base += wsum[i];
    const uint32_t excl = base + incl - h;
    if (rank >= excl && rank < excl + h) {
      sel[0] = t;
      sel[1] = excl;
    }
  }
  __syncthreads();
}

}  // namespace kato
