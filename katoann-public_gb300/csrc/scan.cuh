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

}  // namespace kato
