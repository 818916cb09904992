// Rotation and 16-bit coding of rows on the GPU, bit-identical to the
// reference's float arithmetic.
//
// The reference computes every rotated value out[i][j] = <x_i, r_j> with 16
// lane accumulators: lane l sums x[k] * r[k] over k = l, l + 16, ... by fused
// multiply-add in k order, the 16 lanes are added as (l, l+8), (l, l+4),
// (l, l+2), (0, 1), and the last d % 16 dimensions follow one by one
// (src/index.cpp:139-208). Here 16 consecutive threads of a warp play the 16
// lanes: each thread keeps the lane sums of an 8 x 8 block of outputs, and the
// lane reduction is a xor-butterfly of shuffles (8, 4, 2, 1), which adds the
// same pairs in the same order, so every thread ends with the reference's
// bits. The scalar parts are replayed with explicit rounding: the reference's
// compiler evaluates those chains four products at a time with the products
// rounded, then fuses the last (length % 4) terms.
#include "kcommon.cuh"

namespace kato {

namespace {

constexpr int kRotRows = 32;     // output rows per CTA
constexpr int kRotCols = 32;     // output columns per CTA
constexpr int kRotK = 64;        // k-chunk staged in shared memory
constexpr int kRotStride = 36;   // floats per staged k (rows/columns 0..31 + pad: 16-byte
                                 // aligned and conflict-free for 128-bit reads)

// Scalar tail of one output: dimensions [k0, d), the first ((d - k0) & ~3) of
// them with rounded products, the rest fused.
__device__ __forceinline__ float rot_tail(float s, const float *x, const float *r, uint32_t k0,
                                          uint32_t d) {
  const uint32_t m = k0 + ((d - k0) & ~3u);
  uint32_t k = k0;
  for (; k < m; ++k) s = __fadd_rn(s, __fmul_rn(x[k], r[k]));
  for (; k < d; ++k) s = __fmaf_rn(x[k], r[k], s);
  return s;
}

// 4-byte asynchronous global -> shared copy; src_bytes 0 writes a zero.
__device__ __forceinline__ void cp_async4(float *dst, const float *src, uint32_t src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(
                   static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
               "l"(src), "r"(src_bytes)
               : "memory");
}

// 16-byte asynchronous global -> shared copy (L2 only).
__device__ __forceinline__ void cp_async16(float *dst, const float *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                   static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
               "l"(src)
               : "memory");
}

// kMajor: the staged parts are read from k-major copies xt (d x ldx, rows
// zero-padded to ldx) and rt (d x ldr, columns zero-padded), 16 bytes per
// copy; otherwise from the row-major inputs, 4 bytes per copy.
// Two CTAs per SM (118 registers, no spills): 4096 x 1024 queries in 0.32 ms.
template <bool kMajor>
__global__ void __launch_bounds__(256, 2) rotate_lanes_kernel(const float *__restrict__ in,
                                                              uint32_t nrows, uint32_t d,
                                                              const float *__restrict__ rot,
                                                              const float *__restrict__ xt,
                                                              uint32_t ldx,
                                                              const float *__restrict__ rt,
                                                              uint32_t ldr,
                                                              float *__restrict__ out) {
  // two stages, each staged k-major (xs[k][row], rs[k][column]) so that a
  // thread reads its 8 rows and 8 columns at one k with four 128-bit loads;
  // the next chunk is copied asynchronously while the current one is used
  __shared__ __align__(16) float xs[2][kRotK * kRotStride];
  __shared__ __align__(16) float rs[2][kRotK * kRotStride];
  const uint32_t d4 = d & ~3u, d16 = d & ~15u;
  const uint32_t i0 = blockIdx.x * kRotRows, j0 = blockIdx.y * kRotCols;
  const int t = threadIdx.x, l = t & 15, g = t >> 4;
  const int rb = (g >> 2) * 8, cb = (g & 3) * 8;
  float acc[8][8];
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int b = 0; b < 8; ++b) acc[a][b] = 0.0f;

  auto stage = [&](uint32_t k0, int buf) {
    if constexpr (kMajor) {
      // per k: 32 rows (8 copies) of x and 32 columns of r
      const uint32_t kn = min(static_cast<uint32_t>(kRotK), d16 - k0);
      for (uint32_t idx = t; idx < kn * 8; idx += 256) {
        const uint32_t c = idx >> 3, q = (idx & 7) * 4;
        cp_async16(&xs[buf][c * kRotStride + q], xt + static_cast<size_t>(k0 + c) * ldx + i0 + q);
        cp_async16(&rs[buf][c * kRotStride + q], rt + static_cast<size_t>(k0 + c) * ldr + j0 + q);
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    } else {
      for (int idx = t; idx < kRotRows * kRotK; idx += 256) {
        const int r = idx / kRotK, c = idx % kRotK;
        const uint32_t gk = k0 + c;
        const uint32_t gi = i0 + r, gj = j0 + r;
        const bool okx = gi < nrows && gk < d16, okr = gj < d4 && gk < d16;
        cp_async4(&xs[buf][c * kRotStride + r], okx ? in + static_cast<size_t>(gi) * d + gk : in,
                  okx ? 4u : 0u);
        cp_async4(&rs[buf][c * kRotStride + r], okr ? rot + static_cast<size_t>(gj) * d + gk : rot,
                  okr ? 4u : 0u);
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    }
  };
  int buf = 0;
  if (d16) stage(0, 0);
  for (uint32_t k0 = 0; k0 < d16; k0 += kRotK, buf ^= 1) {
    if (k0 + kRotK < d16) {
      stage(k0 + kRotK, buf ^ 1);
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    __syncthreads();
    const uint32_t kend = min(static_cast<uint32_t>(kRotK), d16 - k0);
    // this lane's dimension of each 16-dimension step: fixed offsets from one
    // base per chunk, the four steps unrolled (kend is a multiple of 16)
    const float *xl = xs[buf] + l * kRotStride + rb, *rl = rs[buf] + l * kRotStride + cb;
#pragma unroll
    for (uint32_t c = 0; c < kRotK; c += 16) {
      if (c < kend) {
        const float4 x0 = *reinterpret_cast<const float4 *>(xl + c * kRotStride);
        const float4 x1 = *reinterpret_cast<const float4 *>(xl + c * kRotStride + 4);
        const float4 r0 = *reinterpret_cast<const float4 *>(rl + c * kRotStride);
        const float4 r1 = *reinterpret_cast<const float4 *>(rl + c * kRotStride + 4);
        const float xv[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
        const float rv[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
          for (int b = 0; b < 8; ++b) acc[a][b] = __fmaf_rn(xv[a], rv[b], acc[a][b]);
      }
    }
    __syncthreads();  // the buffer is refilled by the next iteration's copies
  }
  // Lane reduction as a reduce-scatter: at each step (lane distance 8, 4, 2,
  // 1) a lane keeps half of its outputs and adds its partner's partial sums
  // of them. Every output meets the same pairs in the same order as in the
  // reference's horizontal add (IEEE addition is commutative), and lane l
  // ends with the four outputs a = 4 b3 + 2 b2 + b1, b = 4 b0 .. 4 b0 + 3
  // (b3 .. b0 the bits of l): 60 shuffles instead of 256, and no spills.
  float v[64];
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int b = 0; b < 8; ++b) v[a * 8 + b] = acc[a][b];
#pragma unroll
  for (int step = 0, half = 32, m = 8; step < 4; ++step, half >>= 1, m >>= 1) {
    const bool hi = (l & m) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      const float send = hi ? v[i] : v[i + half];
      const float keep = hi ? v[i + half] : v[i];
      v[i] = __fadd_rn(keep, __shfl_xor_sync(0xffffffffu, send, m));
    }
  }
  // the scalar tail and the store of this lane's four outputs
  const int a = 4 * ((l >> 3) & 1) + 2 * ((l >> 2) & 1) + ((l >> 1) & 1), b0 = 4 * (l & 1);
  const uint32_t i = i0 + rb + a, j = j0 + cb + b0;
  if (i < nrows) {
    const float *x = in + static_cast<size_t>(i) * d;
    float *o = out + static_cast<size_t>(i) * d + j;
    if (d16 == d && j + 4 <= d4 && (reinterpret_cast<uintptr_t>(o) & 15u) == 0) {
      *reinterpret_cast<float4 *>(o) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (j + e < d4) o[e] = rot_tail(v[e], x, rot + static_cast<size_t>(j + e) * d, d16, d);
    }
  }
}

// out[k * ld + r] = in[r * d + k] for r < rows (zero for rows <= r < ld),
// k < kn: 32 x 32 tiles through shared memory.
__global__ void __launch_bounds__(256) transpose_pad_kernel(const float *__restrict__ in,
                                                            uint32_t rows, uint32_t d, uint32_t kn,
                                                            float *__restrict__ out, uint32_t ld) {
  __shared__ float tile[32][33];
  const uint32_t r0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const uint32_t tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (uint32_t y = ty; y < 32; y += 8) {
    const uint32_t r = r0 + y, k = k0 + tx;
    tile[y][tx] = (r < rows && k < kn) ? in[static_cast<size_t>(r) * d + k] : 0.0f;
  }
  __syncthreads();
  for (uint32_t y = ty; y < 32; y += 8) {
    const uint32_t k = k0 + y, r = r0 + tx;
    if (k < kn && r < ld) out[static_cast<size_t>(k) * ld + r] = tile[tx][y];
  }
}

// The same transpose with 16-byte accesses on both sides (d % 4 == 0, `in`
// 16-byte aligned, ld % 32 == 0): 64 x 64 tiles, four float4 loads and four
// float4 stores per thread.
__global__ void __launch_bounds__(256) transpose_pad4_kernel(const float *__restrict__ in,
                                                             uint32_t rows, uint32_t d, uint32_t kn,
                                                             float *__restrict__ out, uint32_t ld) {
  __shared__ float tile[64][65];
  const uint32_t r0 = blockIdx.x * 64, k0 = blockIdx.y * 64;
  const uint32_t t = threadIdx.x;
#pragma unroll
  for (uint32_t i = 0; i < 4; ++i) {
    const uint32_t idx = t + 256 * i, rr = idx >> 4, k = k0 + (idx & 15) * 4;
    float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (r0 + rr < rows && k < kn)
      v = *reinterpret_cast<const float4 *>(in + static_cast<size_t>(r0 + rr) * d + k);
    float *dst = &tile[rr][(idx & 15) * 4];
    dst[0] = v.x, dst[1] = v.y, dst[2] = v.z, dst[3] = v.w;
  }
  __syncthreads();
#pragma unroll
  for (uint32_t i = 0; i < 4; ++i) {
    const uint32_t idx = t + 256 * i, kk = idx >> 4, r = (idx & 15) * 4;
    if (k0 + kk < kn && r0 + r < ld)
      *reinterpret_cast<float4 *>(out + static_cast<size_t>(k0 + kk) * ld + r0 + r) =
          make_float4(tile[r][kk], tile[r + 1][kk], tile[r + 2][kk], tile[r + 3][kk]);
  }
}

// out (kn x ld, k-major) from in (rows x d, row-major), zero-padded rows.
void transpose_pad(const float *in, uint32_t rows, uint32_t d, uint32_t kn, float *out, uint32_t ld,
                   cudaStream_t st) {
  if (d % 4 == 0 && ld % 32 == 0 && reinterpret_cast<uintptr_t>(in) % 16 == 0)
    transpose_pad4_kernel<<<dim3(div_up(ld, 64), div_up(kn, 64)), 256, 0, st>>>(in, rows, d, kn, out,
                                                                                ld);
  else
    transpose_pad_kernel<<<dim3(ld / 32, div_up(kn, 32)), 256, 0, st>>>(in, rows, d, kn, out, ld);
}

// The last d % 4 output columns: one chain over all d dimensions
// (src/index.cpp:171-179, :247-257).
__global__ void rotate_seq_kernel(const float *__restrict__ in, uint32_t nrows, uint32_t d,
                                  const float *__restrict__ rot, float *__restrict__ out) {
  const uint32_t d4 = d & ~3u, nc = d - d4;
  const uint64_t idx = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= static_cast<uint64_t>(nrows) * nc) return;
  const uint32_t i = static_cast<uint32_t>(idx / nc), j = d4 + static_cast<uint32_t>(idx % nc);
  out[static_cast<size_t>(i) * d + j] =
      rot_tail(0.0f, in + static_cast<size_t>(i) * d, rot + static_cast<size_t>(j) * d, 0, d);
}

__global__ void minmax_init_kernel(uint32_t *keys) {
  keys[0] = 0xFFFFFFFFu;  // min
  keys[1] = 0u;           // max
}

__global__ void minmax_kernel(const float *__restrict__ x, size_t n, uint32_t *keys) {
  uint32_t mn = 0xFFFFFFFFu, mx = 0u;
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const uint32_t k = float_order_key(x[i]);
    mn = min(mn, k);
    mx = max(mx, k);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(keys, mn);
    atomicMax(keys + 1, mx);
  }
}

// One warp per row: codes, byte planes (padding zero) and the three norms.
__global__ void quantize_rows_kernel(const float *__restrict__ x, uint32_t nrows, uint32_t d,
                                     uint32_t dc, float lo, double inv_step, uint32_t head,
                                     uint8_t *__restrict__ hi, uint8_t *__restrict__ lop,
                                     int64_t *__restrict__ norm, int64_t *__restrict__ hinorm,
                                     int64_t *__restrict__ headnorm) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t warp = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
  const QuantScale qs = quant_scale(lo, inv_step);
  for (uint64_t row = warp; row < nrows; row += nwarps) {
    const float *xr = x + row * d;
    uint8_t *hr = hi + row * dc;
    uint8_t *lr = lop + row * dc;
    uint64_t s = 0, sh = 0, s0 = 0;
    for (uint32_t k = lane; k < dc; k += 32) {
      uint32_t v = 0;
      if (k < d) v = quantize1(xr[k], qs);
      const uint32_t vh = v >> 8;
      hr[k] = static_cast<uint8_t>(vh);
      lr[k] = static_cast<uint8_t>(v & 0xFFu);
      s += static_cast<uint64_t>(v) * v;
      sh += vh * vh;
      if (k < head) s0 += vh * vh;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_xor_sync(0xffffffffu, s, o);
      sh += __shfl_xor_sync(0xffffffffu, sh, o);
      s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    }
    if (lane == 0) {
      norm[row] = static_cast<int64_t>(s);
      hinorm[row] = static_cast<int64_t>(sh);
      if (headnorm) headnorm[row] = static_cast<int64_t>(s0);
    }
  }
}

}  // namespace

int rotate_rows(const float *in, uint32_t nrows, uint32_t d, const float *rot, float *out,
                cudaStream_t st) {
  if (nrows == 0) return KATO_OK;
  const uint32_t d4 = d & ~3u;
  if (d4) {
    dim3 grid(div_up(nrows, kRotRows), div_up(d4, kRotCols));
    rotate_lanes_kernel<false><<<grid, 256, 0, st>>>(in, nrows, d, rot, nullptr, 0, nullptr, 0, out);
    KATO_LAUNCHED("rotate_lanes_kernel");
  }
  if (d4 < d) {
    const uint64_t n = static_cast<uint64_t>(nrows) * (d - d4);
    rotate_seq_kernel<<<static_cast<uint32_t>((n + 255) / 256), 256, 0, st>>>(in, nrows, d, rot, out);
    KATO_LAUNCHED("rotate_seq_kernel");
  }
  return KATO_OK;
}

size_t rotate_scratch_bytes(uint32_t nrows, uint32_t d) {
  const size_t ldx = (static_cast<size_t>(nrows) + 31) / 32 * 32;
  const size_t ldr = (static_cast<size_t>(d & ~3u) + 31) / 32 * 32;
  return (ldx + ldr) * (d & ~15u) * 4 + 256;
}

size_t rotation_kmajor_bytes(uint32_t d) {
  const size_t ldr = (static_cast<size_t>(d & ~3u) + 31) / 32 * 32;
  return ldr * (d & ~15u) * 4;
}

int rotation_kmajor(const float *rot, uint32_t d, float *out, cudaStream_t st) {
  const uint32_t d4 = d & ~3u, d16 = d & ~15u;
  if (d16 == 0) return KATO_OK;
  transpose_pad(rot, d4, d, d16, out, div_up(d4, 32) * 32, st);
  KATO_LAUNCHED("transpose_pad_kernel");
  return KATO_OK;
}

int rotate_rows_kmajor(const float *in, uint32_t nrows, uint32_t d, const float *rot,
                       const float *rot_kmajor, void *scratch, float *out, cudaStream_t st) {
  if (nrows == 0) return KATO_OK;
  const uint32_t d4 = d & ~3u, d16 = d & ~15u;
  if (d16 == 0) return rotate_rows(in, nrows, d, rot, out, st);
  const uint32_t ldx = div_up(nrows, 32) * 32, ldr = div_up(d4, 32) * 32;
  float *xt = static_cast<float *>(scratch);
  const float *rt = rot_kmajor;
  transpose_pad(in, nrows, d, d16, xt, ldx, st);
  if (!rt) {  // no copy made at load: transpose the rotation here
    float *t = xt + static_cast<size_t>(ldx) * d16;
    transpose_pad(rot, d4, d, d16, t, ldr, st);
    rt = t;
  }
  KATO_LAUNCHED("transpose_pad_kernel");
  dim3 grid(div_up(nrows, kRotRows), div_up(d4, kRotCols));
  rotate_lanes_kernel<true><<<grid, 256, 0, st>>>(in, nrows, d, rot, xt, ldx, rt, ldr, out);
  KATO_LAUNCHED("rotate_lanes_kernel");
  if (d4 < d) {
    const uint64_t n = static_cast<uint64_t>(nrows) * (d - d4);
    rotate_seq_kernel<<<static_cast<uint32_t>((n + 255) / 256), 256, 0, st>>>(in, nrows, d, rot, out);
    KATO_LAUNCHED("rotate_seq_kernel");
  }
  return KATO_OK;
}

int minmax(const float *x, size_t n, uint32_t *d_keys, float *h_out, cudaStream_t st) {
  minmax_init_kernel<<<1, 1, 0, st>>>(d_keys);
  KATO_LAUNCHED("minmax_init_kernel");
  if (n) {
    const uint32_t blocks = static_cast<uint32_t>(std::min<size_t>((n + 255) / 256, 152 * 16));
    minmax_kernel<<<blocks, 256, 0, st>>>(x, n, d_keys);
    KATO_LAUNCHED("minmax_kernel");
  }
  uint32_t keys[2];
  KATO_CUDA(cudaMemcpyAsync(keys, d_keys, sizeof(keys), cudaMemcpyDeviceToHost, st));
  KATO_CUDA(cudaStreamSynchronize(st));
  h_out[0] = float_from_order_key(keys[0]);
  h_out[1] = float_from_order_key(keys[1]);
  return KATO_OK;
}

int quantize_rows(const float *x, uint32_t nrows, uint32_t d, uint32_t dc, float lo,
                  double inv_step, uint32_t head, uint8_t *hi, uint8_t *lop, int64_t *norm,
                  int64_t *hinorm, int64_t *headnorm, cudaStream_t st) {
  if (nrows == 0) return KATO_OK;
  const uint32_t blocks = std::min<uint32_t>(div_up(nrows, 8), 152 * 64);
  quantize_rows_kernel<<<blocks, 256, 0, st>>>(x, nrows, d, dc, lo, inv_step, head, hi, lop, norm,
                                              hinorm, headnorm);
  KATO_LAUNCHED("quantize_rows_kernel");
  return KATO_OK;
}

}  // namespace kato
