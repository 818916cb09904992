// Index build on the device: k-means++ seeding, Lloyd iterations, the
// assignment of every vector to its nearest centroid, and the covariance the
// PCA rotation is computed from.
//
// The reference builds on the host (Index::build, src/index.cpp:419-514):
// k-means++ seeding (src/kmeans.cpp:280-321), Elkan-bounded Lloyd iterations
// (:73-187, :239-278) and closest_centers as three float GEMMs
// (:191-237); the PCA covariance is accumulated in double
// (src/index.cpp:276-312). The partition is not part of search parity (both
// systems search whatever index files they are given), so the device build is
// free to take its own arithmetic:
//
//  * kmeans_assign_kernel: the nearest centroid of every row, as one GEMM on
//    the 5th-generation tensor cores with the argmin fused into its epilogue.
//    The rows and centroids are fp32 in HBM, zero-padded to a multiple of 32
//    dimensions; TMA loads 32-dimension slices (128-byte swizzle) of a
//    128-row tile and a 256-centroid tile into a ring of stages, one thread
//    issues tcgen05.mma kind::tf32 (M = 128, N = 256, K = 8) into
//    double-buffered fp32 TMEM accumulators, and four epilogue warps keep
//    each row's running minimum of |c|^2 - 2 x.c over the centroid tiles
//    (ties to the smaller centroid). TF32 keeps 10 mantissa bits of each
//    operand: rows whose two nearest centroids are closer than that
//    resolution may go to either, which changes the partition, not the
//    search.
//  * kmeans_sums_kernel / kmeans_centres_kernel: the Lloyd update, sums in
//    double, empty clusters keep their centre.
//  * pp_update_kernel / pp_pick_kernel: k-means++ (D^2 sampling). Per new
//    centre, every row's distance to its nearest centre so far is updated
//    and summed in fixed-order blocks; one CTA then walks the block sums and
//    the chosen block's rows to the point where the running sum passes
//    u * total, u from the caller's seeded stream.
//  * cov_kernel: the mean-centred covariance of a sample in double.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cfloat>

#include "kcommon.cuh"
#include "tc.cuh"

namespace kato {

namespace {

constexpr uint32_t kRM = 128;   // rows per tile (the MMA's M)
constexpr uint32_t kCN = 256;   // centroids per tile (the MMA's N)
constexpr uint32_t kKB = 32;    // fp32 dimensions per stage: one 128-byte swizzle row
constexpr uint32_t kStages = 4;
constexpr uint32_t kXTile = kRM * kKB * 4;  // 16 KiB
constexpr uint32_t kCTile = kCN * kKB * 4;  // 32 KiB
constexpr uint32_t kStage = kXTile + kCTile;
static_assert(kXTile % 1024 == 0 && kCTile % 1024 == 0, "swizzle atoms");
constexpr uint32_t kTmemCols = 2 * kCN;     // two accumulator slots of 256 fp32 columns
constexpr int kEpiWarps = 4;                // one per TMEM lane quarter: thread = row
constexpr int kThreads = (2 + kEpiWarps) * 32;
constexpr uint32_t kSmem = kStages * kStage + 4096;  // + alignment, barriers, exchange

// Instruction descriptor of kind::tf32: fp32 accumulator, TF32 A and B (K-major).
__host__ __device__ constexpr uint32_t idesc_tf32(uint32_t m, uint32_t n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr) {
  return static_cast<uint64_t>((addr & 0x3FFFFu) >> 4) | (1ull << 16) | (64ull << 32) |
         (1ull << 46) | (2ull << 61);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

struct AssignArgs {
  const float *cnorm;  // L: |c|^2
  uint32_t *assign;    // n
  float *best;         // n: |c|^2 - 2 x.c of the nearest centroid (may be null)
  uint32_t n, L, ld;
  uint32_t *timeouts;
};

__global__ void __launch_bounds__(kThreads, 1)
    kmeans_assign_kernel(const __grid_constant__ CUtensorMap tx, const __grid_constant__ CUtensorMap tcen,
                         const AssignArgs A) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char *sm = smraw + ((1024 - (tc::smem_addr(smraw) & 1023u)) & 1023u);
  uint64_t *full = reinterpret_cast<uint64_t *>(sm + kStages * kStage);
  uint64_t *empty = full + kStages, *acc_full = empty + kStages, *acc_empty = acc_full + 2;
  uint64_t *done = acc_empty + 2;
  uint32_t *tbase = reinterpret_cast<uint32_t *>(done + 1);
  volatile uint32_t *err = tbase + 1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (uint32_t s = 0; s < kStages; ++s) {
      tc::mbar_init(full + s, 1);
      tc::mbar_init(empty + s, 1);
    }
    for (uint32_t s = 0; s < 2; ++s) {
      tc::mbar_init(acc_full + s, 1);
      tc::mbar_init(acc_empty + s, kEpiWarps);
    }
    tc::mbar_init(done, 1);
    *err = 0;
    tc::fence_barrier_init();
  }
  if (warp == 1) tc::tmem_alloc(tbase, kTmemCols);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tbase;
  const uint32_t nrt = div_up(A.n, kRM), nct = div_up(A.L, kCN), nk = A.ld / kKB;

  if (warp == 0) {
    // ---- TMA producer: per row tile, every centroid tile, every K slice
    if (lane == 0) {
      uint32_t s = 0, ph = 0, issued = 0, last_par[kStages] = {};
      bool ok = true;
      for (uint32_t t = blockIdx.x; ok && t < nrt; t += gridDim.x)
        for (uint32_t ct = 0; ok && ct < nct; ++ct)
          for (uint32_t k = 0; k < nk; ++k) {
            if (!tc::mbar_wait_or(empty + s, ph ^ 1, err)) {
              ok = false;
              break;
            }
            unsigned char *st = sm + s * kStage;
            const int32_t x = static_cast<int32_t>(k * kKB);
            tc::mbar_expect_tx(full + s, kStage);
            tc::tma_load_2d(st, &tx, x, static_cast<int32_t>(t * kRM), full + s);
            tc::tma_load_2d(st + kXTile, &tcen, x, static_cast<int32_t>(ct * kCN), full + s);
            issued |= 1u << s;
            last_par[s] = ph;
            if (++s == kStages) s = 0, ph ^= 1;
          }
      if (*err)  // copies still in flight land before the CTA exits
        for (uint32_t i = 0; i < kStages; ++i)
          if (issued >> i & 1u) tc::mbar_wait(full + i, last_par[i]);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---- MMA issuer: one accumulator slot per (row tile, centroid tile)
    if (lane == 0) {
      const uint32_t idesc = idesc_tf32(kRM, kCN);
      uint32_t s = 0, ph = 0, ab = 0, abph = 0;
      bool ok = true;
      for (uint32_t t = blockIdx.x; ok && t < nrt; t += gridDim.x)
        for (uint32_t ct = 0; ok && ct < nct; ++ct) {
          if (!tc::mbar_wait_or(acc_empty + ab, abph ^ 1, err)) {
            ok = false;
            break;
          }
          tc::fence_after();
          const uint32_t d0 = tmem + ab * kCN;
          for (uint32_t k = 0; k < nk; ++k) {
            if (!tc::mbar_wait_or(full + s, ph, err)) {
              ok = false;
              break;
            }
            tc::fence_after();
            const uint32_t st = tc::smem_addr(sm + s * kStage);
            const uint64_t a = desc_sw128(st), b = desc_sw128(st + kXTile);
#pragma unroll
            for (uint32_t j = 0; j < kKB / 8; ++j)  // K = 8 tf32 = 32 bytes: +2 encoded
              mma_tf32(d0, a + 2 * j, b + 2 * j, idesc, (k | j) != 0);
            tc::commit(empty + s);
            if (++s == kStages) s = 0, ph ^= 1;
          }
          if (!ok) break;
          tc::commit(acc_full + ab);
          if (++ab == 2) ab = 0, abph ^= 1;
        }
      tc::commit(done);  // every MMA issued has completed before TMEM is released
      tc::mbar_wait(done, 0);
    }
    __syncwarp();
  } else {
    // ---- epilogue: thread = row (its TMEM lane), all 256 columns of a tile
    const uint32_t row = (warp & 3) * 32 + lane;
    uint32_t ab = 0, abph = 0;
    bool ok = true;
    for (uint32_t t = blockIdx.x; ok && t < nrt; t += gridDim.x) {
      float best = FLT_MAX;
      uint32_t arg = 0xFFFFFFFFu;
      for (uint32_t ct = 0; ct < nct; ++ct) {
        if (!__all_sync(0xffffffffu, tc::mbar_wait_or(acc_full + ab, abph, err))) {
          ok = false;
          break;
        }
        tc::fence_after();
        const uint32_t taddr = tmem + (((warp & 3) * 32u) << 16) + ab * kCN;
        for (uint32_t g = 0; g < kCN; g += 16) {
          uint32_t dot[16];
          tc::tmem_ld16(taddr + g, dot);
          tc::tmem_wait_ld();
#pragma unroll
          for (uint32_t j = 0; j < 16; ++j) {
            const uint32_t c = ct * kCN + g + j;
            if (c < A.L) {
              const float v = fmaf(-2.0f, __uint_as_float(dot[j]), __ldg(A.cnorm + c));
              if (v < best) best = v, arg = c;  // ascending c: ties keep the smaller
            }
          }
        }
        tc::fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(acc_empty + ab);
        if (++ab == 2) ab = 0, abph ^= 1;
      }
      if (!ok) break;
      const uint32_t r = t * kRM + row;
      if (r < A.n) {
        A.assign[r] = arg;
        if (A.best) A.best[r] = best;
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (tid == 0 && *err) atomicAdd(A.timeouts, 1u);
  if (warp == 1) tc::tmem_dealloc(tmem, kTmemCols);
}

// |c|^2 per centroid row (one warp per row).
__global__ void row_norms_kernel(const float *__restrict__ x, uint32_t n, uint32_t ld,
                                 float *__restrict__ out) {
  const uint32_t r = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
  if (r >= n) return;
  const float *v = x + static_cast<size_t>(r) * ld;
  float s = 0.0f;
  for (uint32_t k = lane; k < ld; k += 32) s = fmaf(v[k], v[k], s);
#pragma unroll
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[r] = s;
}

// Lloyd update, part 1: per-centroid sums (double) and counts. One warp per row.
__global__ void kmeans_sums_kernel(const float *__restrict__ x, uint32_t n, uint32_t ld,
                                   const uint32_t *__restrict__ assign, double *__restrict__ sums,
                                   uint32_t *__restrict__ counts) {
  const uint32_t r = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
  if (r >= n) return;
  const uint32_t c = assign[r];
  const float *v = x + static_cast<size_t>(r) * ld;
  double *s = sums + static_cast<size_t>(c) * ld;
  for (uint32_t k = lane; k < ld; k += 32) atomicAdd(s + k, static_cast<double>(v[k]));
  if (lane == 0) atomicAdd(counts + c, 1u);
}

// Lloyd update, part 2: the mean of each non-empty cluster (an empty one keeps
// its centre), and the new |c|^2.
__global__ void kmeans_centres_kernel(const double *__restrict__ sums,
                                      const uint32_t *__restrict__ counts, uint32_t L, uint32_t ld,
                                      float *__restrict__ cen, float *__restrict__ cnorm) {
  const uint32_t c = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
  if (c >= L) return;
  const uint32_t m = counts[c];
  float *v = cen + static_cast<size_t>(c) * ld;
  float s = 0.0f;
  for (uint32_t k = lane; k < ld; k += 32) {
    if (m) v[k] = static_cast<float>(sums[static_cast<size_t>(c) * ld + k] / m);
    s = fmaf(v[k], v[k], s);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) cnorm[c] = s;
}

// k-means++: every row's squared distance to centre `m` (a copy of row
// chosen[m]) lowers its running minimum; each block sums its rows' minima in
// a fixed order. One warp per row, kPpRows rows per block.
constexpr uint32_t kPpRows = 64;

__global__ void __launch_bounds__(256) pp_update_kernel(const float *__restrict__ x, uint32_t n,
                                                        uint32_t ld, const float *__restrict__ cen,
                                                        uint32_t m, float *__restrict__ dist,
                                                        double *__restrict__ part) {
  __shared__ float rowd[kPpRows];
  const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x & 31;
  const float *c = cen + static_cast<size_t>(m) * ld;
  for (uint32_t i = warp; i < kPpRows; i += blockDim.x / 32) {
    const uint32_t r = blockIdx.x * kPpRows + i;
    float dv = 0.0f;
    if (r < n) {
      const float *v = x + static_cast<size_t>(r) * ld;
      float s = 0.0f;
      for (uint32_t k = lane; k < ld; k += 32) {
        const float t = v[k] - c[k];
        s = fmaf(t, t, s);
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      dv = m == 0 ? s : fminf(dist[r], s);
      if (lane == 0) dist[r] = dv;
    }
    if (lane == 0) rowd[i] = dv;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (uint32_t i = 0; i < kPpRows; ++i) s += rowd[i];
    part[blockIdx.x] = s;
  }
}

// k-means++: picks centre m + 1 by D^2 sampling (one CTA of 256 threads).
// The block sums are cut into 256 contiguous chunks; the target u[m] * total
// is found in the chunk sums, then in the chosen chunk's block sums, then in
// the chosen block's rows, every sum in a fixed order. A total of zero (every
// row already a centre) takes row m + 1.
__global__ void __launch_bounds__(256) pp_pick_kernel(const float *__restrict__ x, uint32_t n,
                                                      uint32_t ld, const float *__restrict__ dist,
                                                      const double *__restrict__ part,
                                                      uint32_t nblocks, const double *__restrict__ u,
                                                      uint32_t m, uint32_t *__restrict__ chosen,
                                                      float *__restrict__ cen) {
  __shared__ double csum[256];
  __shared__ uint32_t pick;
  const uint32_t per = div_up(nblocks, 256u), b0 = threadIdx.x * per;
  double s = 0.0;
  for (uint32_t b = b0; b < min(nblocks, b0 + per); ++b) s += part[b];
  csum[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double total = 0.0;
    for (uint32_t i = 0; i < 256; ++i) total += csum[i];
    uint32_t r = (m + 1) % n;
    if (total > 0.0) {
      const double dart = u[m] * total;
      double acc = 0.0;
      uint32_t c = 0;
      while (c + 1 < 256 && acc + csum[c] <= dart) acc += csum[c++];
      uint32_t b = min(c * per, nblocks - 1);
      const uint32_t bend = min(nblocks, c * per + per);
      while (b + 1 < bend && acc + part[b] <= dart) acc += part[b++];
      const uint32_t r0 = b * kPpRows, r1 = min(n, r0 + kPpRows);
      r = r1 - 1;
      for (uint32_t i = r0; i < r1; ++i) {
        acc += dist[i];
        if (dart < acc && dist[i] > 0.0f) {
          r = i;
          break;
        }
      }
      // the target may lie past the block's last row with a distance (sums
      // round): take the last row that has one
      while (dist[r] <= 0.0f && r > r0) --r;
    }
    pick = r;
    chosen[m + 1] = r;
  }
  __syncthreads();
  const float *v = x + static_cast<size_t>(pick) * ld;
  float *c = cen + static_cast<size_t>(m + 1) * ld;
  for (uint32_t k = threadIdx.x; k < ld; k += blockDim.x) c[k] = v[k];
}

// dst row i (stride ld, zero-padded past d) = src row rows[i] (stride d).
__global__ void gather_rows_kernel(const float *__restrict__ src, uint32_t d,
                                   const uint32_t *__restrict__ rows, uint32_t m, uint32_t ld,
                                   float *__restrict__ dst) {
  const uint32_t i = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
  if (i >= m) return;
  const float *v = src + static_cast<size_t>(rows[i]) * d;
  float *o = dst + static_cast<size_t>(i) * ld;
  for (uint32_t k = lane; k < ld; k += 32) o[k] = k < d ? v[k] : 0.0f;
}

__global__ void copy_row_kernel(const float *__restrict__ x, uint32_t ld, uint32_t r,
                                float *__restrict__ dst) {
  for (uint32_t k = threadIdx.x; k < ld; k += blockDim.x) dst[k] = x[static_cast<size_t>(r) * ld + k];
}

// Column means of n rows (double), one thread per column.
__global__ void col_mean_kernel(const float *__restrict__ x, uint32_t n, uint32_t ld, uint32_t d,
                                double *__restrict__ mean) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d) return;
  double s = 0.0;
  for (uint32_t r = 0; r < n; ++r) s += x[static_cast<size_t>(r) * ld + k];
  mean[k] = s / n;
}

// Covariance (double): cov[i][j] = sum_r (x_ri - mean_i)(x_rj - mean_j) / n
// over 32 x 32 tiles of (i, j) with j >= i's tile; rows staged 32 at a time.
__global__ void __launch_bounds__(256) cov_kernel(const float *__restrict__ x, uint32_t n,
                                                  uint32_t ld, uint32_t d,
                                                  const double *__restrict__ mean,
                                                  double *__restrict__ cov) {
  const uint32_t ti = blockIdx.y, tj = blockIdx.x;
  if (tj < ti) return;
  __shared__ double a[32][33], b[32][33];
  const uint32_t tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 8 rows of 32
  double acc[4] = {0, 0, 0, 0};
  const uint32_t i0 = ti * 32, j0 = tj * 32;
  for (uint32_t r0 = 0; r0 < n; r0 += 32) {
    for (uint32_t rr = ty; rr < 32; rr += 8) {
      const uint32_t r = r0 + rr;
      const uint32_t ci = i0 + tx, cj = j0 + tx;
      a[rr][tx] = (r < n && ci < d) ? x[static_cast<size_t>(r) * ld + ci] - mean[ci] : 0.0;
      b[rr][tx] = (r < n && cj < d) ? x[static_cast<size_t>(r) * ld + cj] - mean[cj] : 0.0;
    }
    __syncthreads();
    for (uint32_t rr = 0; rr < 32; ++rr)
#pragma unroll
      for (uint32_t q = 0; q < 4; ++q) acc[q] += a[rr][ty + 8 * q] * b[rr][tx];
    __syncthreads();
  }
#pragma unroll
  for (uint32_t q = 0; q < 4; ++q) {
    const uint32_t i = i0 + ty + 8 * q, j = j0 + tx;
    if (i < d && j < d) {
      cov[static_cast<size_t>(i) * d + j] = acc[q] / n;
      cov[static_cast<size_t>(j) * d + i] = acc[q] / n;
    }
  }
}

int encode_rows(CUtensorMap *map, const float *base, uint32_t rows, uint32_t ld, uint32_t box_rows) {
  const PFN_cuTensorMapEncodeTiled_v12000 encode = tc::tensor_map_encoder();
  if (!encode) return cuda_status(cudaErrorNotSupported, "cuTensorMapEncodeTiled");
  const cuuint64_t dims[2] = {ld, rows};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld) * 4};
  const cuuint32_t box[2] = {kKB, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims,
                            strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed for k-means rows (error " + std::to_string(r) + ")");
    return KATO_ERUNTIME;
  }
  return KATO_OK;
}

int check_rows(const void *p, uint32_t ld) {
  if (!p) return invalid("null rows");
  if (ld == 0 || ld % kKB) return invalid("row stride must be a positive multiple of 32 floats");
  if (reinterpret_cast<uintptr_t>(p) % 16) return invalid("rows must be 16-byte aligned");
  return KATO_OK;
}

}  // namespace

int kmeans_assign(const float *x, uint32_t n, uint32_t ld, const float *cen, const float *cnorm,
                  uint32_t L, uint32_t *assign, float *best, uint32_t *timeouts, cudaStream_t st) {
  if (n == 0) return KATO_OK;
  int rc;
  if ((rc = check_rows(x, ld)) || (rc = check_rows(cen, ld))) return rc;
  if (L == 0 || !assign || !cnorm || !timeouts) return invalid("k-means assignment: bad arguments");
  CUtensorMap mx, mc;
  if ((rc = encode_rows(&mx, x, n, ld, kRM)) || (rc = encode_rows(&mc, cen, L, ld, kCN))) return rc;
  int sms = 0;
  if ((rc = current_sms(&sms)) ||
      (rc = smem_limit(reinterpret_cast<const void *>(kmeans_assign_kernel), static_cast<int>(kSmem),
                       "kmeans_assign_kernel shared memory")))
    return rc;
  const AssignArgs A{cnorm, assign, best, n, L, ld, timeouts};
  const uint32_t tiles = div_up(n, kRM);
  kmeans_assign_kernel<<<std::min<uint32_t>(tiles, sms), kThreads, kSmem, st>>>(mx, mc, A);
  KATO_LAUNCHED("kmeans_assign_kernel");
  return KATO_OK;
}

int row_norms(const float *x, uint32_t n, uint32_t ld, float *out, cudaStream_t st) {
  if (n == 0) return KATO_OK;
  row_norms_kernel<<<div_up(n, 8), 256, 0, st>>>(x, n, ld, out);
  KATO_LAUNCHED("row_norms_kernel");
  return KATO_OK;
}

int kmeans_update(const float *x, uint32_t n, uint32_t ld, const uint32_t *assign, uint32_t L,
                  double *sums, uint32_t *counts, float *cen, float *cnorm, cudaStream_t st) {
  KATO_CUDA(cudaMemsetAsync(sums, 0, static_cast<size_t>(L) * ld * sizeof(double), st));
  KATO_CUDA(cudaMemsetAsync(counts, 0, static_cast<size_t>(L) * sizeof(uint32_t), st));
  if (n) kmeans_sums_kernel<<<div_up(n, 8), 256, 0, st>>>(x, n, ld, assign, sums, counts);
  kmeans_centres_kernel<<<div_up(L, 8), 256, 0, st>>>(sums, counts, L, ld, cen, cnorm);
  KATO_LAUNCHED("k-means update kernels");
  return KATO_OK;
}

size_t kmeanspp_scratch(uint32_t n) { return static_cast<size_t>(div_up(n, kPpRows)) * sizeof(double); }

int kmeanspp(const float *x, uint32_t n, uint32_t ld, uint32_t L, uint32_t first, const double *u,
             float *cen, float *dist, double *part, uint32_t *chosen, cudaStream_t st) {
  if (n == 0 || L == 0 || L > n || first >= n) return invalid("k-means++: need 1 <= nlist <= rows");
  copy_row_kernel<<<1, 256, 0, st>>>(x, ld, first, cen);
  KATO_CUDA(cudaMemcpyAsync(chosen, &first, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  const uint32_t nb = div_up(n, kPpRows);
  for (uint32_t m = 0; m + 1 < L; ++m) {
    pp_update_kernel<<<nb, 256, 0, st>>>(x, n, ld, cen, m, dist, part);
    pp_pick_kernel<<<1, 256, 0, st>>>(x, n, ld, dist, part, nb, u, m, chosen, cen);
  }
  KATO_LAUNCHED("k-means++ kernels");
  return KATO_OK;
}

int gather_rows(const float *src, uint32_t d, const uint32_t *rows, uint32_t m, uint32_t ld,
                float *dst, cudaStream_t st) {
  if (m == 0) return KATO_OK;
  gather_rows_kernel<<<div_up(m, 8), 256, 0, st>>>(src, d, rows, m, ld, dst);
  KATO_LAUNCHED("gather_rows_kernel");
  return KATO_OK;
}

int covariance(const float *x, uint32_t n, uint32_t ld, uint32_t d, double *mean, double *cov,
               cudaStream_t st) {
  if (n == 0 || d == 0) return invalid("covariance of an empty sample");
  col_mean_kernel<<<div_up(d, 256), 256, 0, st>>>(x, n, ld, d, mean);
  const dim3 grid(div_up(d, 32), div_up(d, 32));
  cov_kernel<<<grid, 256, 0, st>>>(x, n, ld, d, mean, cov);
  KATO_LAUNCHED("covariance kernels");
  return KATO_OK;
}

}  // namespace kato
