// Coarse product on the 5th-generation tensor cores.
//
// The reference's coarse step scores every query against every centroid with
// the exact SQ16 distance (coarse_batched_sq16_, src/index.cpp:846-877, over
// sq16_l2, src/kernels.cpp:187-214): q.x = 65536 (qh.xh) + 256 (qh.xl +
// ql.xh) + ql.xl over the dc bytes of each plane. Here the four byte-plane
// products run as fp16 GEMMs: every byte b is re-centred to b - 128 (exact in
// fp16), so each product is at most 2^14 and a sum over up to 1024 dimensions
// is an exact integer in the fp32 accumulator. With a = b - 128,
//   sum x y = sum a_x a_y + 128 (sum a_x + sum a_y) + 16384 dc,
// so the squared L2 is
//   l2 = T_q + T_c - 2 (65536 HH + 256 (HL + LH) + LL)
// with HH.. the centred products and T a per-row term (centre_planes_kernel).
//
// coarse_tc_kernel: persistent CTAs over (128 centroids x 64 queries) tiles.
// A TMA thread loads 64-dimension slices of the four centred planes (128-byte
// swizzle) into a ring of stages; the query tiles of the high and the low
// plane sit back to back, so they form one 128-row B operand. One MMA thread
// issues two MMAs per 16-dimension step (M = 128 centroids, N = 128: the
// queries' high and low rows, K = 16): the centroids' high plane against both
// gives HH and HL, their low plane against both gives LH and LL, into a
// double-buffered set of four TMEM accumulators (an MMA of N = 128 issues in
// about the time of one of N = 64, so two wide MMAs take 27% less time than
// four narrow ones). Sixteen epilogue warps (thread = centroid row) rebuild
// each l2 exactly in 64-bit integers and write the reference's float distance
// (dist_value), 32 consecutive centroids per warp store.
//
// Rows wider than 1024 dimensions (the reference takes any dc up to kMaxDim
// = 4096, include/katoann/kernels.h:177) are split into chunks of at most
// 1024 dimensions. Each chunk is accumulated on its own in a TMEM slot, so
// each chunk's sums stay exact in fp32; the epilogue drains every chunk and
// adds the chunks' products in 64-bit integers before it writes a distance.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>

#include "kcommon.cuh"
#include "tc.cuh"

namespace kato {

namespace {

constexpr uint32_t kCM = 128;     // centroids per tile (the MMA's M)
constexpr uint32_t kQN = 64;      // queries per tile (the MMA's N)
constexpr uint32_t kBK = 64;      // dimensions per stage (128 bytes of fp16)
constexpr uint32_t kStages = 4;
constexpr uint32_t kChunkSlices = 1024 / kBK;  // 64-dimension slices per exact chunk
constexpr uint32_t kATile = kCM * kBK * 2;  // 16 KiB
constexpr uint32_t kBTile = kQN * kBK * 2;  // 8 KiB
constexpr uint32_t kStage = 2 * kATile + 2 * kBTile;
// the two query tiles form one B operand of 2 kQN rows: each starts on a
// 1 KiB boundary (the swizzle pattern), and an MMA's N is at most 256
static_assert(kATile % 1024 == 0 && kBTile % 1024 == 0 && 2 * kQN <= 256, "paired B operand");
constexpr uint32_t kAccCols = 4 * kQN;      // HH, HL, LH, LL
constexpr uint32_t kTmemCols = 2 * kAccCols;
constexpr int kEpiWarps = 16;  // four per TMEM lane quarter, 16 query columns each
constexpr int kThreads = (2 + kEpiWarps) * 32;  // TMA warp, MMA warp, epilogue
constexpr uint32_t kSmem = kStages * kStage + 2048;  // + alignment slack and barriers

// Shared-memory descriptor of a K-major operand tile in the 128-byte swizzled
// layout: rows of 128 bytes, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr) {
  return static_cast<uint64_t>((addr & 0x3FFFFu) >> 4) | (1ull << 16) | (64ull << 32) |
         (1ull << 46) | (2ull << 61);
}

// Per row of a plane pair: the fp16 centred planes and
//   T = norm - 256 (65792 s_h + 257 s_l) - 16384 dc 66049,
// s = sum over the row of (byte - 128). One warp per row.
__global__ void __launch_bounds__(256) centre_planes_kernel(
    const uint8_t *__restrict__ hi, const uint8_t *__restrict__ lo, const int64_t *__restrict__ norm,
    uint32_t rows, uint32_t dc, __half *__restrict__ hi16, __half *__restrict__ lo16,
    int64_t *__restrict__ term) {
  const uint32_t row = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (row >= rows) return;
  const __half2 bias = __floats2half2_rn(1152.0f, 1152.0f);
  int32_t sh = 0, sl = 0;
  for (uint32_t u = lane; u < dc / 16; u += 32) {
    const size_t at = static_cast<size_t>(row) * dc + u * 16;
    const uint4 vh = *reinterpret_cast<const uint4 *>(hi + at);
    const uint4 vl = *reinterpret_cast<const uint4 *>(lo + at);
    uint4 a, b;
    tc::bytes_to_half16(vh, bias, a, b);
    *reinterpret_cast<uint4 *>(hi16 + at) = a;
    *reinterpret_cast<uint4 *>(hi16 + at + 8) = b;
    tc::bytes_to_half16(vl, bias, a, b);
    *reinterpret_cast<uint4 *>(lo16 + at) = a;
    *reinterpret_cast<uint4 *>(lo16 + at + 8) = b;
    sh += static_cast<int32_t>(dp4(vh.x, 0x01010101u, dp4(vh.y, 0x01010101u, dp4(vh.z, 0x01010101u, dp4(vh.w, 0x01010101u, 0))))) - 2048;
    sl += static_cast<int32_t>(dp4(vl.x, 0x01010101u, dp4(vl.y, 0x01010101u, dp4(vl.z, 0x01010101u, dp4(vl.w, 0x01010101u, 0))))) - 2048;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    sh += __shfl_xor_sync(0xffffffffu, sh, o);
    sl += __shfl_xor_sync(0xffffffffu, sl, o);
  }
  if (lane == 0)
    term[row] = norm[row] - 256 * (65792ll * sh + 257ll * sl) - 16384ll * dc * 66049ll;
}

struct CoarseArgs {
  const int64_t *cterm, *qterm;
  float *out;  // m x n
  uint32_t m, n, dc;
  DistScale scale;
  uint32_t *timeouts;
  unsigned long long *prof;  // optional: TMA wait/total, MMA waits/total, epilogue wait/total
};

__device__ __forceinline__ bool cwait(uint64_t *b, uint32_t ph, volatile uint32_t *err,
                                      unsigned long long &acc) {
  const long long t = clock64();
  const bool ok = tc::mbar_wait_or(b, ph, err);
  acc += clock64() - t;
  return ok;
}

__global__ void __launch_bounds__(kThreads, 1)
    coarse_tc_kernel(const __grid_constant__ CUtensorMap tch, const __grid_constant__ CUtensorMap tcl,
                     const __grid_constant__ CUtensorMap tqh, const __grid_constant__ CUtensorMap tql,
                     const CoarseArgs A) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  // 1 KiB-aligned stages (the swizzle pattern repeats every 1024 bytes)
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
  const uint32_t nct = (A.n + kCM - 1) / kCM, nqt = (A.m + kQN - 1) / kQN;
  const uint32_t ntiles = nct * nqt, nk = A.dc / kBK;
  unsigned long long pw[2] = {0, 0};
  const long long tstart = clock64();

  if (warp == 0) {
    // ---- TMA producer
    if (lane == 0) {
      uint32_t s = 0, ph = 0, issued = 0, last_par[kStages] = {};
      for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int32_t c0 = static_cast<int32_t>((t % nct) * kCM), q0 = static_cast<int32_t>((t / nct) * kQN);
        bool ok = true;
        for (uint32_t k = 0; k < nk; ++k) {
          if (!cwait(empty + s, ph ^ 1, err, pw[0])) {
            ok = false;
            break;
          }
          unsigned char *st = sm + s * kStage;
          const int32_t x = static_cast<int32_t>(k * kBK);
          tc::mbar_expect_tx(full + s, kStage);
          tc::tma_load_2d(st, &tch, x, c0, full + s);
          tc::tma_load_2d(st + kATile, &tcl, x, c0, full + s);
          tc::tma_load_2d(st + 2 * kATile, &tqh, x, q0, full + s);
          tc::tma_load_2d(st + 2 * kATile + kBTile, &tql, x, q0, full + s);
          issued |= 1u << s;
          last_par[s] = ph;
          if (++s == kStages) s = 0, ph ^= 1;
        }
        if (!ok) break;
      }
      if (*err)  // copies still in flight land before the CTA exits
        for (uint32_t i = 0; i < kStages; ++i)
          if (issued >> i & 1u) tc::mbar_wait(full + i, last_par[i]);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---- MMA issuer: per 16-dimension step, [HH | HL] and [LH | LL]
    if (lane == 0) {
      const uint32_t idesc = tc::idesc_f16(kCM, 2 * kQN);
      uint32_t s = 0, ph = 0, ab = 0, abph = 0;
      bool ok = true;
      for (uint32_t t = blockIdx.x; ok && t < ntiles; t += gridDim.x) {
        // one accumulator slot per chunk of at most 1024 dimensions
        for (uint32_t k0 = 0; ok && k0 < nk; k0 += kChunkSlices) {
          if (!cwait(acc_empty + ab, abph ^ 1, err, pw[0])) {
            ok = false;
            break;
          }
          tc::fence_after();
          const uint32_t d0 = tmem + ab * kAccCols;
          const uint32_t k1 = min(nk, k0 + kChunkSlices);
          for (uint32_t k = k0; k < k1; ++k) {
            if (!cwait(full + s, ph, err, pw[1])) {
              ok = false;
              break;
            }
            tc::fence_after();
            const uint32_t st = tc::smem_addr(sm + s * kStage);
            const uint64_t ah = desc_sw128(st), al = desc_sw128(st + kATile);
            // the high-plane query tile (64 rows) is followed by the low-plane
            // one at the next 1 KiB boundary, in the same swizzle: one operand
            // of 128 rows, 8-row groups 1024 bytes apart
            const uint64_t b = desc_sw128(st + 2 * kATile);
#pragma unroll
            for (uint32_t j = 0; j < kBK / 16; ++j) {
              const uint32_t acc = (k != k0 || j != 0);
              // a 16-dimension step is 32 bytes along the swizzled row: +2 encoded
              tc::mma_f16(d0 + 0 * kQN, ah + 2 * j, b + 2 * j, idesc, acc);  // HH, HL
              tc::mma_f16(d0 + 2 * kQN, al + 2 * j, b + 2 * j, idesc, acc);  // LH, LL
            }
            tc::commit(empty + s);
            if (++s == kStages) s = 0, ph ^= 1;
          }
          if (!ok) break;
          tc::commit(acc_full + ab);
          if (++ab == 2) ab = 0, abph ^= 1;
        }
      }
      // every MMA issued has completed before tensor memory is released
      tc::commit(done);
      tc::mbar_wait(done, 0);
    }
    __syncwarp();
  } else {
    // ---- epilogue: thread = centroid row (its TMEM lane); the four warps of
    // a lane quarter take 16 query columns each
    const uint32_t q4 = warp & 3, part = (warp - 2) >> 2;
    const uint32_t row = q4 * 32 + lane;
    const uint32_t nchunks = div_up(nk, kChunkSlices);
    uint32_t ab = 0, abph = 0;
    bool ok = true;
    for (uint32_t t = blockIdx.x; ok && t < ntiles; t += gridDim.x) {
      const uint32_t c = (t % nct) * kCM + row, qb = (t / nct) * kQN + part * 16;
      const int64_t ct = c < A.n ? A.cterm[c] : 0;
      // lane j < 16 holds query qb + j's term; the pairs take it by shuffle
      const int64_t qt_lane = (lane < 16 && qb + lane < A.m) ? A.qterm[qb + lane] : 0;
      // the centred cross product of each query column, summed over the chunks
      int64_t p[16];
#pragma unroll
      for (uint32_t j = 0; j < 16; ++j) p[j] = 0;
      for (uint32_t ch = 0; ch < nchunks; ++ch) {
        if (!__all_sync(0xffffffffu, cwait(acc_full + ab, abph, err, pw[0]))) {
          ok = false;
          break;
        }
        tc::fence_after();
        const uint32_t taddr = tmem + ((q4 * 32u) << 16) + ab * kAccCols + part * 16;
        // columns: HH (centroid high x query high), HL, LH, LL
        uint32_t hh[16], hl[16], lh[16], ll[16];
        tc::tmem_ld16(taddr + 0 * kQN, hh);
        tc::tmem_ld16(taddr + 1 * kQN, hl);
        tc::tmem_ld16(taddr + 2 * kQN, lh);
        tc::tmem_ld16(taddr + 3 * kQN, ll);
        tc::tmem_wait_ld();
#pragma unroll
        for (uint32_t j = 0; j < 16; ++j)
          p[j] += 65536ll * __float2int_rn(__uint_as_float(hh[j])) +
                  256ll * (__float2int_rn(__uint_as_float(hl[j])) +
                           __float2int_rn(__uint_as_float(lh[j]))) +
                  __float2int_rn(__uint_as_float(ll[j]));
        // the slot has been read: hand it back for the next chunk or tile
        tc::fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(acc_empty + ab);
        if (++ab == 2) ab = 0, abph ^= 1;
      }
      if (!ok) break;
#pragma unroll
      for (uint32_t j = 0; j < 16; ++j) {
        const uint32_t q = qb + j;
        const int64_t qt = __shfl_sync(0xffffffffu, qt_lane, j);
        if (q >= A.m || c >= A.n) continue;
        A.out[static_cast<size_t>(q) * A.n + c] = dist_value(qt + ct - 2 * p[j], A.scale);
      }
    }
  }
  if (A.prof && lane == 0 && warp <= 2) {
    // slots: TMA wait, total; MMA wait for accumulators, for stages, total;
    // first epilogue warp wait, total
    const int base = warp == 0 ? 0 : warp == 1 ? 2 : 5;
    const int nw = warp == 1 ? 2 : 1;
    for (int i = 0; i < nw; ++i) atomicAdd(A.prof + base + i, pw[i]);
    atomicAdd(A.prof + base + nw, static_cast<unsigned long long>(clock64() - tstart));
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (tid == 0 && *err) atomicAdd(A.timeouts, 1u);
  if (warp == 1) tc::tmem_dealloc(tmem, kTmemCols);
}

int encode_plane(CUtensorMap *map, const __half *base, uint32_t rows, uint32_t dc, uint32_t box_rows) {
  const PFN_cuTensorMapEncodeTiled_v12000 encode = tc::tensor_map_encoder();
  if (!encode) return cuda_status(cudaErrorNotSupported, "cuTensorMapEncodeTiled");
  const cuuint64_t dims[2] = {dc, rows};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(dc) * 2};
  const cuuint32_t box[2] = {kBK, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<__half *>(base), dims,
                            strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed for a coarse plane (error " + std::to_string(r) + ")");
    return KATO_ERUNTIME;
  }
  return KATO_OK;
}

}  // namespace

int centre_planes(const uint8_t *hi, const uint8_t *lo, const int64_t *norm, uint32_t rows,
                  uint32_t dc, __half *hi16, __half *lo16, int64_t *term, cudaStream_t st) {
  if (rows == 0) return KATO_OK;
  if (dc == 0 || dc % 64) return invalid("dc must be a positive multiple of 64");
  centre_planes_kernel<<<div_up(rows, 8), 256, 0, st>>>(hi, lo, norm, rows, dc, hi16, lo16, term);
  KATO_LAUNCHED("centre_planes_kernel");
  return KATO_OK;
}

bool coarse_tc_ok(uint32_t dc) { return dc >= kBK && dc % kBK == 0 && dc <= 4096; }

int coarse_tc(const __half *ch, const __half *cl, const int64_t *cterm, uint32_t n, const __half *qh,
              const __half *ql, const int64_t *qterm, uint32_t m, uint32_t dc, double step_sq,
              float *out, uint32_t *timeouts, unsigned long long *prof, cudaStream_t st) {
  if (m == 0 || n == 0) return KATO_OK;
  if (!coarse_tc_ok(dc)) return invalid("the tensor-core coarse product needs dc in [64, 4096], a multiple of 64");
  CUtensorMap mch, mcl, mqh, mql;
  int rc;
  if ((rc = encode_plane(&mch, ch, n, dc, kCM)) || (rc = encode_plane(&mcl, cl, n, dc, kCM)) ||
      (rc = encode_plane(&mqh, qh, m, dc, kQN)) || (rc = encode_plane(&mql, ql, m, dc, kQN)))
    return rc;
  int sms = 0;
  if ((rc = current_sms(&sms)) ||
      (rc = smem_limit(reinterpret_cast<const void *>(coarse_tc_kernel), static_cast<int>(kSmem),
                       "coarse_tc_kernel shared memory")))
    return rc;
  const CoarseArgs A{cterm, qterm, out, m, n, dc, make_dist_scale(step_sq), timeouts, prof};
  const uint32_t ntiles = div_up(n, kCM) * div_up(m, kQN);
  coarse_tc_kernel<<<std::min<uint32_t>(ntiles, sms), kThreads, kSmem, st>>>(mch, mcl, mqh, mql, A);
  KATO_LAUNCHED("coarse_tc_kernel");
  return KATO_OK;
}

}  // namespace kato
