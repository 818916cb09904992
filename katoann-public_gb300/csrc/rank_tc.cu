// Ranking pass on the 5th-generation tensor cores.
//
// The reference scores every row of every probed list against the queries
// that probe it with the high bytes of the leading h rotated dimensions
// (sq16_high_l2, src/kernels.cpp:216-243, called from src/index.cpp:1016-1042)
// and keeps each query's best S by (distance, id) (:63-97 / :101-135). Here:
//   1. rank_seed_kernel gives every query an upper bound on its final S-th
//      ranking l2: the S-th smallest one over the first rows of its nearest
//      lists (any S of its candidates bound its S-th best from above), widened
//      so that every l2 with the same float distance stays inside;
//   2. rank_tc_kernel scores (row, query) pairs on the tensor cores. Work
//      items are (list, up to N of the queries probing it); each of a list's
//      128-row tiles is scored against the item's queries. One CTA per SM
//      takes an equal share of all tiles and runs them through a pipeline of
//      warp roles connected by mbarriers:
//        - a TMA thread loads raw tiles of high bytes (128 rows x 128 bytes,
//          128-byte swizzle) into a ring of stages;
//        - two staging warps gather each item's query rows, re-centred to
//          (byte - 128) as exact fp16, into a double-buffered B tile in the
//          canonical K-major layout, with each query's bound;
//        - eight converter warps (two threads per row) re-centre the raw tiles
//          to fp16 and store them into tensor memory (the A operand, two
//          stages) with tcgen05.st, and sum each row's centred norm xn';
//        - one MMA thread issues tcgen05.mma (M = 128 rows, N queries, K = 16)
//          into double-buffered fp32 TMEM accumulators. Products are at most
//          128 * 128, so up to 1024 dimensions add up exactly;
//        - eight epilogue warps (thread = row, each warpgroup half of the
//          columns) test l2 = qn' + xn' - 2 dot' against the query's bound
//          (translating both vectors by 128 leaves every squared distance
//          unchanged) and append passing (query, l2, row) records to the
//          CTA's list; tc_bucket_kernel then sorts the records into per-query
//          buffers with their float distances;
//   3. a query whose buffer overflowed is rescanned exactly (rescan_*
//      kernels), and the merge kernel takes the exact best S by (distance, id)
//      from each buffer, so results never depend on the bound or the buffer
//      size.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <type_traits>
#include <climits>
#include <cmath>

#include "kcommon.cuh"
#include "rank_tc.cuh"
#include "scan.cuh"
#include "tc.cuh"

namespace kato {

namespace {

constexpr uint32_t kSeedCap = 4096;  // rows a seed bound looks at, at most

// Warp roles of rank_tc_kernel.
constexpr int kConvWarps = 8, kEpiWarps = 8, kQueryWarps = 2;
constexpr int kTmaWarp = kConvWarps + kEpiWarps;  // 16
constexpr int kMmaWarp = kTmaWarp + 1;             // 17
constexpr int kQueryWarp0 = kMmaWarp + 1;          // 18, 19
constexpr int kTcThreads = (kQueryWarp0 + kQueryWarps) * 32;
constexpr uint32_t kDropped = 0x80000000u;  // qcount flag: a record did not fit

struct QInfo {
  uint32_t qid;
  int32_t qn;   // centred norm of the query's ranking bytes
  int32_t qb;   // bound - qn: a row is a candidate iff xn' - 2 dot' <= qb
  float qbf;    // qb as float (exact below 2^24; beyond, every row passes anyway)
};
static_assert(sizeof(QInfo) == kTcQInfo, "query slot size");

struct Bars {
  uint64_t *raw_full, *raw_empty, *a_full, *a_empty, *b_full, *b_empty, *acc_full, *acc_empty,
      *xn_full, *done;
};

// Barrier slots in order: raw full/empty (4 each, at most), A full/empty,
// query buffers full/empty (2 each, at most), accumulators full/empty, row
// norms full, done.
__device__ __forceinline__ Bars bars_at(unsigned char *sm, const TcSmem &L) {
  uint64_t *b = reinterpret_cast<uint64_t *>(sm + L.bars);
  uint64_t *a = b + 8, *q = a + 2 * kTcAStages, *c = q + 4;
  return Bars{b, b + 4, a, a + kTcAStages, q, q + 2, c, c + kTcAcc, c + 2 * kTcAcc, c + 3 * kTcAcc};
}

// sum over 16 bytes of (b - 128)^2 = sum b^2 - 256 sum b + 16 * 16384
__device__ __forceinline__ int32_t centred_sq_sum16(uint4 v) {
  const uint32_t s2 = dp4(v.x, v.x, dp4(v.y, v.y, dp4(v.z, v.z, dp4(v.w, v.w, 0))));
  const uint32_t s1 =
      dp4(v.x, 0x01010101u, dp4(v.y, 0x01010101u, dp4(v.z, 0x01010101u, dp4(v.w, 0x01010101u, 0))));
  return static_cast<int32_t>(s2) - 256 * static_cast<int32_t>(s1) + 16 * 16384;
}

// Walk over this CTA's tiles [t0, t1) and the items they belong to; the next
// item's description is loaded one item ahead.
struct TileWalk {
  const uint32_t *tile_off;
  const TcItem *items;
  uint32_t nitems, t0, t1, t, item, start, next, next2;
  TcItem cur, nxt;
  __device__ void init(const uint32_t *to, const TcItem *it, uint32_t n, uint32_t a, uint32_t b) {
    tile_off = to;
    items = it;
    nitems = n;
    t0 = a;
    t1 = b;
    t = a;
    uint32_t lo = 0, hi = n;  // tile_off[lo] <= a < tile_off[hi]
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) / 2;
      if (tile_off[mid] <= a) lo = mid;
      else hi = mid;
    }
    item = lo;
    start = tile_off[lo];
    next = tile_off[lo + 1];
    next2 = lo + 2 <= n ? tile_off[lo + 2] : 0xFFFFFFFFu;
    cur = items[lo];
    nxt = lo + 1 < n ? items[lo + 1] : cur;
  }
  // Called at the top of each tile.
  __device__ void step() {
    if (t == next) {
      ++item;
      start = next;
      next = next2;
      cur = nxt;
      next2 = item + 2 <= nitems ? tile_off[item + 2] : 0xFFFFFFFFu;
      nxt = item + 1 < nitems ? items[item + 1] : cur;
    }
  }
  __device__ bool first() const { return t == t0 || t == start; }
  __device__ bool last() const { return t + 1 == t1 || t + 1 == next; }
};

// The MMA width (queries) an item of ne queries uses: 16, 32 or N.
template <uint32_t N>
__device__ __forceinline__ uint32_t mma_width(uint32_t ne) {
  return ne <= 16 ? 16u : (ne <= 32 && N > 32 ? 32u : N);
}

// A pipeline wait that also adds the cycles it took to `acc`.
__device__ __forceinline__ bool timed_wait(uint64_t *b, uint32_t phase, volatile uint32_t *err,
                                           unsigned long long &acc, long long limit) {
  const long long t = clock64();
  const bool ok = tc::mbar_wait_or(b, phase, err, limit);
  acc += clock64() - t;
  return ok;
}

template <uint32_t N, bool kFloat>
__global__ void __launch_bounds__(kTcThreads, 1)
    rank_tc_kernel(const __grid_constant__ CUtensorMap tmap, const RankTcArgs A, const TcShape S) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const uint32_t h = A.h;
  const TcSmem L = tc_smem_layout(h, S);
  const Bars bar = bars_at(sm, L);
  volatile uint32_t *err = reinterpret_cast<volatile uint32_t *>(sm + L.err);
  uint32_t *tbase = reinterpret_cast<uint32_t *>(sm + L.tbase);
  uint32_t *rcount = reinterpret_cast<uint32_t *>(sm + L.rcount);
  int32_t *sxn = reinterpret_cast<int32_t *>(sm + L.sxn);
  QInfo *qinfo = reinterpret_cast<QInfo *>(sm + L.qinfo);
  uint32_t *swidth = reinterpret_cast<uint32_t *>(sm + L.width);  // per query buffer: queries
  const uint32_t btile = N * h * 2, rtile = kTcRows * S.inner;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    for (uint32_t s = 0; s < S.Rs; ++s) {
      tc::mbar_init(bar.raw_full + s, 1);
      tc::mbar_init(bar.raw_empty + s, kConvWarps);
    }
    for (uint32_t s = 0; s < kTcAStages; ++s) {
      tc::mbar_init(bar.a_full + s, kConvWarps);
      tc::mbar_init(bar.a_empty + s, 1);
    }
    for (uint32_t s = 0; s < kTcAcc; ++s) {
      tc::mbar_init(bar.acc_full + s, 1);
      tc::mbar_init(bar.acc_empty + s, kEpiWarps);
      tc::mbar_init(bar.xn_full + s, kConvWarps);
    }
    for (uint32_t s = 0; s < S.Bs; ++s) {
      tc::mbar_init(bar.b_full + s, kQueryWarps);
      tc::mbar_init(bar.b_empty + s, 1 + kEpiWarps);
    }
    tc::mbar_init(bar.done, 1);
    *rcount = 0;
    // the TMA swizzle pattern repeats every 1024 bytes of shared address
    *err = (tc::smem_addr(sm + L.raw) & 1023u) ? 2u : 0u;
    tc::fence_barrier_init();
  }
  if (warp == kMmaWarp) tc::tmem_alloc(tbase, S.tcols);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tbase;
  const uint32_t acol = kTcAcc * N;  // TMEM columns of the A stages follow the accumulators
  const uint32_t nitems = *A.nitems;
  const uint32_t T = nitems ? A.tile_off[nitems] : 0;
  uint32_t t0, t1;
  if (A.cost_off && nitems) {
    // an equal share of the cost; cost unit c lies in tile tile_at(c)
    const uint32_t C = A.cost_off[nitems];
    auto tile_at = [&](uint32_t c) -> uint32_t {
      if (c >= C) return T;
      uint32_t lo = 0, hi = nitems;  // cost_off[lo] <= c < cost_off[hi]
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (A.cost_off[mid] <= c) lo = mid;
        else hi = mid;
      }
      const uint32_t tiles = A.tile_off[lo + 1] - A.tile_off[lo];
      const uint32_t per = (A.cost_off[lo + 1] - A.cost_off[lo]) / tiles;
      return A.tile_off[lo] + (c - A.cost_off[lo]) / per;
    };
    t0 = tile_at(static_cast<uint32_t>(static_cast<uint64_t>(C) * blockIdx.x / gridDim.x));
    t1 = tile_at(static_cast<uint32_t>(static_cast<uint64_t>(C) * (blockIdx.x + 1) / gridDim.x));
  } else {
    t0 = static_cast<uint32_t>(static_cast<uint64_t>(T) * blockIdx.x / gridDim.x);
    t1 = static_cast<uint32_t>(static_cast<uint64_t>(T) * (blockIdx.x + 1) / gridDim.x);
  }
  const uint32_t nkc = (h + S.inner - 1) / S.inner;
  const __half2 bias = __floats2half2_rn(1152.0f, 1152.0f);  // 1024 + 128
  // per-role cycle profile (first thread of each role): waits, then total
  unsigned long long pw[3] = {0, 0, 0};
  const long long tstart = clock64();

  if (t0 < t1 && !*err) {
    TileWalk w;
    w.init(A.tile_off, A.items, nitems, t0, t1);
    if (warp < kConvWarps) {
      // ---- converters: raw stage -> fp16 A stage and the row's centred
      // norm; two threads per row, each half of every chunk's 16-byte columns
      const uint32_t r = tid & (kTcRows - 1), hf = tid >> 7, swm = S.inner == 128 ? 7u : 3u;
      const uint32_t nuh = S.inner / 32;  // 16-byte columns per half of a full chunk
      uint32_t rs = 0, rph = 0, as = 0, aph = 0, ab = 0, abph = 0;
      bool ok = true;
      for (; ok && w.t < t1; ++w.t) {
        int32_t xs = 0;
        for (uint32_t kc = 0; kc < nkc; ++kc) {
          // warp-uniform waits: a warp arrives once for all its lanes below
          if (!__all_sync(0xffffffffu, timed_wait(bar.raw_full + rs, rph, err, pw[0], A.wait) &&
                                           timed_wait(bar.a_empty + as, aph ^ 1, err, pw[1], A.wait))) {
            ok = false;
            break;
          }
          tc::fence_after();  // the MMAs that read A stage `as` before have completed
          const unsigned char *raw = sm + L.raw + rs * rtile;
          const uint32_t nu = min(S.inner, h - kc * S.inner) / 16;
          // the row's half of the chunk as fp16 pairs: 16 dimensions = 8 columns
          uint32_t cols[32];
#pragma unroll
          for (uint32_t i = 0; i < 4; ++i) {
            const uint32_t u = hf * nuh + i;
            uint4 lo = make_uint4(0, 0, 0, 0), hi = lo;
            if (i < nuh && u < nu) {
              const uint32_t o = r * S.inner + u * 16;
              const uint4 v = *reinterpret_cast<const uint4 *>(raw + (o ^ (((o >> 7) & swm) << 4)));
              tc::bytes_to_half16(v, bias, lo, hi);
              xs += centred_sq_sum16(v);
            }
            cols[8 * i + 0] = lo.x, cols[8 * i + 1] = lo.y, cols[8 * i + 2] = lo.z, cols[8 * i + 3] = lo.w;
            cols[8 * i + 4] = hi.x, cols[8 * i + 5] = hi.y, cols[8 * i + 6] = hi.z, cols[8 * i + 7] = hi.w;
          }
          __syncwarp();
          if (lane == 0) tc::mbar_arrive(bar.raw_empty + rs);  // the raw stage has been read
          // into this row's TMEM lane: A stage `as`, the half's columns
          if (hf * nuh < nu) {
            const uint32_t taddr =
                tmem + (((warp & 3) * 32u) << 16) + acol + as * (S.inner / 2) + hf * nuh * 8;
            if (nuh == 4) tc::tmem_st32(taddr, cols);
            else tc::tmem_st16(taddr, *reinterpret_cast<const uint32_t(*)[16]>(cols));
          }
          tc::tmem_wait_st();
          tc::fence_before();
          __syncwarp();
          if (lane == 0) tc::mbar_arrive(bar.a_full + as);
          if (++rs == S.Rs) rs = 0, rph ^= 1;
          if (++as == kTcAStages) as = 0, aph ^= 1;
        }
        if (!ok) break;
        // the row norms of this tile's accumulator slot, once the epilogue
        // has finished with the slot's previous tile
        if (!__all_sync(0xffffffffu, timed_wait(bar.acc_empty + ab, abph ^ 1, err, pw[1], A.wait))) break;
        sxn[(ab * 2 + hf) * kTcRows + r] = xs;
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(bar.xn_full + ab);
        if (++ab == kTcAcc) ab = 0, abph ^= 1;
      }
    } else if (warp < kTmaWarp) {
      // ---- epilogue: thread = row (its TMEM lane), warpgroup = column half
      constexpr uint32_t CH = N / 2;  // columns per half
      const uint32_t q4 = warp & 3, half = (warp - kConvWarps) >> 2;
      const uint32_t row = q4 * 32 + lane;
      uint32_t cph = CH, c0 = half * CH;  // columns per half and this half's first, per item
      uint4 *rec = A.rec + static_cast<size_t>(blockIdx.x) * A.rec_cap;
      uint32_t ab = 0, abph = 0, ib = 0, bph = 0;
      unsigned long long tiles = 0, found = 0;
      const uint32_t *qbv = reinterpret_cast<const uint32_t *>(sm + L.qbv);
      for (; w.t < t1; ++w.t) {
        w.step();
        const QInfo *qi = qinfo + ib * N;
        // waits are made warp-uniform: the warp-collective steps below need all lanes
        if (w.first()) {
          if (!__all_sync(0xffffffffu, timed_wait(bar.b_full + ib, bph, err, pw[0], A.wait))) break;
          cph = mma_width<N>(swidth[ib]) / 2;
          c0 = half * cph;
        }
        const uint32_t rin = (w.t - w.start) * kTcRows + row;
        const bool valid = rin < w.cur.nrows;
        const uint32_t grow = w.cur.row0 + rin;
        if (!__all_sync(0xffffffffu, timed_wait(bar.acc_full + ab, abph, err, pw[1], A.wait) &&
                                         timed_wait(bar.xn_full + ab, abph, err, pw[1], A.wait)))
          break;
        tc::fence_after();
        const int32_t xn = sxn[ab * 2 * kTcRows + row] + sxn[(ab * 2 + 1) * kTcRows + row];
        const uint32_t taddr = tmem + ((q4 * 32u) << 16) + ab * N;
        const float xnf = static_cast<float>(xn);
        // this warpgroup's columns: half of the item's MMA width. In groups
        // of up to 16: load the group's accumulators and bounds, compare each
        // pair (or-ed into one predicate), and resolve the columns only when
        // the warp has a passing pair (rare)
        auto process = [&](auto gsize, uint32_t g) {
          constexpr uint32_t G = decltype(gsize)::value;
          uint32_t d[G], qb[G];
          if constexpr (G == 16) tc::tmem_ld16(taddr + c0 + g, d);
          else tc::tmem_ld8(taddr + c0 + g, d);
#pragma unroll
          for (uint32_t j = 0; j < G; j += 4)
            *reinterpret_cast<uint4 *>(qb + j) =
                *reinterpret_cast<const uint4 *>(qbv + ib * N + c0 + g + j);
          tc::tmem_wait_ld();
          auto pass = [&](uint32_t j) -> bool {
            if constexpr (kFloat)
              return fmaf(-2.0f, __uint_as_float(d[j]), xnf) <= __uint_as_float(qb[j]);
            else return xn - 2 * __float2int_rn(__uint_as_float(d[j])) <= static_cast<int32_t>(qb[j]);
          };
          bool hit = false;
#pragma unroll
          for (uint32_t j = 0; j < G; ++j) hit |= pass(j);
          hit = hit && valid;
          if (__any_sync(0xffffffffu, hit)) {
            uint32_t mask = 0;
#pragma unroll
            for (uint32_t j = 0; j < G; ++j) mask |= static_cast<uint32_t>(pass(j)) << j;
            if (!valid) mask = 0;
            // records (query, l2, row) go to this CTA's list: one shared slot
            // reservation per warp (a warp scan of the lanes' hit counts),
            // then each lane writes its own records; the per-query count is a
            // fire-and-forget global add per record
            const uint32_t mine = __popc(mask);
            uint32_t incl = mine;
#pragma unroll
            for (uint32_t o = 1; o < 32; o <<= 1) {
              const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
              if (lane >= o) incl += t;
            }
            const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
            uint32_t at = 0;
            if (lane == 0) {
              at = atomicAdd(rcount, total);
              found += total;
            }
            at = __shfl_sync(0xffffffffu, at, 0) + incl - mine;
            while (mask) {
              const uint32_t j = __ffs(mask) - 1;
              mask &= mask - 1;
              uint32_t dj = 0;
#pragma unroll
              for (uint32_t k = 0; k < G; ++k) dj = k == j ? d[k] : dj;
              const QInfo q = qi[c0 + g + j];
              atomicAdd(A.qcount + q.qid, 1u);
              if (at < A.rec_cap) {
                const int32_t l2 = q.qn + xn - 2 * __float2int_rn(__uint_as_float(dj));
                rec[at] = make_uint4(q.qid, static_cast<uint32_t>(l2), grow, 0);
              } else {
                atomicOr(A.qcount + q.qid, kDropped);
              }
              ++at;
            }
          }
        };
        if (cph == 8) {
          process(std::integral_constant<uint32_t, 8>{}, 0);
        } else if constexpr (CH >= 16) {
          for (uint32_t g = 0; g < cph; g += 16) process(std::integral_constant<uint32_t, 16>{}, g);
        }
        // the slot's accumulators and row norms have been read: hand it back
        tc::fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(bar.acc_empty + ab);
        if (++ab == kTcAcc) ab = 0, abph ^= 1;
        ++tiles;
        if (w.last()) {
          __syncwarp();
          if (lane == 0) tc::mbar_arrive(bar.b_empty + ib);
          if (++ib == S.Bs) ib = 0, bph ^= 1;
        }
      }
      if (lane == 0) {
        if (half == 0 && q4 == 0) atomicAdd(A.counters, tiles);
        if (found) atomicAdd(A.counters + 1, found);
      }
    } else if (warp == kTmaWarp) {
      // ---- TMA producer
      if (lane == 0) {
        uint32_t rs = 0, rph = 0;
        uint32_t issued = 0, last_par[4] = {0, 0, 0, 0};
        for (; w.t < t1; ++w.t) {
          w.step();
          const int32_t y = static_cast<int32_t>(w.cur.row0 + (w.t - w.start) * kTcRows);
          bool ok = true;
          for (uint32_t kc = 0; kc < nkc; ++kc) {
            if (!timed_wait(bar.raw_empty + rs, rph ^ 1, err, pw[0], A.wait)) {
              ok = false;
              break;
            }
            tc::mbar_expect_tx(bar.raw_full + rs, rtile);
            tc::tma_load_2d(sm + L.raw + rs * rtile, &tmap, static_cast<int32_t>(kc * S.inner), y,
                            bar.raw_full + rs);
            issued |= 1u << rs;
            last_par[rs] = rph;
            if (++rs == S.Rs) rs = 0, rph ^= 1;
          }
          if (!ok) break;
        }
        if (*err)  // copies still in flight land before the CTA exits
          for (uint32_t s = 0; s < S.Rs; ++s)
            if (issued >> s & 1u) tc::mbar_wait(bar.raw_full + s, last_par[s]);
      }
      __syncwarp();
    } else if (warp == kMmaWarp) {
      // ---- MMA issuer
      if (lane == 0) {
        uint32_t idesc = tc::idesc_f16(kTcRows, N);
        uint32_t as = 0, aph = 0, ab = 0, abph = 0, ib = 0, bph = 0;
        unsigned long long pi = 0;  // cycles issuing MMAs and commits
        bool ok = true;
        for (; ok && w.t < t1; ++w.t) {
          w.step();
          if (w.first()) {
            if (!timed_wait(bar.b_full + ib, bph, err, pw[0], A.wait)) break;
            idesc = tc::idesc_f16(kTcRows, mma_width<N>(swidth[ib]));  // the item's queries
          }
          if (!timed_wait(bar.acc_empty + ab, abph ^ 1, err, pw[1], A.wait)) break;
          tc::fence_after();
          const uint32_t bbase = tc::smem_addr(sm + L.b + ib * btile);
          for (uint32_t kc = 0; kc < nkc; ++kc) {
            if (!timed_wait(bar.a_full + as, aph, err, pw[2], A.wait)) {
              ok = false;
              break;
            }
            tc::fence_after();
            const long long ti = clock64();
            // A from TMEM (8 columns per 16-dimension step); B's descriptor
            // advances 256 bytes (two core matrices), i.e. 16 encoded, per step
            const uint32_t a0 = tmem + acol + as * (S.inner / 2);
            const uint64_t bd0 = tc::desc(bbase + kc * S.inner * 16, 128, (h / 8) * 128);
            const uint32_t steps = min(S.inner, h - kc * S.inner) / 16;
            const uint32_t dcol = tmem + ab * N;
#pragma unroll
            for (uint32_t s = 0; s < 8; ++s)
              if (s < steps) tc::mma_f16_ts(dcol, a0 + 8 * s, bd0 + 16 * s, idesc, (kc | s) != 0);
            tc::commit(bar.a_empty + as);
            pi += clock64() - ti;
            if (++as == kTcAStages) as = 0, aph ^= 1;
          }
          if (!ok) break;
          tc::commit(bar.acc_full + ab);
          if (++ab == kTcAcc) ab = 0, abph ^= 1;
          if (w.last()) {
            tc::commit(bar.b_empty + ib);
            if (++ib == S.Bs) ib = 0, bph ^= 1;
          }
        }
        // every MMA issued has completed before tensor memory is released
        tc::commit(bar.done);
        tc::mbar_wait(bar.done, 0);
        if (A.prof) atomicAdd(A.prof + 14, pi);
      }
      __syncwarp();
    } else {
      // ---- query staging: thread j < N gathers query j of each item; each
      // staging warp arrives once per item
      const uint32_t j = tid - kQueryWarp0 * 32;
      uint32_t ib = 0, bph = 0;
      for (; w.t < t1; ++w.t) {
        w.step();
        if (!w.first()) continue;
        if (!__all_sync(0xffffffffu, timed_wait(bar.b_empty + ib, bph ^ 1, err, pw[0], A.wait))) break;
        if (j < N) {
          const uint32_t e0 = A.off[w.cur.list] + w.cur.qfirst;
          const uint32_t ne = min(N, A.off[w.cur.list + 1] - e0);
          if (j == 0) swidth[ib] = ne;
          unsigned char *b = sm + L.b + ib * btile;
          QInfo q{0, 0, INT_MIN, -INFINITY};
          if (j < ne) {
            q.qid = A.entries[e0 + j] / A.nprobe;
            const uint4 *src = reinterpret_cast<const uint4 *>(A.qhi + static_cast<size_t>(q.qid) * A.dc);
            uint32_t s1 = 0;
#pragma unroll 8
            for (uint32_t u = 0; u < h / 16; ++u) {
              const uint4 v = __ldg(src + u);
              uint4 lo, hi;
              tc::bytes_to_half16(v, bias, lo, hi);
              *reinterpret_cast<uint4 *>(b + tc::canon_off(j, u * 16, h)) = lo;
              *reinterpret_cast<uint4 *>(b + tc::canon_off(j, u * 16 + 8, h)) = hi;
              s1 = dp4(v.x, 0x01010101u, dp4(v.y, 0x01010101u, dp4(v.z, 0x01010101u, dp4(v.w, 0x01010101u, s1))));
            }
            // sum (q - 128)^2 = sum q^2 - 256 sum q + 16384 h
            const int64_t qn = A.qnorm[q.qid] - 256 * static_cast<int64_t>(s1) + 16384ll * h;
            q.qn = static_cast<int32_t>(qn);
            q.qb = static_cast<int32_t>(static_cast<int64_t>(A.bound[q.qid]) - qn);
            q.qbf = static_cast<float>(q.qb);
          } else {
            const uint4 zero = make_uint4(0, 0, 0, 0);  // fp16 zeros: a centred byte of 128
            for (uint32_t u = 0; u < h / 16; ++u) {
              *reinterpret_cast<uint4 *>(b + tc::canon_off(j, u * 16, h)) = zero;
              *reinterpret_cast<uint4 *>(b + tc::canon_off(j, u * 16 + 8, h)) = zero;
            }
          }
          qinfo[ib * N + j] = q;
          reinterpret_cast<uint32_t *>(sm + L.qbv)[ib * N + j] =
              kFloat ? __float_as_uint(q.qbf) : static_cast<uint32_t>(q.qb);
          tc::fence_smem_to_async();
        }
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(bar.b_full + ib);
        if (++ib == S.Bs) ib = 0, bph ^= 1;
      }
    }
  }
  if (A.prof) {
    // slots: converters 0-2, MMA 3-6, epilogue 7-9, TMA 10-11, staging 12-13
    const int base = warp < kConvWarps ? 0 : warp < kTmaWarp ? 7 : warp == kTmaWarp ? 10
                   : warp == kMmaWarp ? 3 : 12;
    const int nw = base == 3 ? 3 : base == 10 || base == 12 ? 1 : 2;
    const bool lead = tid == 0 || tid == kConvWarps * 32 || tid == kTmaWarp * 32 ||
                      tid == kMmaWarp * 32 || tid == kQueryWarp0 * 32;
    if (lead) {
      for (int i = 0; i < nw; ++i) atomicAdd(A.prof + base + i, pw[i]);
      atomicAdd(A.prof + base + nw, static_cast<unsigned long long>(clock64() - tstart));
    }
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (tid == 0) {
    if (*err) atomicAdd(A.timeouts, 1u);
    A.rec_n[blockIdx.x] = min(*rcount, A.rec_cap);
    // the longest CTA (cycles): against the average it shows the schedule's imbalance
    if (A.prof) atomicMax(A.prof + 15, static_cast<unsigned long long>(clock64() - tstart));
  }
  if (warp == kMmaWarp) tc::tmem_dealloc(tmem, S.tcols);
}

// The squared L2 over the first h high bytes of a row and a query whose bytes
// are in shared memory as words; dp4a over 16 bytes per step.
__device__ __forceinline__ uint32_t row_dot(const uint8_t *row, const uint32_t *qw, uint32_t h) {
  const uint4 *rv = reinterpret_cast<const uint4 *>(row);
  uint32_t dot = 0;
  uint32_t u = 0;
  for (; u + 4 <= h / 16; u += 4) {  // four loads in flight
    uint4 v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = __ldg(rv + u + j);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t *w = qw + 4 * (u + j);
      dot = dp4(v[j].x, w[0], dp4(v[j].y, w[1], dp4(v[j].z, w[2], dp4(v[j].w, w[3], dot))));
    }
  }
  for (; u < h / 16; ++u) {
    const uint4 v = __ldg(rv + u);
    const uint32_t *w = qw + 4 * u;
    dot = dp4(v.x, w[0], dp4(v.y, w[1], dp4(v.z, w[2], dp4(v.w, w[3], dot))));
  }
  return dot;
}

// Dot products of a query (its h bytes as words in shared memory) with rows
// row(0) .. row(n - 1) of a byte plane, lanes split along each row: a group of
// G = min(32, h / 16) lanes reads a row as one coalesced run of 16-byte
// loads and sums over the group by shuffles. A warp takes 32 rows at a time
// (G steps, all loads of the batch in flight together) and hands row
// base + l of the batch to one lane, so f(i, dot) runs on all 32 lanes at
// once. All threads of the CTA take part.
//
// pre(i) - a per-row value the callback needs (e.g. the row's norm) - is
// loaded at the start of the batch by the lane that later calls
// f(i, dot, pre(i)), so that it arrives with the rows instead of after them.

template <uint32_t G, typename F, typename Pre, typename RowAt>
__device__ __forceinline__ void rows_split(const uint8_t *__restrict__ x, uint32_t dc, uint32_t h,
                                           const uint32_t *qw, RowAt row, uint32_t n, Pre pre,
                                           F f) {
  constexpr uint32_t RPW = 32 / G;  // rows per step
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const uint32_t sub = lane / G, gl = lane % G, cpl = (h / 16) / G;
  for (uint32_t base = warp * 32; base < n; base += nw * 32) {
    uint32_t mine = 0;
    const uint32_t my_row = base + gl * RPW + sub;
    const int64_t pv = my_row < n ? pre(my_row) : 0;
    if (G <= 16 && cpl == 1) {
      // every load of the batch first, then the sums
      uint4 v[G <= 16 ? G : 1];
      const uint32_t *w = qw + 4 * gl;
#pragma unroll
      for (uint32_t it = 0; it < (G <= 16 ? G : 1); ++it) {
        const uint32_t i = base + it * RPW + sub;
        v[it] = i < n ? __ldg(reinterpret_cast<const uint4 *>(x + static_cast<size_t>(row(i)) * dc) + gl)
                      : make_uint4(0, 0, 0, 0);
      }
#pragma unroll
      for (uint32_t it = 0; it < (G <= 16 ? G : 1); ++it) {
        uint32_t dot = dp4(v[it].x, w[0], dp4(v[it].y, w[1], dp4(v[it].z, w[2], dp4(v[it].w, w[3], 0))));
#pragma unroll
        for (uint32_t o = G / 2; o; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
        if (gl == it) mine = dot;
      }
    } else {
#pragma unroll
      for (uint32_t it = 0; it < G; ++it) {
        const uint32_t i = base + it * RPW + sub;
        uint32_t dot = 0;
        if (i < n) {
          const uint4 *rv = reinterpret_cast<const uint4 *>(x + static_cast<size_t>(row(i)) * dc);
          for (uint32_t c = 0; c < cpl; ++c) {
            const uint32_t u = gl + c * G;
            const uint4 vv = __ldg(rv + u);
            const uint32_t *w = qw + 4 * u;
            dot = dp4(vv.x, w[0], dp4(vv.y, w[1], dp4(vv.z, w[2], dp4(vv.w, w[3], dot))));
          }
        }
#pragma unroll
        for (uint32_t o = G / 2; o; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
        if (gl == it) mine = dot;
      }
    }
    if (my_row < n) f(my_row, mine, pv);
  }
}

// rows_split with the group size for h.
template <typename F, typename Pre, typename RowAt>
__device__ __forceinline__ void for_rows_at(const uint8_t *__restrict__ x, uint32_t dc, uint32_t h,
                                            const uint32_t *qw, RowAt row, uint32_t n, F f, Pre pre) {
  const uint32_t g = min(32u, h / 16);
  if (g == 16) rows_split<16>(x, dc, h, qw, row, n, pre, f);
  else if (g == 32) rows_split<32>(x, dc, h, qw, row, n, pre, f);
  else if (g == 8) rows_split<8>(x, dc, h, qw, row, n, pre, f);
  else rows_split<4>(x, dc, h, qw, row, n, pre, f);
}

// The same over the contiguous rows r0 .. r0 + n - 1.
template <typename F, typename Pre>
__device__ __forceinline__ void for_rows_split(const uint8_t *__restrict__ x, uint32_t dc, uint32_t h,
                                               const uint32_t *qw, uint32_t r0, uint32_t n, F f,
                                               Pre pre) {
  for_rows_at(x, dc, h, qw, [r0](uint32_t i) { return r0 + i; }, n, f, pre);
}

// ------------------------------------------------------------- seed bounds
// One CTA per query. It looks at the first `want` rows of the query's probed
// lists (probe order, nearest list first). When there are more than `full` of
// them, a sketch picks the ones to score: the squared distance over the first
// 32 head dimensions (the leading rotated dimensions, which carry most of the
// variance), of which the `full` smallest, and any others in the last one's
// bin of sketch distance / 16, are scored over all h dimensions.
// The bound is the S-th smallest scored l2, widened to L + (L >> 22) + 1: the
// distance value is monotone in l2 and two l2 that far apart never round to
// the same float, so every row whose distance can tie the S-th best is still
// inside. Any S of a query's candidates bound its S-th best from above, so
// the rows the sketch picks change no result, only how tight the bound is
// and how many bytes it costs: 2,048 sketched rows (32 bytes each) and 3S
// scored rows read 2.3 times fewer bytes than 1,024 scored rows of 256 bytes
// and leave fewer candidates. Fewer than S rows: no bound.
// The queries grouped by their nearest list: a counting sort by one CTA, so
// that seed CTAs reading the same list's rows run together and share them
// through L2. order[i] = the query the i-th seed CTA takes.
constexpr uint32_t kOrderLists = 16384;  // lists the counting sort holds in shared memory

__global__ void __launch_bounds__(1024) seed_order_kernel(const uint32_t *__restrict__ probed,
                                                          uint32_t p, uint32_t B, uint32_t L,
                                                          uint32_t *__restrict__ order) {
  extern __shared__ uint32_t lh[];  // L counters, then offsets
  for (uint32_t i = threadIdx.x; i < L; i += blockDim.x) lh[i] = 0;
  __syncthreads();
  for (uint32_t q = threadIdx.x; q < B; q += blockDim.x)
    atomicAdd(&lh[probed[static_cast<size_t>(q) * p]], 1u);
  __syncthreads();
  block_scan2(
      L, [&](uint32_t i) { return make_uint2(lh[i], 0u); },
      [&](uint32_t i, uint32_t a, uint32_t) { lh[i] = a; });
  __syncthreads();
  for (uint32_t q = threadIdx.x; q < B; q += blockDim.x)
    order[atomicAdd(&lh[probed[static_cast<size_t>(q) * p]], 1u)] = q;
}

constexpr uint32_t kSketchBytes = 32;  // head bytes of a row the sketch reads

__device__ __forceinline__ uint32_t sq_diff4(uint32_t a, uint32_t b, uint32_t acc) {
  const uint32_t d = __vabsdiffu4(a, b);  // |a - b| per byte
  return dp4(d, d, acc);
}

__global__ void __launch_bounds__(256, 3) rank_seed_kernel(
    const uint8_t *__restrict__ xhi, const int64_t *__restrict__ xnorm,
    const uint8_t *__restrict__ qhi, const int64_t *__restrict__ qnorm,
    const uint32_t *__restrict__ probed, const uint32_t *__restrict__ qprobes,
    const uint32_t *__restrict__ list_off, const uint32_t *__restrict__ order, uint32_t p,
    uint32_t dc, uint32_t h, uint32_t S, uint32_t want, uint32_t full, int32_t *__restrict__ bound) {
  // rowof: the rows looked at; val: their sketch keys. After the pick the
  // scored rows are in val and their l2 go to rowof.
  __shared__ uint32_t rowof[kSeedCap], val[kSeedCap];
  __shared__ __align__(16) uint32_t qw[2048 / 4];
  __shared__ uint32_t hist[256], sel[2], wsum[8], npick;
  const uint32_t q = order ? order[blockIdx.x] : blockIdx.x, tid = threadIdx.x;
  for (uint32_t i = tid; i < h / 4; i += blockDim.x)
    qw[i] = reinterpret_cast<const uint32_t *>(qhi + static_cast<size_t>(q) * dc)[i];
  const uint32_t pq = qprobes ? qprobes[q] : p;  // the query's own budget
  uint32_t count = 0;
  for (uint32_t r = 0; r < pq && count < want; ++r) {
    const uint32_t c = probed[static_cast<size_t>(q) * p + r];
    const uint32_t r0 = list_off[c], n = min(list_off[c + 1] - r0, want - count);
    for (uint32_t i = tid; i < n; i += blockDim.x) rowof[count + i] = r0 + i;
    count += n;
  }
  if (tid == 0) npick = 0;
  __syncthreads();
  if (count < S) {
    if (tid == 0) bound[q] = 0x7FFFFFFF;
    return;
  }
  // radix selection of the rank-th smallest of v[0 .. n) by 8-bit digits,
  // from the digit at bit `start` down to the one at bit `stop` (the lower
  // bits of the result stay 0; digits above `start` must be 0 in every value)
  auto select = [&](const uint32_t *v, uint32_t n, uint32_t rank, int start, int stop) {
    uint32_t prefix = 0;
    for (int shift = start; shift >= stop; shift -= 8) {
      for (uint32_t i = tid; i < 256; i += blockDim.x) hist[i] = 0;
      __syncthreads();
      const uint32_t hm = shift == 24 ? 0u : (0xFFFFFFFFu << (shift + 8));
      for (uint32_t i = tid; i < n; i += blockDim.x)
        if ((v[i] & hm) == prefix) atomicAdd(&hist[(v[i] >> shift) & 0xFFu], 1u);
      __syncthreads();
      block_pick_digit(hist, rank, sel, wsum);
      rank -= sel[1];
      prefix |= sel[0] << shift;
      __syncthreads();
    }
    return prefix;
  };
  const uint32_t *rows = rowof;
  uint32_t *l2s = val, n = count;
  if (count > full) {
    // keys (sketch distance, at most 20 bits) << 12 | i. Two digits find the
    // 16-bit bin (sketch distance >> 4) of the full-th smallest key; every
    // row in or below that bin is scored: at least `full`, a few more when
    // the bin holds several
    const uint32_t parts = min(kSketchBytes, h) / 16;  // lanes per row, 16 bytes each
    const uint32_t part = tid % parts, per = blockDim.x / parts;
    const uint4 qv = reinterpret_cast<const uint4 *>(qw)[part];
    for (uint32_t base = 0; base < count; base += 4 * per) {
      uint4 v[4];
#pragma unroll
      for (uint32_t j = 0; j < 4; ++j) {
        const uint32_t i = base + j * per + tid / parts;
        v[j] = i < count ? __ldg(reinterpret_cast<const uint4 *>(
                               xhi + static_cast<size_t>(rowof[i]) * dc) + part)
                         : make_uint4(0, 0, 0, 0);
      }
#pragma unroll
      for (uint32_t j = 0; j < 4; ++j) {
        uint32_t d2 = sq_diff4(v[j].x, qv.x, sq_diff4(v[j].y, qv.y,
                      sq_diff4(v[j].z, qv.z, sq_diff4(v[j].w, qv.w, 0))));
        if (parts == 2) d2 += __shfl_xor_sync(0xffffffffu, d2, 1);
        const uint32_t i = base + j * per + tid / parts;
        if (part == 0 && i < count) val[i] = (min(d2, 0xFFFFFu) << 12) | i;
      }
    }
    __syncthreads();
    const uint32_t kth = select(val, count, full - 1, 24, 16) | 0xFFFFu;
    uint32_t mine = 0;  // bit j: key tid + 256 j is picked (count <= 16 x 256)
    for (uint32_t j = 0, i = tid; i < count; ++j, i += blockDim.x)
      if (val[i] <= kth) mine |= 1u << j;
    __syncthreads();
    for (uint32_t j = 0, i = tid; i < count; ++j, i += blockDim.x)
      if (mine >> j & 1u) val[atomicAdd(&npick, 1u)] = rowof[i];
    __syncthreads();
    rows = val;
    l2s = rowof;
    n = npick;
  }
  const int64_t qn = qnorm[q];
  for_rows_at(
      xhi, dc, h, qw, [&](uint32_t i) { return rows[i]; }, n,
      [&](uint32_t i, uint32_t dot, int64_t xn) {
        l2s[i] = static_cast<uint32_t>(qn + xn - 2 * static_cast<int64_t>(dot));
      },
      [&](uint32_t i) { return xnorm[rows[i]]; });
  __syncthreads();
  // l2 < 255^2 h: below 2^24 (no top digit) for h up to 258
  const uint32_t L2 = select(l2s, n, S - 1, h * 65025u < (1u << 24) ? 16 : 24, 0);
  if (tid == 0) {
    const int32_t v = static_cast<int32_t>(L2);
    bound[q] = v + (v >> 22) + 1;
  }
}

// --------------------------------------------------------- overflow rescan
// A query whose buffer overflowed (more than `cap` rows within its seed
// bound; the buffer holds the first cap of them) is rescanned in rounds:
//   * rescan_bound_kernel: K = the S-th smallest key (distance bits << 32 |
//     id) among the rows in its buffer - an upper bound on the query's true
//     S-th best key, as they are some of its candidates; the query is listed
//     and its count reset;
//   * rescan_rows_kernel: CTAs over (listed query, probed list) pairs put the
//     rows with key <= K into the buffer. If they fit, the buffer holds every
//     row that can be selected. Otherwise the next round's K comes from the
//     new buffer and is strictly smaller (its cap > S distinct keys are all
//     <= K), which shrinks the count by about cap / S per round;
//   * rescan_exact_kernel, after kRescanRounds rounds: the S smallest keys by
//     8-bit radix selection over all of a query's candidates, one CTA each.
// Distances are recomputed from the codes; results never depend on the
// buffer size.
constexpr int kRescanRounds = 2;

// The rank-th smallest 64-bit key produced by key(i), i < n, by 8-bit radix
// digits; all threads of the CTA call it and get the key.
template <typename KeyAt>
__device__ unsigned long long block_select64(uint32_t n, uint32_t rank, KeyAt key, uint32_t *hist,
                                             uint32_t *sel) {
  __shared__ uint32_t wsum[8];
  unsigned long long prefix = 0;
  for (int shift = 56; shift >= 0; shift -= 8) {
    for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    const unsigned long long hm = shift == 56 ? 0ull : (~0ull << (shift + 8));
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
      const unsigned long long k = key(i);
      if ((k & hm) == prefix) atomicAdd(&hist[(k >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    block_pick_digit(hist, rank, sel, wsum);
    rank -= sel[1];
    prefix |= static_cast<unsigned long long>(sel[0]) << shift;
    __syncthreads();
  }
  return prefix;
}

struct RowKey {
  const uint8_t *xhi;
  const int64_t *xnorm;
  const uint32_t *ids;
  uint32_t dc, h;
  DistScale scale;
  __device__ unsigned long long operator()(uint32_t row, const uint32_t *qw, int64_t qn) const {
    const uint32_t dot = row_dot(xhi + static_cast<size_t>(row) * dc, qw, h);
    const int64_t l2 = qn + xnorm[row] - 2 * static_cast<int64_t>(dot);
    return (static_cast<unsigned long long>(__float_as_uint(dist_value(l2, scale))) << 32) | ids[row];
  }
};

__device__ __forceinline__ void load_query_words(const uint8_t *qhi, uint32_t q, uint32_t dc,
                                                 uint32_t h, uint32_t *qw) {
  for (uint32_t i = threadIdx.x; i < h / 4; i += blockDim.x)
    qw[i] = reinterpret_cast<const uint32_t *>(qhi + static_cast<size_t>(q) * dc)[i];
}

__global__ void __launch_bounds__(256) rescan_bound_kernel(
    const uint32_t *__restrict__ ids, uint32_t *__restrict__ qcount,
    const uint32_t *__restrict__ qfill, const uint2 *__restrict__ qbuf, uint32_t cap, uint32_t S,
    uint32_t round, uint32_t *__restrict__ list, unsigned long long *__restrict__ kbound,
    uint32_t *__restrict__ nlisted, unsigned long long *__restrict__ stats) {
  __shared__ uint32_t hist[256], sel[2];
  const uint32_t q = blockIdx.x;
  const uint32_t n = qcount[q];  // bit 31: records were dropped
  if (round == 0 && threadIdx.x == 0)
    atomicMax(stats + 1, static_cast<unsigned long long>(n & ~kDropped));
  if (n <= cap) return;
  // entries actually in the buffer: the bucketing step's fill in round 0,
  // the previous round's count after that
  // (a subset's S-th smallest key is a bound as well: look at 2048 at most)
  const uint32_t valid = min(min(round == 0 ? qfill[q] : n, cap), 2048u);
  const uint2 *buf = qbuf + static_cast<size_t>(q) * cap;
  const unsigned long long K =
      valid < S ? ~0ull
                : block_select64(
                      valid, S - 1,
                      [&](uint32_t i) {
                        const uint2 e = buf[i];
                        return (static_cast<unsigned long long>(e.x) << 32) | ids[e.y];
                      },
                      hist, sel);
  if (threadIdx.x == 0) {
    kbound[q] = K;
    qcount[q] = 0;
    list[atomicAdd(nlisted, 1u)] = q;
    if (round == 0) atomicAdd(stats, 1ull);
  }
}

__global__ void __launch_bounds__(256) rescan_rows_kernel(
    RowKey key, const uint8_t *__restrict__ qhi, const int64_t *__restrict__ qnorm,
    const uint32_t *__restrict__ probed, const uint32_t *__restrict__ qprobes,
    const uint32_t *__restrict__ list_off, uint32_t p, uint32_t *__restrict__ qcount,
    uint2 *__restrict__ qbuf, uint32_t cap, const uint32_t *__restrict__ list,
    const unsigned long long *__restrict__ kbound, const uint32_t *__restrict__ nlisted) {
  __shared__ uint32_t qw[2048 / 4];
  const size_t pairs = static_cast<size_t>(*nlisted) * p;
  for (size_t pair = blockIdx.x; pair < pairs; pair += gridDim.x) {
    const uint32_t q = list[pair / p];
    if (qprobes && pair % p >= qprobes[q]) continue;  // beyond the query's budget
    const uint32_t c = probed[static_cast<size_t>(q) * p + pair % p];
    __syncthreads();
    load_query_words(qhi, q, key.dc, key.h, qw);
    __syncthreads();
    const int64_t qn = qnorm[q];
    const unsigned long long K = kbound[q];
    uint2 *buf = qbuf + static_cast<size_t>(q) * cap;
    const uint32_t r0 = list_off[c];
    for_rows_split(
        key.xhi, key.dc, key.h, qw, r0, list_off[c + 1] - r0,
        [&](uint32_t i, uint32_t dot, int64_t xn) {
      const uint32_t row = r0 + i;
      const int64_t l2 = qn + xn - 2 * static_cast<int64_t>(dot);
      const unsigned long long k =
          (static_cast<unsigned long long>(__float_as_uint(dist_value(l2, key.scale))) << 32) |
          key.ids[row];
      if (k <= K) {
        const uint32_t at = atomicAdd(qcount + q, 1u);
        if (at < cap) buf[at] = make_uint2(static_cast<uint32_t>(k >> 32), row);
      }
    },
        [&](uint32_t i) { return key.xnorm[r0 + i]; });
  }
}

__global__ void __launch_bounds__(256) rescan_exact_kernel(
    RowKey key, const uint8_t *__restrict__ qhi, const int64_t *__restrict__ qnorm,
    const uint32_t *__restrict__ probed, const uint32_t *__restrict__ qprobes,
    const uint32_t *__restrict__ list_off, uint32_t p, uint32_t S, uint32_t *__restrict__ qcount,
    uint2 *__restrict__ qbuf, uint32_t cap) {
  const uint32_t q = blockIdx.x, tid = threadIdx.x;
  if (qcount[q] <= cap) return;
  __shared__ uint32_t qw[2048 / 4];
  __shared__ uint32_t hist[256], sel[2], taken;
  load_query_words(qhi, q, key.dc, key.h, qw);
  if (tid == 0) taken = 0;
  __syncthreads();
  const int64_t qn = qnorm[q];
  const uint32_t *pq = probed + static_cast<size_t>(q) * p;
  const uint32_t np = qprobes ? qprobes[q] : p;  // the query's own budget
  uint32_t total = 0;
  for (uint32_t r = 0; r < np; ++r) total += list_off[pq[r] + 1] - list_off[pq[r]];
  // more than cap >= S candidates, so the S-th smallest key exists
  const unsigned long long K = block_select64(
      total, S - 1,
      [&](uint32_t i) {
        uint32_t r = 0;
        for (;;) {
          const uint32_t len = list_off[pq[r] + 1] - list_off[pq[r]];
          if (i < len) break;
          i -= len;
          ++r;
        }
        return key(list_off[pq[r]] + i, qw, qn);
      },
      hist, sel);
  uint2 *buf = qbuf + static_cast<size_t>(q) * cap;
  for (uint32_t r = 0; r < np; ++r)
    for (uint32_t row = list_off[pq[r]] + tid; row < list_off[pq[r] + 1]; row += blockDim.x) {
      const unsigned long long k = key(row, qw, qn);
      if (k <= K) {
        const uint32_t at = atomicAdd(&taken, 1u);  // exactly S rows (distinct ids)
        if (at < cap) buf[at] = make_uint2(static_cast<uint32_t>(k >> 32), row);
      }
    }
  __syncthreads();
  if (tid == 0) qcount[q] = min(taken, cap);
}

// -------------------------------------------------- work items and offsets
// Per list: items = ceil(queries / N) (none for an empty list), tiles per
// item = ceil(rows / 128); counts[c] = items, counts[L + 1 + c] = items x tiles.
// MMA width of an item of ne queries (host and device, as mma_width<N>).
__host__ __device__ __forceinline__ uint32_t item_width(uint32_t ne, uint32_t N) {
  return ne <= 16 ? 16u : (ne <= 32 && N > 32 ? 32u : N);
}

// probed (optional, 2 counters): the distinct lists the batch probes (not
// empty) and their rows, i.e. the rows the pass reads once each.
__global__ void tc_count_kernel(const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ list_off,
                                uint32_t L, uint32_t N, uint32_t B, uint32_t beta,
                                uint32_t *__restrict__ counts, uint32_t *__restrict__ qcount,
                                uint32_t *__restrict__ qfill, unsigned long long *__restrict__ probed) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < B) {
    qcount[c] = 0;
    qfill[c] = 0;
  }
  uint32_t lists = 0, rows = 0;
  if (c < L) {
    const uint32_t n = list_off[c + 1] - list_off[c];
    const uint32_t items = n ? (cnt[c] + N - 1) / N : 0;
    const uint32_t tiles = (n + kTcRows - 1) / kTcRows;
    counts[c] = items;
    counts[L + 1 + c] = items * tiles;
    if (beta) {  // full items first, then the remainder
      const uint32_t full = n ? cnt[c] / N : 0, rem = n ? cnt[c] % N : 0;
      counts[2 * (L + 1) + c] =
          tiles * (full * (64 + beta * N) + (rem ? 64 + beta * item_width(rem, N) : 0));
    }
    if (items) lists = 1, rows = n;
  }
  if (probed) {  // whole warps take part: one add per warp and counter
    const uint32_t wl = __reduce_add_sync(0xffffffffu, lists);
    const uint32_t wr = __reduce_add_sync(0xffffffffu, rows);
    if ((threadIdx.x & 31) == 0 && wl) {
      atomicAdd(probed, static_cast<unsigned long long>(wl));
      atomicAdd(probed + 1, static_cast<unsigned long long>(wr));
    }
  }
}

// Exclusive scans of the two count arrays by one CTA of 1024 threads (in
// place); the totals go to *nitems and tile_off[*nitems].
__global__ void __launch_bounds__(1024) tc_scan_kernel(uint32_t *__restrict__ counts, uint32_t L,
                                                       uint32_t *__restrict__ nitems,
                                                       uint32_t *__restrict__ tile_off,
                                                       uint32_t *__restrict__ cost_off) {
  uint32_t *ca = counts, *cb = counts + L + 1, *cc = counts + 2 * (L + 1);
  const uint2 tot = block_scan2(
      L, [&](uint32_t i) { return make_uint2(ca[i], cb[i]); },
      [&](uint32_t i, uint32_t a, uint32_t b) {
        ca[i] = a;
        cb[i] = b;
      });
  uint32_t cost = 0;
  if (cost_off) {
    __syncthreads();
    cost = block_scan2(
               L, [&](uint32_t i) { return make_uint2(cc[i], 0u); },
               [&](uint32_t i, uint32_t a, uint32_t) { cc[i] = a; })
               .x;
  }
  if (threadIdx.x == 0) {
    *nitems = tot.x;
    tile_off[tot.x] = tot.y;
    if (cost_off) cost_off[tot.x] = cost;
  }
}

// tile_hist (optional, 6 counters): the tiles of the items with 1-2, 3-4,
// 5-8, 9-16, 17-32 and 33-64 queries.
__global__ void tc_expand_kernel(const uint32_t *__restrict__ list_off, const uint32_t *__restrict__ counts,
                                 const uint32_t *__restrict__ cnt, uint32_t L, uint32_t N,
                                 uint32_t beta, const uint32_t *__restrict__ nitems,
                                 TcItem *__restrict__ items, uint32_t *__restrict__ tile_off,
                                 uint32_t *__restrict__ cost_off,
                                 unsigned long long *__restrict__ tile_hist) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t hist[6] = {0, 0, 0, 0, 0, 0};
  if (c < L) {
    const uint32_t i0 = counts[c], i1 = c + 1 < L ? counts[c + 1] : *nitems;
    const uint32_t tiles = (list_off[c + 1] - list_off[c] + kTcRows - 1) / kTcRows;
    const uint32_t tb = counts[L + 1 + c];
    for (uint32_t j = 0; j < i1 - i0; ++j) {
      items[i0 + j] = TcItem{c, j * N, list_off[c], list_off[c + 1] - list_off[c]};
      tile_off[i0 + j] = tb + j * tiles;
      // every item before the last of its list is full (width N)
      if (cost_off) cost_off[i0 + j] = counts[2 * (L + 1) + c] + j * tiles * (64 + beta * N);
      const uint32_t ne = min(N, cnt[c] - j * N);
      hist[ne <= 2 ? 0 : ne <= 4 ? 1 : ne <= 8 ? 2 : ne <= 16 ? 3 : ne <= 32 ? 4 : 5] += tiles;
    }
  }
  if (tile_hist) {  // whole warps take part: one add per warp and bin
#pragma unroll
    for (int b = 0; b < 6; ++b) {
      const uint32_t v = __reduce_add_sync(0xffffffffu, hist[b]);
      if ((threadIdx.x & 31) == 0 && v) atomicAdd(tile_hist + b, static_cast<unsigned long long>(v));
    }
  }
}

// The pass's candidate records (query, l2, row) into per-query buffers of
// (distance bits, row); one CTA per pass CTA.
__global__ void __launch_bounds__(512) tc_bucket_kernel(const uint4 *__restrict__ rec,
                                                        const uint32_t *__restrict__ rec_n,
                                                        uint32_t rec_cap, uint32_t *__restrict__ qfill,
                                                        uint2 *__restrict__ qbuf, uint32_t cap,
                                                        DistScale scale) {
  // gridDim.y CTAs share each ranking CTA's list, so that enough records
  // (each a global atomic and a scattered store) are in flight per SM
  const uint4 *r = rec + static_cast<size_t>(blockIdx.x) * rec_cap;
  const uint32_t n = rec_n[blockIdx.x];
  for (uint32_t i = blockIdx.y * blockDim.x + threadIdx.x; i < n; i += gridDim.y * blockDim.x) {
    const uint4 e = r[i];
    const uint32_t at = atomicAdd(qfill + e.x, 1u);
    if (at < cap)
      qbuf[static_cast<size_t>(e.x) * cap + at] =
          make_uint2(__float_as_uint(dist_value(static_cast<int32_t>(e.y), scale)), e.z);
  }
}

}  // namespace

uint32_t rank_tc_ctas() {
  int sms = 0;
  if (current_sms(&sms) != KATO_OK) sms = 1;
  return static_cast<uint32_t>(std::max(sms, 1));
}

std::atomic<uint32_t> g_tc_width{0}, g_tc_beta{0};
std::atomic<unsigned long long> g_tc_wait{0};

bool rank_tc_plan(uint32_t h, uint32_t dc, TcShape *s) {
  if (h == 0 || h % 64 || h > 1024 || h > dc || dc % 64) return false;
  TcShape t{};
  t.N = h <= 256 ? 64 : (h <= 512 ? 32 : 16);
  const uint32_t cap = g_tc_width.load();
  if (cap >= 16 && cap < t.N) t.N = cap;
  t.inner = dc >= 128 ? 128 : 64;
  // accumulators (kTcAcc slots of N columns), then the A stages (inner / 2 columns each)
  t.tcols = 32;
  while (t.tcols < kTcAcc * t.N + kTcAStages * t.inner / 2) t.tcols <<= 1;
  for (uint32_t bs = 2; bs >= 1; --bs)
    for (uint32_t rs = 4; rs >= 2; --rs) {
      t.Bs = bs;
      t.Rs = rs;
      t.smem = tc_smem_layout(h, t).total;
      if (t.smem <= 227 * 1024) {
        *s = t;
        return true;
      }
    }
  return false;
}

int rank_tc(const RankTcArgs &A, const uint8_t *xhi, uint32_t npts, const TcShape &s,
            cudaStream_t st) {
  const PFN_cuTensorMapEncodeTiled_v12000 encode = tc::tensor_map_encoder();
  if (!encode) return cuda_status(cudaErrorNotSupported, "cuTensorMapEncodeTiled");
  // the high-byte plane as a 2-D tensor of bytes: x = byte in row, y = row
  CUtensorMap tmap;
  const cuuint64_t dims[2] = {A.dc, npts};
  const cuuint64_t strides[1] = {A.dc};
  const cuuint32_t box[2] = {s.inner, kTcRows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult cr = encode(&tmap, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<uint8_t *>(xhi), dims,
                             strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                             s.inner == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed for the high-byte plane (error " + std::to_string(cr) + ")");
    return KATO_ERUNTIME;
  }
  const uint32_t ctas = rank_tc_ctas();
  auto go = [&](auto kern) -> int {
    if (const int rc = smem_limit(reinterpret_cast<const void *>(kern), static_cast<int>(s.smem),
                                  "rank_tc_kernel shared memory"))
      return rc;
    kern<<<ctas, kTcThreads, s.smem, st>>>(tmap, A, s);
    KATO_LAUNCHED("rank_tc_kernel");
    return KATO_OK;
  };
  // the float comparison is exact while |xn' - 2 dot'| < 2^24: h <= 320
  if (s.N == 64) return go(rank_tc_kernel<64, true>);
  if (s.N == 32) return A.h <= 320 ? go(rank_tc_kernel<32, true>) : go(rank_tc_kernel<32, false>);
  if (s.N == 16) return go(rank_tc_kernel<16, false>);
  return invalid("unsupported ranking shape");
}

int rank_tc_bucket(const uint4 *rec, const uint32_t *rec_n, uint32_t rec_cap, uint32_t ctas,
                   uint32_t *qfill, uint2 *qbuf, uint32_t cap, DistScale scale, cudaStream_t st) {
  tc_bucket_kernel<<<dim3(ctas, 4), 512, 0, st>>>(rec, rec_n, rec_cap, qfill, qbuf, cap, scale);
  KATO_LAUNCHED("tc_bucket_kernel");
  return KATO_OK;
}

int rank_seed(const uint8_t *xhi, const int64_t *xnorm, const uint8_t *qhi, const int64_t *qnorm,
              const uint32_t *probed, const uint32_t *qprobes, const uint32_t *list_off,
              uint32_t L, uint32_t B, uint32_t p, uint32_t dc, uint32_t h, uint32_t S,
              uint32_t rows, uint32_t *order, int32_t *bound, cudaStream_t st) {
  if (h > 2048 || h % 16) return invalid("seed bounds need h <= 2048, a multiple of 16");
  if (B == 0) return KATO_OK;
  const uint32_t *ord = nullptr;
  if (order && L <= kOrderLists) {
    if (const int rc = smem_limit(reinterpret_cast<const void *>(seed_order_kernel),
                                  static_cast<int>(kOrderLists * 4), "seed_order_kernel shared memory"))
      return rc;
    seed_order_kernel<<<1, 1024, L * 4, st>>>(probed, p, B, L, order);
    KATO_LAUNCHED("seed_order_kernel");
    ord = order;
  }
  // rows the sketch picks to score in full: 3S (fewer loosen the bound, more
  // cost bytes)
  const uint32_t want = std::min(std::max(rows, S), kSeedCap);
  rank_seed_kernel<<<B, 256, 0, st>>>(xhi, xnorm, qhi, qnorm, probed, qprobes, list_off, ord, p, dc,
                                      h, S, want, std::min(want, 3 * S), bound);
  KATO_LAUNCHED("rank_seed_kernel");
  return KATO_OK;
}

int rank_tc_prepare(const uint32_t *cnt, const uint32_t *list_off, uint32_t L, uint32_t N,
                    uint32_t B, uint32_t beta, uint32_t *scratch, TcItem *items,
                    uint32_t *tile_off, uint32_t *cost_off, uint32_t *nitems, uint32_t *qcount,
                    uint32_t *qfill, unsigned long long *tile_hist, cudaStream_t st) {
  uint32_t *co = beta ? cost_off : nullptr;
  // the distinct probed lists and rows go to the two counters after the histogram
  tc_count_kernel<<<div_up(std::max(std::max(L, B), 1u), 256), 256, 0, st>>>(
      cnt, list_off, L, N, B, beta, scratch, qcount, qfill, tile_hist ? tile_hist + 6 : nullptr);
  tc_scan_kernel<<<1, 1024, 0, st>>>(scratch, L, nitems, tile_off, co);
  tc_expand_kernel<<<div_up(L, 256), 256, 0, st>>>(list_off, scratch, cnt, L, N, beta, nitems,
                                                   items, tile_off, co, tile_hist);
  KATO_LAUNCHED("ranking work preparation");
  return KATO_OK;
}

int rank_overflow(const uint8_t *xhi, const int64_t *xnorm, const uint32_t *ids,
                  const uint8_t *qhi, const int64_t *qnorm, const uint32_t *probed,
                  const uint32_t *qprobes, const uint32_t *list_off, uint32_t B, uint32_t p,
                  uint32_t dc, uint32_t h,
                  uint32_t S, DistScale scale, uint32_t *qcount, uint2 *qbuf, uint32_t cap,
                  const RescanBufs &rb, unsigned long long *stats, cudaStream_t st) {
  if (S > cap) return invalid("candidate buffer smaller than the survivor count");
  if (B == 0) return KATO_OK;
  const uint32_t sms = rank_tc_ctas();
  const RowKey key{xhi, xnorm, ids, dc, h, scale};
  KATO_CUDA(cudaMemsetAsync(rb.nlisted, 0, kRescanRounds * sizeof(uint32_t), st));
  for (int r = 0; r < kRescanRounds; ++r) {
    rescan_bound_kernel<<<B, 256, 0, st>>>(ids, qcount, rb.qfill, qbuf, cap, S, r, rb.list,
                                           rb.kbound, rb.nlisted + r, stats);
    rescan_rows_kernel<<<4 * sms, 256, 0, st>>>(key, qhi, qnorm, probed, qprobes, list_off, p,
                                                qcount, qbuf, cap, rb.list, rb.kbound,
                                                rb.nlisted + r);
  }
  rescan_exact_kernel<<<B, 256, 0, st>>>(key, qhi, qnorm, probed, qprobes, list_off, p, S, qcount,
                                         qbuf, cap);
  KATO_LAUNCHED("overflow rescan kernels");
  return KATO_OK;
}

}  // namespace kato
