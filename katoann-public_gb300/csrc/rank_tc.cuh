// Declarations shared by the tensor-core ranking pass (rank_tc.cu) and the
// search orchestration (search.cu).
#pragma once

#include <atomic>

#include <cstdint>

#include "kcommon.cuh"

namespace kato {

// One work item: a list and up to N of the queries that probe it (probe
// entries [off[list] + qfirst, +N)); its tiles are the list's rows, 128 each.
struct TcItem {
  uint32_t list, qfirst, row0, nrows;
};

struct RankTcArgs {
  const uint8_t *qhi;        // B x dc query high bytes
  const int64_t *qnorm;      // per query: sum of squared high bytes over the h ranking dimensions
  const uint32_t *entries;   // probe slots (query * nprobe + rank) grouped by list
  const uint32_t *off;       // nlist + 1
  const TcItem *items;
  const uint32_t *tile_off;  // per item: first global tile; [nitems] = total tiles
  const uint32_t *cost_off;  // per item: first cost unit; [nitems] = total (null: split by tiles)
  const uint32_t *nitems;
  const int32_t *bound;      // per query: rows with a larger l2 cannot be selected
  uint32_t *qcount;          // per query: candidates found (bit 31: some were dropped)
  uint4 *rec;                // per CTA: rec_cap candidate records (query, l2, row)
  uint32_t *rec_n;           // per CTA: records written
  uint32_t rec_cap;
  uint32_t *timeouts;        // CTAs whose bounded pipeline wait ran out
  unsigned long long *counters;  // [0] 128-row tiles scored, [1] candidates found
  unsigned long long *prof;      // optional: 14 cycle counters of the warp roles
  uint32_t dc, h, nprobe;
  long long wait;            // cycles a pipeline wait may take before the CTA gives up
  DistScale scale;
};

// Launch shape: N queries per item (the MMA's N), Bs query buffers, Rs
// raw-tile stages of `inner` bytes per row, TMEM columns.
struct TcShape {
  uint32_t N, Bs, Rs, inner, smem, tcols;
};

// Shared-memory carve-up of the ranking CTA.
struct TcSmem {
  uint32_t raw, a, b, qinfo, qbv, width, sxn, bars, tbase, err, rcount, total;
};

__host__ __device__ inline uint32_t tc_take(uint32_t &o, uint32_t bytes, uint32_t align) {
  o = (o + align - 1) / align * align;
  const uint32_t at = o;
  o += bytes;
  return at;
}

constexpr uint32_t kTcRows = 128;                        // rows per tile (the MMA's M)
// Two A stages and two accumulators: four A stages (TMEM has the columns)
// measured no faster at 10M (1.234 against 1.221 ms for the pass).
constexpr uint32_t kTcAStages = 2;                       // converted row chunks (TMEM)
constexpr uint32_t kTcAcc = 2;                           // accumulator slots (TMEM)
constexpr uint32_t kTcATile = kTcRows * 128 * 2;         // 128 rows x 128 dims of fp16
constexpr uint32_t kTcQInfo = 16;                        // bytes per query slot
constexpr uint32_t kTcBars = 8 + 2 * kTcAStages + 4 + 3 * kTcAcc + 1;  // barrier slots

__host__ __device__ inline TcSmem tc_smem_layout(uint32_t h, const TcShape &s) {
  TcSmem L{};
  uint32_t o = 0;
  L.raw = tc_take(o, s.Rs * kTcRows * s.inner, 1024);
  L.a = tc_take(o, 0, 1024);  // the A stages live in tensor memory
  L.b = tc_take(o, s.Bs * s.N * h * 2, 128);
  L.qinfo = tc_take(o, s.Bs * s.N * kTcQInfo, 16);
  L.qbv = tc_take(o, s.Bs * s.N * 4, 16);
  L.width = tc_take(o, 2 * 4, 16);
  L.sxn = tc_take(o, kTcAcc * 2 * kTcRows * 4, 16);
  L.bars = tc_take(o, kTcBars * 8, 8);
  L.tbase = tc_take(o, 4, 4);
  L.err = tc_take(o, 4, 4);
  L.rcount = tc_take(o, 4, 4);
  L.total = (o + 127) / 128 * 128;
  return L;
}

// The shape for h ranking dimensions over rows of dc bytes, or false when h
// does not suit the pass (the caller then uses the CUDA-core pass).
bool rank_tc_plan(uint32_t h, uint32_t dc, TcShape *s);
// One CTA per SM walks an equal share of all tiles.
int rank_tc(const RankTcArgs &A, const uint8_t *xhi, uint32_t npts, const TcShape &s,
            cudaStream_t st);
// Per query, an upper bound on its final S-th ranking l2 from the first
// `rows` rows (at most 4096) of its probed lists in probe order.
int rank_seed(const uint8_t *xhi, const int64_t *xnorm, const uint8_t *qhi, const int64_t *qnorm,
              const uint32_t *probed, const uint32_t *qprobes, const uint32_t *list_off,
              uint32_t L, uint32_t B, uint32_t p, uint32_t dc, uint32_t h, uint32_t S,
              uint32_t rows, uint32_t *order, int32_t *bound, cudaStream_t st);
// Work items of the pass (per list: groups of N queries) and their tile
// offsets; also zeroes the B candidate counts and buffer fills. With
// beta > 0, also per-item cost offsets: a tile of an item of MMA width w
// costs 64 + beta * w, and the CTAs split the cost instead of the tiles.
// scratch: 3 x (L + 1) words.
int rank_tc_prepare(const uint32_t *cnt, const uint32_t *list_off, uint32_t L, uint32_t N,
                    uint32_t B, uint32_t beta, uint32_t *scratch, TcItem *items,
                    uint32_t *tile_off, uint32_t *cost_off, uint32_t *nitems, uint32_t *qcount,
                    uint32_t *qfill, unsigned long long *tile_hist, cudaStream_t st);
// Process-wide knobs of the pass (0 = default): the largest item width and
// the cost weight of the CTA split.
extern std::atomic<uint32_t> g_tc_width, g_tc_beta;
// The pass's bounded pipeline waits give up after this many cycles (0: the
// default of 4e9, about 2 s); a CTA that gives up is counted in stats[3].
extern std::atomic<unsigned long long> g_tc_wait;
// Candidate records of the pass into per-query buffers of cap entries
// (distance bits, row); qfill counts the entries each query was offered.
int rank_tc_bucket(const uint4 *rec, const uint32_t *rec_n, uint32_t rec_cap, uint32_t ctas,
                   uint32_t *qfill, uint2 *qbuf, uint32_t cap, DistScale scale, cudaStream_t st);
// CTAs of rank_tc (one per SM).
uint32_t rank_tc_ctas();

// Scratch of the overflow rescan: B listed queries, B 64-bit key bounds, and
// one listed-query count per round.
struct RescanBufs {
  uint32_t *list;
  unsigned long long *kbound;
  uint32_t *nlisted;
  const uint32_t *qfill;  // entries the buffers were offered by the bucketing step
};
constexpr uint32_t kRescanCounters = 4;

// The queries whose candidate buffer overflowed are rescanned from the lists
// (rare): afterwards their buffers hold every row that can be selected.
// stats[0] counts them, stats[1] is the largest candidate count of a query.
int rank_overflow(const uint8_t *xhi, const int64_t *xnorm, const uint32_t *ids,
                  const uint8_t *qhi, const int64_t *qnorm, const uint32_t *probed,
                  const uint32_t *qprobes, const uint32_t *list_off, uint32_t B, uint32_t p,
                  uint32_t dc, uint32_t h,
                  uint32_t S, DistScale scale, uint32_t *qcount, uint2 *qbuf, uint32_t cap,
                  const RescanBufs &rb, unsigned long long *stats, cudaStream_t st);

}  // namespace kato
