// The batched search pipeline after the coarse step: inversion of the probe
// lists, the ranking pass, the survivor merge and the exact refinement.
//
// Reference: Index::search_sq16_ranked_ (src/index.cpp:909-1128) and
// Index::search_sq16_full_ (:1131-1219). The reference inverts the probe
// lists into a hash map (invert, :403-412) and scans each probed list once
// for all the queries that probe it (:998-1044); here the inversion is a CSR
// built with a histogram, a scan and an atomic scatter, and each CTA of the
// ranking kernel takes one list and up to kQG of its queries, stages the
// list's rows in shared memory tile by tile and keeps, per query, the best S
// candidates by (distance, id) in shared memory. Selection by (distance, id)
// is the reference's Selection::kLocal result (:101-135 then :1063-1069) and
// its kThreshold result wherever that has no tie on the survivor boundary.
#include <algorithm>
#include <atomic>
#include <vector>

#include <cuda_fp16.h>

#include "kcommon.cuh"
#include "probe.cuh"
#include "rank_tc.cuh"
#include "scan.cuh"

namespace kato {

thread_local uint32_t g_launches = 0;  // kernel launches of the last search pass
// Entries per query of the tensor-core ranking pass's candidate buffer.
std::atomic<uint32_t> g_candidate_cap{32768};
// Rows a query's seed bound looks at (0: max(2048, 16 survivors)).
std::atomic<uint32_t> g_seed_rows{0};

namespace {

constexpr int kQG = 16;            // queries per ranking work item
constexpr int kRT = 16;            // list rows per ranking tile
constexpr uint32_t kChunk = 1024;  // bytes of a row staged at once
constexpr uint32_t kSelMax = 256;  // largest per-slot S kept in shared memory
constexpr uint32_t kEmpty = 0xFFFFFFFFu;
constexpr int kThreads = 256;
constexpr uint32_t kSortMax = 4096;

struct Work {
  uint32_t list, first;
};

// ---------------------------------------------------------------- inversion
// A (query, rank) pair i = query * p + rank is probed when the query's
// budget (if any) exceeds the rank: its p nearest lists are in order, so a
// budget of b probes exactly the lists a fixed nprobe of b would.
__device__ __forceinline__ bool probed_pair(uint32_t i, uint32_t p,
                                            const uint32_t *__restrict__ qprobes) {
  return !qprobes || i % p < qprobes[i / p];
}

__global__ void count_kernel(const uint32_t *__restrict__ probed, uint32_t total, uint32_t p,
                             const uint32_t *__restrict__ qprobes, uint32_t *__restrict__ cnt) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < total && probed_pair(i, p, qprobes)) atomicAdd(&cnt[probed[i]], 1u);
}

// One CTA: exclusive scans of the per-list query counts (off) and of the
// per-list work-item counts (woff); clears the scatter cursors.
__global__ void __launch_bounds__(1024) scan_kernel(const uint32_t *__restrict__ cnt, uint32_t L,
                                                    uint32_t *__restrict__ off,
                                                    uint32_t *__restrict__ woff,
                                                    uint32_t *__restrict__ cursor) {
  const uint2 tot = block_scan2(
      L,
      [&](uint32_t c) {
        const uint32_t v = cnt[c];
        return make_uint2(v, (v + kQG - 1) / kQG);
      },
      [&](uint32_t c, uint32_t a, uint32_t b) {
        off[c] = a;
        woff[c] = b;
        cursor[c] = 0;
      });
  if (threadIdx.x == 0) {
    off[L] = tot.x;
    woff[L] = tot.y;
  }
}

__global__ void scatter_kernel(const uint32_t *__restrict__ probed, uint32_t total, uint32_t p,
                               const uint32_t *__restrict__ qprobes,
                               const uint32_t *__restrict__ off, uint32_t *__restrict__ cursor,
                               uint32_t *__restrict__ entries) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total || !probed_pair(i, p, qprobes)) return;
  const uint32_t c = probed[i];
  entries[off[c] + atomicAdd(&cursor[c], 1u)] = i;  // i = query * nprobe + rank
}

__global__ void work_kernel(const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ woff,
                            uint32_t L, Work *__restrict__ work) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L) return;
  const uint32_t nw = (cnt[c] + kQG - 1) / kQG;
  for (uint32_t j = 0; j < nw; ++j) work[woff[c] + j] = Work{c, j * kQG};
}

// ------------------------------------------------------------- ranking pass
struct RankArgs {
  const uint8_t *xhi, *xlo;
  const int64_t *xnorm;  // per row norm matching the mode
  const uint32_t *ids, *list_off;
  const uint8_t *qhi, *qlo;
  const int64_t *qnorm;  // per query norm matching the mode
  const Work *work;
  const uint32_t *woff_total;
  const uint32_t *off, *entries;
  uint32_t dc, dims, nprobe, S, SC;
  uint2 *slots;  // (query * nprobe + rank) * SC entries of (key, row)
  DistScale scale;
};

__host__ __device__ inline size_t rank_smem_bytes(int planes, bool select, uint32_t dims,
                                                  uint32_t S) {
  const uint32_t qw = dims / 4 + 1, kch = dims < kChunk ? dims : kChunk, rw = kch / 4 + 1;
  size_t b = static_cast<size_t>(planes) * kQG * qw * 4 + static_cast<size_t>(planes) * kRT * rw * 4;
  b += kRT * 4 + 3 * kQG * 4;           // sids, ccount, bcount, query ids
  b = (b + 15) / 16 * 16;
  b += kQG * 8;                         // query norms
  if (select) b += static_cast<size_t>(kQG) * S * 12 + static_cast<size_t>(kQG) * kRT * 12;
  return b;
}

// kFull: four products over dc (Ranking::kFull); otherwise high bytes over
// `dims` (kHighBytes: dims = dc; kPrefix: dims = head dims).
// kSelect: keep the best S per (query, list) in shared memory (S <= kSelMax);
// otherwise write every candidate to its slot (slot capacity >= list size).
template <bool kFull, bool kSelect>
__global__ void __launch_bounds__(kThreads) rank_kernel(RankArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t w = blockIdx.x;
  if (w >= *A.woff_total) return;
  const Work wk = A.work[w];
  const uint32_t c = wk.list;
  const uint32_t e0 = A.off[c] + wk.first;
  const uint32_t ne = min(static_cast<uint32_t>(kQG), A.off[c + 1] - e0);
  const uint32_t r0 = A.list_off[c], nrows = A.list_off[c + 1] - r0;
  const uint32_t dims = A.dims, qw = dims / 4 + 1;
  const uint32_t kch = min(dims, kChunk), rw = kch / 4 + 1;
  constexpr int kPlanes = kFull ? 2 : 1;
  const uint32_t S = A.S;

  uint32_t *sq = reinterpret_cast<uint32_t *>(smem);   // [planes][kQG][qw]
  uint32_t *sr = sq + kPlanes * kQG * qw;              // [planes][kRT][rw]
  uint32_t *sids = sr + kPlanes * kRT * rw;            // [kRT]
  uint32_t *ccount = sids + kRT;                       // [kQG]
  uint32_t *bcount = ccount + kQG;                     // [kQG]
  uint32_t *sslot = bcount + kQG;                      // [kQG]
  size_t off = (reinterpret_cast<unsigned char *>(sslot + kQG) - smem + 15) / 16 * 16;
  int64_t *sqn = reinterpret_cast<int64_t *>(smem + off);                      // [kQG]
  unsigned long long *bkid = reinterpret_cast<unsigned long long *>(sqn + kQG);  // [kQG][S]
  unsigned long long *ckid = bkid + (kSelect ? kQG * S : 0);                   // [kQG][kRT]
  uint32_t *brow = reinterpret_cast<uint32_t *>(ckid + (kSelect ? kQG * kRT : 0));  // [kQG][S]
  uint32_t *crow = brow + (kSelect ? kQG * S : 0);                             // [kQG][kRT]

  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int j = t & 15, rr = t >> 4;
  if (t < kQG) {
    ccount[t] = 0;
    bcount[t] = 0;
    sslot[t] = t < static_cast<int>(ne) ? A.entries[e0 + t] : 0;
  }
  __syncthreads();
  if (t < static_cast<int>(ne)) sqn[t] = A.qnorm[sslot[t] / A.nprobe];
  // Stage the queries' bytes (16-byte loads; dims is a multiple of 64).
  const uint32_t v16 = dims / 16;
  for (uint32_t idx = t; idx < ne * v16 * kPlanes; idx += kThreads) {
    const uint32_t pl = idx / (ne * v16), rem = idx % (ne * v16);
    const uint32_t jj = rem / v16, v = rem % v16;
    const uint32_t q = sslot[jj] / A.nprobe;
    const uint8_t *src = (pl == 0 ? A.qhi : A.qlo) + static_cast<size_t>(q) * A.dc + v * 16;
    const uint4 x = *reinterpret_cast<const uint4 *>(src);
    uint32_t *dst = sq + (pl * kQG + jj) * qw + v * 4;
    dst[0] = x.x; dst[1] = x.y; dst[2] = x.z; dst[3] = x.w;
  }
  // Slots of rows past the list end are padding (store-all mode writes every row).
  if (!kSelect) {
    for (uint32_t idx = t; idx < ne * (A.SC - min(nrows, A.SC)); idx += kThreads) {
      const uint32_t jj = idx / (A.SC - nrows), pos = nrows + idx % (A.SC - nrows);
      A.slots[static_cast<size_t>(sslot[jj]) * A.SC + pos] = make_uint2(kEmpty, 0);
    }
  }
  __syncthreads();

  for (uint32_t rt = 0; rt < nrows; rt += kRT) {
    const uint32_t nr = min(static_cast<uint32_t>(kRT), nrows - rt);
    uint32_t hh = 0, mx = 0, ll = 0;
    for (uint32_t k0 = 0; k0 < dims; k0 += kch) {
      const uint32_t kc = min(kch, dims - k0), c16 = kc / 16;
      __syncthreads();
      for (uint32_t idx = t; idx < nr * c16 * kPlanes; idx += kThreads) {
        const uint32_t pl = idx / (nr * c16), rem = idx % (nr * c16);
        const uint32_t i = rem / c16, v = rem % c16;
        const uint8_t *src =
            (pl == 0 ? A.xhi : A.xlo) + static_cast<size_t>(r0 + rt + i) * A.dc + k0 + v * 16;
        const uint4 x = *reinterpret_cast<const uint4 *>(src);
        uint32_t *dst = sr + (pl * kRT + i) * rw + v * 4;
        dst[0] = x.x; dst[1] = x.y; dst[2] = x.z; dst[3] = x.w;
      }
      if (k0 == 0 && t < static_cast<int>(nr)) sids[t] = A.ids[r0 + rt + t];
      __syncthreads();
      if (j < static_cast<int>(ne) && rr < static_cast<int>(nr)) {
        const uint32_t *qa = sq + j * qw + k0 / 4;
        const uint32_t *xa = sr + rr * rw;
        const uint32_t nw = kc / 4;
        if (kFull) {
          const uint32_t *qb = sq + (kQG + j) * qw + k0 / 4;
          const uint32_t *xb = sr + (kRT + rr) * rw;
#pragma unroll 8
          for (uint32_t u = 0; u < nw; ++u) {
            const uint32_t ah = qa[u], al = qb[u], bh = xa[u], bl = xb[u];
            hh = dp4(ah, bh, hh);
            mx = dp4(ah, bl, mx);
            mx = dp4(al, bh, mx);
            ll = dp4(al, bl, ll);
          }
        } else {
#pragma unroll 8
          for (uint32_t u = 0; u < nw; ++u) hh = dp4(qa[u], xa[u], hh);
        }
      }
    }
    // The candidate of (row rr, query j).
    if (j < static_cast<int>(ne) && rr < static_cast<int>(nr)) {
      const uint32_t row = r0 + rt + rr;
      const int64_t dot = kFull ? static_cast<int64_t>((static_cast<uint64_t>(hh) << 16) +
                                                       (static_cast<uint64_t>(mx) << 8) + ll)
                                : static_cast<int64_t>(hh);
      const float dist = dist_value(sqn[j] + A.xnorm[row] - 2 * dot, A.scale);
      const uint32_t key = __float_as_uint(dist);
      if (kSelect) {
        const unsigned long long kid = (static_cast<unsigned long long>(key) << 32) | sids[rr];
        const unsigned long long thr = bcount[j] == S ? bkid[j * S + S - 1] : ~0ull;
        if (kid < thr) {
          const uint32_t pos = atomicAdd(&ccount[j], 1u);
          ckid[j * kRT + pos] = kid;
          crow[j * kRT + pos] = row;
        }
      } else {
        A.slots[static_cast<size_t>(sslot[j]) * A.SC + rt + rr] = make_uint2(key, row);
      }
    }
    if (kSelect) {
      __syncthreads();
      // Merge each query's new candidates (at most kRT, unsorted) into its
      // sorted best list: one warp per query.
      for (int jj = warp; jj < static_cast<int>(ne); jj += kThreads / 32) {
        const uint32_t nc = ccount[jj];
        if (nc == 0) continue;
        const uint32_t nb = bcount[jj];
        unsigned long long *B = bkid + jj * S;
        uint32_t *Br = brow + jj * S;
        const unsigned long long ck = lane < static_cast<int>(nc) ? ckid[jj * kRT + lane] : ~0ull;
        const uint32_t cr = lane < static_cast<int>(nc) ? crow[jj * kRT + lane] : 0;
        // rank of this candidate among the candidates (ties by lane)
        uint32_t crank = 0;
        for (uint32_t i = 0; i < nc; ++i) {
          const unsigned long long o = __shfl_sync(0xffffffffu, ck, i);
          crank += (o < ck) || (o == ck && static_cast<int>(i) < lane);
        }
        // number of best entries <= candidate (upper bound)
        uint32_t lo = 0, hi = nb;
        while (lo < hi) {
          const uint32_t mid = (lo + hi) >> 1;
          if (B[mid] <= ck) lo = mid + 1;
          else hi = mid;
        }
        const uint32_t cpos = lo + crank;
        // new index of each old entry
        constexpr int kPer = kSelMax / 32;
        unsigned long long okid[kPer];
        uint32_t orow[kPer], onew[kPer];
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
          const uint32_t b = lane + 32 * u;
          okid[u] = b < nb ? B[b] : ~0ull;
          orow[u] = b < nb ? Br[b] : 0;
          onew[u] = b < nb ? b : 0xFFFFFFFFu;
        }
        for (uint32_t i = 0; i < nc; ++i) {
          const unsigned long long o = __shfl_sync(0xffffffffu, ck, i);
#pragma unroll
          for (int u = 0; u < kPer; ++u) onew[u] += (onew[u] != 0xFFFFFFFFu && o < okid[u]);
        }
        __syncwarp();
#pragma unroll
        for (int u = 0; u < kPer; ++u)
          if (onew[u] < S) {
            B[onew[u]] = okid[u];
            Br[onew[u]] = orow[u];
          }
        if (lane < static_cast<int>(nc) && cpos < S) {
          B[cpos] = ck;
          Br[cpos] = cr;
        }
        __syncwarp();
        if (lane == 0) {
          bcount[jj] = min(S, nb + nc);
          ccount[jj] = 0;
        }
      }
      __syncthreads();
    }
  }
  if (kSelect) {
    for (uint32_t idx = t; idx < ne * S; idx += kThreads) {
      const uint32_t jj = idx / S, i = idx % S;
      uint2 v = make_uint2(kEmpty, 0);
      if (i < bcount[jj]) v = make_uint2(static_cast<uint32_t>(bkid[jj * S + i] >> 32), brow[jj * S + i]);
      A.slots[static_cast<size_t>(sslot[jj]) * A.SC + i] = v;
    }
  }
}

// ---------------------------------------------------- block selection helper
// Chooses the `p` smallest of n entries by (key, id), where entry i gives
// key = K(i) and id = I(i); keys == kEmpty are never chosen. Writes the chosen
// (key << 32 | id, position) pairs into sel/pos (unsorted) and returns how
// many were chosen (min(p, non-empty)). Radix selection over 8-bit digits,
// first of the key, then of the id among the entries tied at the boundary key.
template <class KeyF, class IdF>
__device__ uint32_t block_select(uint32_t n, uint32_t p, KeyF K, IdF I, unsigned long long *sel,
                                 uint32_t *pos, uint32_t *hist, uint32_t *scratch, uint32_t *wsum,
                                 bool *boundary_tie) {
  const uint32_t tid = threadIdx.x, nt = blockDim.x;
  // count non-empty
  if (tid == 0) scratch[0] = 0;
  __syncthreads();
  {
    uint32_t m = 0;
    for (uint32_t i = tid; i < n; i += nt) m += K(i) != kEmpty;
    atomicAdd(&scratch[0], m);
  }
  __syncthreads();
  const uint32_t valid = scratch[0];
  __syncthreads();
  const uint32_t want = min(p, valid);
  *boundary_tie = false;
  if (want == 0) return 0;
  uint32_t T = kEmpty, idmax = 0xFFFFFFFFu;
  if (want < valid) {
    // radix select of the want-th key
    uint32_t prefix = 0, rank = want - 1;
    for (int shift = 24; shift >= 0; shift -= 8) {
      for (uint32_t i = tid; i < 256; i += nt) hist[i] = 0;
      __syncthreads();
      const uint32_t hm = shift == 24 ? 0u : (0xFFFFFFFFu << (shift + 8));
      for (uint32_t i = tid; i < n; i += nt) {
        const uint32_t k = K(i);
        if (k != kEmpty && (k & hm) == prefix) atomicAdd(&hist[(k >> shift) & 0xFFu], 1u);
      }
      __syncthreads();
      block_pick_digit(hist, rank, scratch + 1, wsum);
      rank -= scratch[2];
      prefix |= scratch[1] << shift;
      __syncthreads();
    }
    T = prefix;
    const uint32_t need = rank + 1;
    if (tid == 0) scratch[3] = 0;
    __syncthreads();
    {
      uint32_t m = 0;
      for (uint32_t i = tid; i < n; i += nt) m += K(i) == T;
      atomicAdd(&scratch[3], m);
    }
    __syncthreads();
    const uint32_t neq = scratch[3];
    *boundary_tie = neq > need;
    if (neq > need) {
      uint32_t ip = 0, ir = need - 1;
      for (int shift = 24; shift >= 0; shift -= 8) {
        for (uint32_t i = tid; i < 256; i += nt) hist[i] = 0;
        __syncthreads();
        const uint32_t hm = shift == 24 ? 0u : (0xFFFFFFFFu << (shift + 8));
        for (uint32_t i = tid; i < n; i += nt) {
          if (K(i) != T) continue;
          const uint32_t id = I(i);
          if ((id & hm) == ip) atomicAdd(&hist[(id >> shift) & 0xFFu], 1u);
        }
        __syncthreads();
        block_pick_digit(hist, ir, scratch + 1, wsum);
        ir -= scratch[2];
        ip |= scratch[1] << shift;
        __syncthreads();
      }
      idmax = ip;
    }
  }
  if (tid == 0) scratch[4] = 0;
  __syncthreads();
  for (uint32_t i = tid; i < n; i += nt) {
    const uint32_t k = K(i);
    if (k == kEmpty) continue;
    bool take = k < T;
    uint32_t id = 0;
    if (!take && k == T) {
      id = I(i);
      take = id <= idmax;
    } else if (take) {
      id = I(i);
    }
    if (take) {
      const uint32_t at = atomicAdd(&scratch[4], 1u);
      if (at < want) {
        sel[at] = (static_cast<unsigned long long>(k) << 32) | id;
        pos[at] = i;
      }
    }
  }
  __syncthreads();
  return want;
}

// In-shared-memory bitonic sort of n (key, payload) pairs, ascending by key.
__device__ void block_sort_pairs(unsigned long long *key, uint32_t *val, uint32_t n) {
  uint32_t np2 = 1;
  while (np2 < n) np2 <<= 1;
  for (uint32_t i = n + threadIdx.x; i < np2; i += blockDim.x) {
    key[i] = ~0ull;
    val[i] = 0;
  }
  __syncthreads();
  for (uint32_t size = 2; size <= np2; size <<= 1)
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t i = threadIdx.x; i < np2; i += blockDim.x) {
        const uint32_t jx = i ^ stride;
        if (jx > i) {
          const bool up = (i & size) == 0;
          const unsigned long long a = key[i], b = key[jx];
          if ((a > b) == up) {
            key[i] = b;
            key[jx] = a;
            const uint32_t tv = val[i];
            val[i] = val[jx];
            val[jx] = tv;
          }
        }
      }
      __syncthreads();
    }
}

// -------------------------------------------------------------------- merge
// Per query: the best S of its nprobe * SC slot entries (or of the first
// qcount[q] entries of its candidate buffer) by (distance, id).
// Ranked modes write the survivors in descending (distance, id) order - the
// order in which the reference pops its merged heap into the refinement
// (:1088-1112). The full mode writes the final top-k, ascending, padded.
__global__ void __launch_bounds__(kThreads) merge_kernel(
    const uint2 *__restrict__ slots, uint32_t per_query, const uint32_t *__restrict__ qcount,
    const uint32_t *__restrict__ qprobes, uint32_t per_probe, const uint32_t *__restrict__ ids,
    uint32_t S, bool final_topk, uint32_t k, uint2 *__restrict__ surv, uint32_t *__restrict__ nsurv,
    uint32_t *__restrict__ out_ids, float *__restrict__ out_dists,
    unsigned long long *__restrict__ tie_count) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t hist[256], scratch[8], wsum[8];
  __shared__ bool tie;
  unsigned long long *sel = reinterpret_cast<unsigned long long *>(smem);
  uint32_t np2 = 1;
  while (np2 < S) np2 <<= 1;
  uint32_t *pos = reinterpret_cast<uint32_t *>(sel + np2);
  const uint32_t q = blockIdx.x;
  const uint2 *e = slots + static_cast<size_t>(q) * per_query;
  // the tensor-core pass counts each query's candidates; on the CUDA-core
  // pass a query's slots are its probes' (rank-major), of which the first
  // budget ones were written
  const uint32_t n = qcount    ? min(qcount[q], per_query)
                     : qprobes ? min(per_query, qprobes[q] * per_probe)
                               : per_query;
  auto K = [&](uint32_t i) { return e[i].x; };
  auto I = [&](uint32_t i) { return ids[e[i].y]; };
  const uint32_t got = block_select(n, S, K, I, sel, pos, hist, scratch, wsum, &tie);
  if (threadIdx.x == 0 && tie && tie_count) atomicAdd(tie_count, 1ull);
  block_sort_pairs(sel, pos, got);
  if (final_topk) {
    for (uint32_t i = threadIdx.x; i < k; i += blockDim.x) {
      uint32_t id = 0xFFFFFFFFu;
      float dd = 3.402823466e+38f;
      if (i < got) {
        id = static_cast<uint32_t>(sel[i] & 0xFFFFFFFFu);
        dd = __uint_as_float(static_cast<uint32_t>(sel[i] >> 32));
      }
      out_ids[static_cast<size_t>(q) * k + i] = id;
      out_dists[static_cast<size_t>(q) * k + i] = dd;
    }
    return;
  }
  for (uint32_t i = threadIdx.x; i < got; i += blockDim.x) {
    const uint32_t src = got - 1 - i;  // descending
    surv[static_cast<size_t>(q) * S + i] = e[pos[src]];
  }
  if (threadIdx.x == 0) nsurv[q] = got;
}

// ------------------------------------------------------------------- refine
// Per query: exact distances of the survivors (in the order given), then the
// reference's top-k heap: the first k enter, later ones replace the largest
// (distance, id) when their distance is strictly smaller (:1113-1124); output
// ascending by (distance, id), padded (emit_topk, :384-398).
__global__ void __launch_bounds__(kThreads, 4) refine_kernel(
    const uint8_t *__restrict__ qhi, const uint8_t *__restrict__ qlo,
    const int64_t *__restrict__ qnorm, const uint8_t *__restrict__ xhi,
    const uint8_t *__restrict__ xlo, const int64_t *__restrict__ xnorm,
    const uint32_t *__restrict__ ids, uint32_t npts, uint32_t dc, const uint2 *__restrict__ surv,
    const uint32_t *__restrict__ nsurv, uint32_t S, uint32_t k, DistScale scale,
    uint32_t *__restrict__ out_ids, float *__restrict__ out_dists) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t q = blockIdx.x, ns = nsurv[q];
  const uint32_t n16 = dc / 16;                        // 16-byte words of a plane row
  uint4 *sq = reinterpret_cast<uint4 *>(smem);         // [2][n16]
  float *ex = reinterpret_cast<float *>(sq + 2 * n16);  // [S]
  uint32_t *eid = reinterpret_cast<uint32_t *>(ex + S);  // [S]
  float *hd = reinterpret_cast<float *>(eid + S);      // [k]
  uint32_t *hid = reinterpret_cast<uint32_t *>(hd + k);  // [k]
  uint32_t *srow = hid + k;                             // [S] the survivors' rows
  for (uint32_t i = threadIdx.x; i < n16; i += blockDim.x) {
    sq[i] = reinterpret_cast<const uint4 *>(qhi + static_cast<size_t>(q) * dc)[i];
    sq[n16 + i] = reinterpret_cast<const uint4 *>(qlo + static_cast<size_t>(q) * dc)[i];
  }
  for (uint32_t i = threadIdx.x; i < ns; i += blockDim.x)
    srow[i] = surv[static_cast<size_t>(q) * S + i].y;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nwarps = blockDim.x / 32;
  const int64_t qn = qnorm[q];
  // one survivor per warp step, its row loads issued before the products (a
  // smaller register set than two survivors per step: four CTAs per SM)
  for (uint32_t s0 = warp; s0 < ns; s0 += nwarps) {
    const uint32_t r0 = srow[s0];
    uint32_t id0 = 0;
    int64_t xn0 = 0;
    if (lane == 0) {
      id0 = ids[r0];
      xn0 = xnorm[r0];
    }
    const uint4 *h0 = reinterpret_cast<const uint4 *>(xhi + static_cast<size_t>(r0) * dc);
    const uint4 *l0 = reinterpret_cast<const uint4 *>(xlo + static_cast<size_t>(r0) * dc);
    uint32_t hh0 = 0, mx0 = 0, ll0 = 0;
#pragma unroll 2
    for (uint32_t u = lane; u < n16; u += 32) {
      const uint4 bh0 = h0[u], bl0 = l0[u];
      const uint4 ah = sq[u], al = sq[n16 + u];
      const uint32_t a_h[4] = {ah.x, ah.y, ah.z, ah.w}, a_l[4] = {al.x, al.y, al.z, al.w};
      const uint32_t b_h0[4] = {bh0.x, bh0.y, bh0.z, bh0.w}, b_l0[4] = {bl0.x, bl0.y, bl0.z, bl0.w};
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        hh0 = dp4(a_h[w], b_h0[w], hh0);
        mx0 = dp4(a_h[w], b_l0[w], mx0);
        mx0 = dp4(a_l[w], b_h0[w], mx0);
        ll0 = dp4(a_l[w], b_l0[w], ll0);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      hh0 += __shfl_xor_sync(0xffffffffu, hh0, o);
      mx0 += __shfl_xor_sync(0xffffffffu, mx0, o);
      ll0 += __shfl_xor_sync(0xffffffffu, ll0, o);
    }
    if (lane == 0) {
      const int64_t dot0 = static_cast<int64_t>((static_cast<uint64_t>(hh0) << 16) +
                                                (static_cast<uint64_t>(mx0) << 8) + ll0);
      ex[s0] = dist_value(qn + xn0 - 2 * dot0, scale);
      eid[s0] = id0;
    }
  }
  __syncthreads();
  // The reference's heap (:1113-1124), survivors in the given order: the
  // first k enter; a later one replaces the largest (distance, id) when its
  // distance is strictly smaller; then ascending by (distance, id).
  if (k <= 32) {
    // one warp holds the heap sorted descending by (distance, id) across its
    // lanes - lane 0 is the largest, the one the reference evicts - so an
    // insertion is one ballot and one shift; unused lanes sort below all
    if (warp != 0) return;
    const uint32_t u = static_cast<uint32_t>(lane);
    float d = -1.0f;
    uint32_t id = 0u, n = 0;
    for (uint32_t s = 0; s < ns; ++s) {
      const float dd = ex[s];
      const uint32_t ii = eid[s];
      if (ii >= npts) continue;  // ids without a row are skipped (:1091-1094)
      const bool gt = d > dd || (d == dd && id > ii);  // this slot sorts above the new one
      if (n < k) {
        // enters after the g larger ones; the rest move up one lane
        const uint32_t g = __popc(__ballot_sync(0xffffffffu, gt && u < n));
        const float ud = __shfl_up_sync(0xffffffffu, d, 1);
        const uint32_t uid = __shfl_up_sync(0xffffffffu, id, 1);
        if (u == g) {
          d = dd;
          id = ii;
        } else if (u > g && u <= n) {
          d = ud;
          id = uid;
        }
        ++n;
        continue;
      }
      if (!(dd < __shfl_sync(0xffffffffu, d, 0))) continue;  // strictly below the largest
      // the largest leaves; the g larger ones below it move down one lane
      const uint32_t g = __popc(__ballot_sync(0xffffffffu, gt && u >= 1 && u < k));
      const float nd = __shfl_down_sync(0xffffffffu, d, 1);
      const uint32_t nid = __shfl_down_sync(0xffffffffu, id, 1);
      if (u < g) {
        d = nd;
        id = nid;
      } else if (u == g) {
        d = dd;
        id = ii;
      }
    }
    if (u < n) {  // ascending: lane u is the (n - 1 - u)-th
      out_ids[static_cast<size_t>(q) * k + (n - 1 - u)] = id;
      out_dists[static_cast<size_t>(q) * k + (n - 1 - u)] = d;
    } else if (u < k) {
      out_ids[static_cast<size_t>(q) * k + u] = 0xFFFFFFFFu;
      out_dists[static_cast<size_t>(q) * k + u] = 3.402823466e+38f;
    }
    return;
  }
  if (threadIdx.x == 0) {
    uint32_t n = 0;
    for (uint32_t s = 0; s < ns; ++s) {
      const float dd = ex[s];
      const uint32_t id = eid[s];
      if (id >= npts) continue;  // ids without a row are skipped (:1091-1094)
      if (n < k) {
        hd[n] = dd;
        hid[n] = id;
        ++n;
        continue;
      }
      uint32_t mi = 0;  // the largest (distance, id)
      for (uint32_t i = 1; i < n; ++i)
        if (hd[i] > hd[mi] || (hd[i] == hd[mi] && hid[i] > hid[mi])) mi = i;
      if (dd < hd[mi]) {
        hd[mi] = dd;
        hid[mi] = id;
      }
    }
    // ascending by (distance, id)
    for (uint32_t i = 1; i < n; ++i) {
      const float d0 = hd[i];
      const uint32_t i0 = hid[i];
      uint32_t m = i;
      while (m > 0 && (hd[m - 1] > d0 || (hd[m - 1] == d0 && hid[m - 1] > i0))) {
        hd[m] = hd[m - 1];
        hid[m] = hid[m - 1];
        --m;
      }
      hd[m] = d0;
      hid[m] = i0;
    }
    for (uint32_t i = 0; i < k; ++i) {
      out_ids[static_cast<size_t>(q) * k + i] = i < n ? hid[i] : 0xFFFFFFFFu;
      out_dists[static_cast<size_t>(q) * k + i] = i < n ? hd[i] : 3.402823466e+38f;
    }
  }
}

}  // namespace

// ------------------------------------------------------------ orchestration
int rotate_rows(const float *in, uint32_t nrows, uint32_t d, const float *rot, float *out,
                cudaStream_t st);
int quantize_rows(const float *x, uint32_t nrows, uint32_t d, uint32_t dc, float lo,
                  double inv_step, uint32_t head, uint8_t *hi, uint8_t *lop, int64_t *norm,
                  int64_t *hinorm, int64_t *headnorm, cudaStream_t st);
int sq16_tiles(const uint8_t *qhi, const uint8_t *qlo, const uint8_t *xhi, const uint8_t *xlo,
               const int64_t *qn, const int64_t *xn, double step_sq, uint32_t m, uint32_t n,
               uint32_t dims, uint32_t qstride, uint32_t xstride, float *out, bool full,
               cudaStream_t st);
int centre_planes(const uint8_t *hi, const uint8_t *lo, const int64_t *norm, uint32_t rows,
                  uint32_t dc, __half *hi16, __half *lo16, int64_t *term, cudaStream_t st);
bool coarse_tc_ok(uint32_t dc);
int coarse_tc(const __half *ch, const __half *cl, const int64_t *cterm, uint32_t n, const __half *qh,
              const __half *ql, const int64_t *qterm, uint32_t m, uint32_t dc, double step_sq,
              float *out, uint32_t *timeouts, unsigned long long *prof, cudaStream_t st);
size_t rotate_scratch_bytes(uint32_t nrows, uint32_t d);
int rotate_rows_kmajor(const float *in, uint32_t nrows, uint32_t d, const float *rot,
                       const float *rot_kmajor, void *scratch, float *out, cudaStream_t st);
int select_topp_ex(const float *dists, uint32_t nq, uint32_t n, uint32_t p, uint32_t stride,
                   uint32_t *probed, unsigned long long *tie_count, const uint32_t *only,
                   uint32_t only_above, cudaStream_t st);

// Per pass: the KATO_PHASES + 1 phase boundaries, then a start and an end
// event around each timed kernel (KATO_TIMED_KERNELS: the query rotation,
// coarse_tc_kernel, rank_tc_kernel).
constexpr uint32_t kTimerStride = KATO_PHASES + 1 + 2 * KATO_TIMED_KERNELS;

struct PhaseTimer {
  std::vector<cudaEvent_t> ev;  // kTimerStride per pass
  std::vector<uint8_t> kdone;   // per pass: the kernels whose two events were recorded
  uint32_t max_passes = 0, used = 0;
  float kms[KATO_TIMED_KERNELS] = {};      // of the passes the last read summed
  uint32_t kn[KATO_TIMED_KERNELS] = {};
};

static void mark(PhaseTimer *t, uint32_t phase, cudaStream_t st) {
  if (!t || t->used >= t->max_passes) return;
  cudaEventRecord(t->ev[t->used * kTimerStride + phase], st);
}

static void kmark(PhaseTimer *t, uint32_t kernel, bool end, cudaStream_t st) {
  if (!t || t->used >= t->max_passes) return;
  cudaEventRecord(t->ev[t->used * kTimerStride + KATO_PHASES + 1 + 2 * kernel + end], st);
  if (end) t->kdone[t->used] |= static_cast<uint8_t>(1u << kernel);
}

struct Plan {
  uint32_t B, k, p, S, SC, dims;
  int ranking;
  bool select;
  bool tc;                          // tensor-core ranking pass
  bool coarse_tc;                   // tensor-core coarse product
  TcShape tcs;
  uint32_t tcitems, cap, seed_rows, ctas, rec_cap, beta;
  size_t off_fq, off_qhi, off_qlo, off_qn, off_qhn, off_qh0, off_cd, off_probed, off_cnt, off_off,
      off_woff, off_cur, off_work, off_ent, off_slots, off_surv, off_nsurv, off_stats,
      off_tcscratch, off_tcitems, off_tileoff, off_nitems, off_qcount, off_qfill, off_bound,
      off_rec, off_recn, off_rlist, off_rkey, off_rcount, off_qh16, off_ql16, off_qterm, off_rot,
      off_qprobes, off_z, off_costoff, off_seedorder, total;
};

static size_t align256(size_t x) { return (x + 255) / 256 * 256; }

int make_plan(const katoann_gpu_index *ix, uint32_t B, uint32_t k, uint32_t p, int ranking,
              uint32_t survivors, Plan *P) {
  if (k == 0 || p == 0 || p > ix->nlist) return invalid("need k >= 1 and 1 <= nprobe <= nlist");
  if (ranking == KATO_RANK_PREFIX && ix->head_dims == 0)
    return invalid("prefix ranking needs the rotation file (.dimc)");
  if (ranking < 0 || ranking > 2) return invalid("unknown ranking");
  Plan &pl = *P;
  pl.B = B;
  pl.k = k;
  pl.p = p;
  pl.ranking = ranking;
  pl.S = ranking == KATO_RANK_FULL ? k : std::max(survivors, k);
  if (pl.S > kSortMax) return invalid("survivors (or k) above 4096 are not supported on the GPU");
  const uint32_t ml = std::max(ix->max_list, 1u);
  pl.SC = std::min(pl.S, ml);
  pl.select = pl.SC <= kSelMax;
  if (!pl.select) pl.SC = ml;
  pl.dims = ranking == KATO_RANK_PREFIX ? ix->head_dims : ix->dc;
  const uint32_t L = ix->nlist;
  const size_t bp = static_cast<size_t>(B) * p;
  const size_t wmax = std::min<size_t>(L, bp) + bp / kQG + 1;
  // tensor-core ranking: every query's candidates within its seed bound go
  // to a buffer of `cap` entries (an overflowing query is rescanned exactly)
  pl.cap = g_candidate_cap.load();
  pl.tc = ranking != KATO_RANK_FULL && pl.S <= pl.cap && rank_tc_plan(pl.dims, ix->dc, &pl.tcs);
  if (pl.tc) {
    pl.select = true;
    pl.SC = pl.S;
    const uint32_t sr = g_seed_rows.load();
    pl.seed_rows = sr ? std::max(sr, pl.S) : std::max(2048u, 16 * pl.S);
    pl.tcitems = static_cast<uint32_t>(bp / pl.tcs.N + std::min<size_t>(L, bp) + 1);
    // candidate records per CTA: room for 32 S per query of the batch, spread
    // over the CTAs (a CTA that runs out flags the queries it drops)
    pl.ctas = rank_tc_ctas();
    pl.rec_cap = static_cast<uint32_t>(
        std::max<size_t>(8192, static_cast<size_t>(B) * pl.S * 32 / pl.ctas));
    // the cost split, unless its 32-bit cost units could overflow
    pl.beta = g_tc_beta.load();
    const uint64_t worst = static_cast<uint64_t>(pl.tcitems) * ((ix->max_list + 127) / 128) *
                           (64 + static_cast<uint64_t>(pl.beta) * pl.tcs.N);
    if (worst >= (1ull << 31)) pl.beta = 0;
  } else {
    pl.ctas = 1;
    pl.rec_cap = 0;
  }
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += align256(bytes);
    return at;
  };
  pl.off_stats = take(48 * sizeof(unsigned long long));
  pl.off_fq = take(static_cast<size_t>(B) * ix->dim * 4);
  pl.off_qhi = take(static_cast<size_t>(B) * ix->dc);
  pl.off_qlo = take(static_cast<size_t>(B) * ix->dc);
  pl.off_qn = take(static_cast<size_t>(B) * 8);
  pl.off_qhn = take(static_cast<size_t>(B) * 8);
  pl.off_qh0 = take(static_cast<size_t>(B) * 8);
  pl.off_cd = take(static_cast<size_t>(B) * L * 4);
  pl.off_probed = take(bp * 4);
  pl.off_cnt = take(static_cast<size_t>(L) * 4);
  pl.off_off = take((static_cast<size_t>(L) + 1) * 4);
  pl.off_woff = take((static_cast<size_t>(L) + 1) * 4);
  pl.off_cur = take(static_cast<size_t>(L) * 4);
  pl.off_work = take(wmax * sizeof(Work));
  pl.off_ent = take(bp * 4);
  pl.off_slots = take((pl.tc ? static_cast<size_t>(B) * pl.cap : bp * pl.SC) * sizeof(uint2));
  pl.off_tcscratch = take(3 * (static_cast<size_t>(L) + 1) * 4);
  pl.off_costoff = take(pl.tc ? (static_cast<size_t>(pl.tcitems) + 1) * 4 : 16);
  pl.off_tcitems = take(pl.tc ? (static_cast<size_t>(pl.tcitems) + 1) * sizeof(TcItem) : 16);
  pl.off_tileoff = take(pl.tc ? (static_cast<size_t>(pl.tcitems) + 1) * 4 : 16);
  pl.off_nitems = take(16);
  pl.off_qcount = take(static_cast<size_t>(B) * 4);
  pl.off_qfill = take(static_cast<size_t>(B) * 4);
  pl.off_bound = take(static_cast<size_t>(B) * 4);
  pl.off_rec = take(pl.tc ? static_cast<size_t>(pl.ctas) * pl.rec_cap * 16 : 16);
  pl.off_recn = take(static_cast<size_t>(pl.ctas) * 4);
  pl.coarse_tc = ix->d_chi16 && ix->d_clo16 && ix->d_cterm && coarse_tc_ok(ix->dc);
  pl.off_qh16 = take(pl.coarse_tc ? static_cast<size_t>(B) * ix->dc * 2 : 16);
  pl.off_ql16 = take(pl.coarse_tc ? static_cast<size_t>(B) * ix->dc * 2 : 16);
  pl.off_qterm = take(static_cast<size_t>(B) * 8);
  pl.off_rot = take(ix->rotated ? rotate_scratch_bytes(B, ix->dim) : 16);
  pl.off_rlist = take(static_cast<size_t>(B) * 4);
  pl.off_rkey = take(static_cast<size_t>(B) * 8);
  pl.off_rcount = take(kRescanCounters * 4);
  pl.off_qprobes = take(static_cast<size_t>(B) * 4);
  pl.off_seedorder = take(static_cast<size_t>(B) * 4);
  pl.off_z = take(static_cast<size_t>(B) * KATO_PROBE_FEATURES * 4);
  pl.off_surv = take(static_cast<size_t>(B) * pl.S * sizeof(uint2));
  pl.off_nsurv = take(static_cast<size_t>(B) * 4);
  pl.total = o;
  return KATO_OK;
}

// Rotation, quantization, coarse product and top-p1 selection of nq queries
// (phases 0-2): leaves the query planes, the coarse distances (cd) and each
// query's p1 nearest lists in order (probed, rows pl.p apart) in the
// workspace.
int coarse_pass(const katoann_gpu_index *ix, const Plan &pl, const float *queries, uint32_t nq,
                unsigned char *ws, uint32_t p1, cudaStream_t st, PhaseTimer *tm) {
  int rc;
  const uint32_t L = ix->nlist, p = pl.p, dc = ix->dc;
  float *fq = reinterpret_cast<float *>(ws + pl.off_fq);
  uint8_t *qhi = ws + pl.off_qhi, *qlo = ws + pl.off_qlo;
  int64_t *qn = reinterpret_cast<int64_t *>(ws + pl.off_qn);
  int64_t *qhn = reinterpret_cast<int64_t *>(ws + pl.off_qhn);
  int64_t *qh0 = reinterpret_cast<int64_t *>(ws + pl.off_qh0);
  float *cd = reinterpret_cast<float *>(ws + pl.off_cd);
  uint32_t *probed = reinterpret_cast<uint32_t *>(ws + pl.off_probed);
  unsigned long long *stats = reinterpret_cast<unsigned long long *>(ws + pl.off_stats);

  mark(tm, 0, st);
  // 1. rotation and quantization of the queries (src/index.cpp:895-899, :917-943)
  const float *src = queries;
  if (ix->rotated) {
    kmark(tm, 0, false, st);
    if ((rc = rotate_rows_kmajor(queries, nq, ix->dim, ix->d_rotation, ix->d_rotation_t,
                                 ws + pl.off_rot, fq, st)))
      return rc;
    kmark(tm, 0, true, st);
    src = fq;
  }
  if ((rc = quantize_rows(src, nq, ix->dim, dc, ix->lo, ix->inv_step, ix->head_dims, qhi, qlo, qn,
                          qhn, qh0, st)))
    return rc;
  // rotation (the queries' transpose, the rotation's unless the index holds
  // its k-major copy, and the product, plus the d % 4 columns), quantize,
  // coarse, select
  g_launches += (ix->rotated ? ((ix->dim & ~15u) ? (ix->d_rotation_t ? 2 : 3) : 1) +
                                   ((ix->dim & 3) ? 1 : 0)
                             : 0) +
                1 + 2;
  mark(tm, 1, st);
  // 2. coarse product and top-nprobe (:846-877)
  if (pl.coarse_tc) {
    // fp16 tensor cores: the queries' centred planes, then the exact product
    __half *qh16 = reinterpret_cast<__half *>(ws + pl.off_qh16);
    __half *ql16 = reinterpret_cast<__half *>(ws + pl.off_ql16);
    int64_t *qterm = reinterpret_cast<int64_t *>(ws + pl.off_qterm);
    if ((rc = centre_planes(qhi, qlo, qn, nq, dc, qh16, ql16, qterm, st))) return rc;
    kmark(tm, 1, false, st);
    if ((rc = coarse_tc(reinterpret_cast<const __half *>(ix->d_chi16),
                        reinterpret_cast<const __half *>(ix->d_clo16), ix->d_cterm, L, qh16, ql16,
                        qterm, nq, dc, ix->step_sq, cd, reinterpret_cast<uint32_t *>(stats + 3),
                        stats + 32, st)))
      return rc;
    kmark(tm, 1, true, st);
    ++g_launches;
  } else if ((rc = sq16_tiles(qhi, qlo, ix->d_chi, ix->d_clo, qn, ix->d_cnorm, ix->step_sq, nq, L,
                              dc, dc, dc, cd, true, st))) {
    return rc;
  }
  mark(tm, 2, st);
  if ((rc = select_topp_ex(cd, nq, L, p1, p, probed, stats + 0, nullptr, 0, st))) return rc;
  mark(tm, 3, st);
  return KATO_OK;
}

int search_pass(const katoann_gpu_index *ix, const Plan &pl, const float *queries, uint32_t nq,
                unsigned char *ws, uint32_t *out_ids, float *out_dists, const Budget &bud,
                cudaStream_t st, PhaseTimer *tm) {
  int rc;
  const uint32_t L = ix->nlist, p = pl.p, dc = ix->dc;
  uint8_t *qhi = ws + pl.off_qhi, *qlo = ws + pl.off_qlo;
  int64_t *qn = reinterpret_cast<int64_t *>(ws + pl.off_qn);
  int64_t *qhn = reinterpret_cast<int64_t *>(ws + pl.off_qhn);
  int64_t *qh0 = reinterpret_cast<int64_t *>(ws + pl.off_qh0);
  float *cd = reinterpret_cast<float *>(ws + pl.off_cd);
  uint32_t *probed = reinterpret_cast<uint32_t *>(ws + pl.off_probed);
  uint32_t *cnt = reinterpret_cast<uint32_t *>(ws + pl.off_cnt);
  uint32_t *off = reinterpret_cast<uint32_t *>(ws + pl.off_off);
  uint32_t *woff = reinterpret_cast<uint32_t *>(ws + pl.off_woff);
  uint32_t *cur = reinterpret_cast<uint32_t *>(ws + pl.off_cur);
  Work *work = reinterpret_cast<Work *>(ws + pl.off_work);
  uint32_t *ent = reinterpret_cast<uint32_t *>(ws + pl.off_ent);
  uint2 *slots = reinterpret_cast<uint2 *>(ws + pl.off_slots);
  uint2 *surv = reinterpret_cast<uint2 *>(ws + pl.off_surv);
  uint32_t *nsurv = reinterpret_cast<uint32_t *>(ws + pl.off_nsurv);
  unsigned long long *stats = reinterpret_cast<unsigned long long *>(ws + pl.off_stats);

  // with a model, the selection first goes as deep as its features and then,
  // for the queries whose budget is deeper, to the cap
  const bool model = bud.model && !bud.nprobe_in;
  const uint32_t p1 = model ? std::min(p, bud.model->depth) : p;
  if ((rc = coarse_pass(ix, pl, queries, nq, ws, p1, st, tm))) return rc;
  // 2'. per-query budgets: given, or from the model over the coarse distances
  uint32_t *qprobes = nullptr;
  if (bud.active()) {
    qprobes = reinterpret_cast<uint32_t *>(ws + pl.off_qprobes);
    if (bud.nprobe_in) {
      if ((rc = clamp_budget(bud.nprobe_in, nq, bud.cap, qprobes, st))) return rc;
      ++g_launches;
    } else {
      float *z = reinterpret_cast<float *>(ws + pl.off_z);
      if ((rc = probe_features(cd, L, probed, p, bud.model->d_rank, nq, z, st))) return rc;
      if ((rc = probe_budget(*bud.model, z, nq, bud.cap, nullptr, qprobes, st))) return rc;
      g_launches += 2;
      if (p1 < p) {
        if ((rc = select_topp_ex(cd, nq, L, p, p, probed, nullptr, qprobes, p1, st))) return rc;
        ++g_launches;
      }
    }
    if (bud.nprobe_out)
      KATO_CUDA(cudaMemcpyAsync(bud.nprobe_out, qprobes, static_cast<size_t>(nq) * 4,
                                cudaMemcpyDeviceToDevice, st));
  } else if (bud.nprobe_out) {
    if ((rc = clamp_budget(nullptr, nq, p, bud.nprobe_out, st))) return rc;  // all p
    ++g_launches;
  }
  mark(tm, 4, st);
  // 3. inversion (:403-412)
  const uint32_t total = nq * p;
  KATO_CUDA(cudaMemsetAsync(cnt, 0, static_cast<size_t>(L) * 4, st));
  count_kernel<<<div_up(total, 256), 256, 0, st>>>(probed, total, p, qprobes, cnt);
  scan_kernel<<<1, 1024, 0, st>>>(cnt, L, off, woff, cur);
  scatter_kernel<<<div_up(total, 256), 256, 0, st>>>(probed, total, p, qprobes, off, cur, ent);
  g_launches += 3;
  if (!pl.tc) {
    work_kernel<<<div_up(L, 256), 256, 0, st>>>(cnt, woff, L, work);
    ++g_launches;
  }
  KATO_LAUNCHED("inversion kernels");
  mark(tm, 5, st);
  uint32_t *qcount = nullptr;
  if (!pl.tc) mark(tm, 6, st);  // no seed-bound phase on the CUDA-core pass
  if (pl.tc) {
    // 4'. ranking pass on the tensor cores: seed bounds, work items, the
    // scan, and the exact rescan of any query whose buffer overflowed
    int32_t *bound = reinterpret_cast<int32_t *>(ws + pl.off_bound);
    TcItem *items = reinterpret_cast<TcItem *>(ws + pl.off_tcitems);
    uint32_t *tile_off = reinterpret_cast<uint32_t *>(ws + pl.off_tileoff);
    uint32_t *nitems = reinterpret_cast<uint32_t *>(ws + pl.off_nitems);
    uint32_t *qfill = reinterpret_cast<uint32_t *>(ws + pl.off_qfill);
    uint4 *rec = reinterpret_cast<uint4 *>(ws + pl.off_rec);
    uint32_t *rec_n = reinterpret_cast<uint32_t *>(ws + pl.off_recn);
    qcount = reinterpret_cast<uint32_t *>(ws + pl.off_qcount);
    const bool prefix_mode = pl.ranking == KATO_RANK_PREFIX;
    const int64_t *xnorm = prefix_mode ? ix->d_headnorm : ix->d_hinorm;
    const int64_t *qnorm = prefix_mode ? qh0 : qhn;
    const DistScale scale = make_dist_scale(ix->step_sq);
    if ((rc = rank_seed(ix->d_hi, xnorm, qhi, qnorm, probed, qprobes, ix->d_list_off, L, nq, p, dc,
                        pl.dims, pl.S, pl.seed_rows,
                        reinterpret_cast<uint32_t *>(ws + pl.off_seedorder), bound, st)))
      return rc;
    g_launches += L <= 16384 ? 1 : 0;  // the seed order
    mark(tm, 6, st);
    uint32_t *cost_off = reinterpret_cast<uint32_t *>(ws + pl.off_costoff);
    if ((rc = rank_tc_prepare(cnt, ix->d_list_off, L, pl.tcs.N, nq, pl.beta,
                              reinterpret_cast<uint32_t *>(ws + pl.off_tcscratch), items, tile_off,
                              cost_off, nitems, qcount, qfill, stats + 40, st)))
      return rc;
    RankTcArgs T{};
    T.qhi = qhi;
    T.qnorm = qnorm;
    T.entries = ent;
    T.off = off;
    T.items = items;
    T.tile_off = tile_off;
    T.cost_off = pl.beta ? cost_off : nullptr;
    T.nitems = nitems;
    T.bound = bound;
    T.qcount = qcount;
    T.rec = rec;
    T.rec_n = rec_n;
    T.rec_cap = pl.rec_cap;
    T.timeouts = reinterpret_cast<uint32_t *>(stats + 3);
    T.counters = stats + 4;
    T.prof = stats + 16;
    T.dc = dc;
    T.h = pl.dims;
    T.nprobe = p;
    T.wait = g_tc_wait.load() ? static_cast<long long>(g_tc_wait.load()) : 4000000000ll;
    T.scale = scale;
    kmark(tm, 2, false, st);
    if ((rc = rank_tc(T, ix->d_hi, ix->npts, pl.tcs, st))) return rc;
    kmark(tm, 2, true, st);
    if ((rc = rank_tc_bucket(rec, rec_n, pl.rec_cap, pl.ctas, qfill, slots, pl.cap, scale, st)))
      return rc;
    const RescanBufs rb{reinterpret_cast<uint32_t *>(ws + pl.off_rlist),
                        reinterpret_cast<unsigned long long *>(ws + pl.off_rkey),
                        reinterpret_cast<uint32_t *>(ws + pl.off_rcount), qfill};
    if ((rc = rank_overflow(ix->d_hi, xnorm, ix->d_ids, qhi, qnorm, probed, qprobes, ix->d_list_off, nq, p,
                            dc, pl.dims, pl.S, scale, qcount, slots, pl.cap, rb, stats + 6, st)))
      return rc;
    g_launches += 11;  // seed, 3 preparation, scan, bucket, 2 x 2 rescan rounds, exact rescan
  }
  // 4. ranking pass (:998-1044 / :1167-1204)
  const bool full = pl.ranking == KATO_RANK_FULL;
  RankArgs A{};
  A.xhi = ix->d_hi;
  A.xlo = ix->d_lo;
  A.xnorm = full ? ix->d_norm : (pl.ranking == KATO_RANK_PREFIX ? ix->d_headnorm : ix->d_hinorm);
  A.ids = ix->d_ids;
  A.list_off = ix->d_list_off;
  A.qhi = qhi;
  A.qlo = qlo;
  A.qnorm = full ? qn : (pl.ranking == KATO_RANK_PREFIX ? qh0 : qhn);
  A.work = work;
  A.woff_total = woff + L;
  A.off = off;
  A.entries = ent;
  A.dc = dc;
  A.dims = pl.dims;
  A.nprobe = p;
  A.S = pl.SC;  // a slot never holds more than min(S, largest list) candidates
  A.SC = pl.SC;
  A.slots = slots;
  A.scale = make_dist_scale(ix->step_sq);
  const size_t bp = static_cast<size_t>(nq) * p;
  const uint32_t grid = static_cast<uint32_t>(std::min<size_t>(L, bp) + bp / kQG + 1);
  const size_t smem = rank_smem_bytes(full ? 2 : 1, pl.select, pl.dims, pl.SC);
  if (!pl.tc && smem > 227 * 1024) return invalid("ranking tile does not fit in shared memory");
  auto launch = [&](auto kern) -> int {
    if (const int rc2 = smem_limit(reinterpret_cast<const void *>(kern), static_cast<int>(smem),
                                   "rank_kernel shared memory"))
      return rc2;
    kern<<<grid, kThreads, smem, st>>>(A);
    KATO_LAUNCHED("rank_kernel");
    return KATO_OK;
  };
  if (!pl.tc) {
    if (full) rc = pl.select ? launch(rank_kernel<true, true>) : launch(rank_kernel<true, false>);
    else rc = pl.select ? launch(rank_kernel<false, true>) : launch(rank_kernel<false, false>);
    if (rc) return rc;
    ++g_launches;
  }
  mark(tm, 7, st);
  // 5. per-query merge of the slot lists (:1058-1080 / :1205-1218)
  uint32_t np2 = 1;
  while (np2 < pl.S) np2 <<= 1;
  const size_t msmem = static_cast<size_t>(np2) * 12;
  if ((rc = smem_limit(reinterpret_cast<const void *>(merge_kernel), static_cast<int>(msmem),
                       "merge_kernel shared memory")))
    return rc;
  merge_kernel<<<nq, kThreads, msmem, st>>>(slots, pl.tc ? pl.cap : p * pl.SC, qcount, qprobes,
                                            pl.SC, ix->d_ids, pl.S, full, pl.k, surv, nsurv,
                                            out_ids, out_dists, stats + 1);
  ++g_launches;
  KATO_LAUNCHED("merge_kernel");
  mark(tm, 8, st);
  if (full) {
    mark(tm, 9, st);
    if (tm && tm->used < tm->max_passes) ++tm->used;
    return KATO_OK;
  }
  // 6. exact refinement and top-k (:1081-1125)
  const size_t rsmem = static_cast<size_t>(dc) * 2 + static_cast<size_t>(pl.S) * 12 +
                       static_cast<size_t>(pl.k) * 8;
  if ((rc = smem_limit(reinterpret_cast<const void *>(refine_kernel), static_cast<int>(rsmem),
                       "refine_kernel shared memory")))
    return rc;
  refine_kernel<<<nq, kThreads, rsmem, st>>>(qhi, qlo, qn, ix->d_hi, ix->d_lo, ix->d_norm,
                                             ix->d_ids, ix->npts, dc, surv, nsurv, pl.S, pl.k,
                                             make_dist_scale(ix->step_sq), out_ids, out_dists);
  KATO_LAUNCHED("refine_kernel");
  ++g_launches;
  mark(tm, 9, st);
  if (tm && tm->used < tm->max_passes) ++tm->used;
  return KATO_OK;
}

int search(const katoann_gpu_index *ix, const float *queries, uint32_t nq, uint32_t k, uint32_t p,
           int ranking, uint32_t survivors, uint32_t max_batch, void *ws, size_t ws_bytes,
           uint32_t *out_ids, float *out_dists, const Budget &budget, cudaStream_t st,
           void *timer) {
  if (nq == 0) return KATO_OK;
  if (max_batch == 0) return invalid("max_batch must be positive");
  // with a budget, the selection depth covers the cap and the model's features
  uint32_t depth = p;
  if (budget.active()) {
    if (budget.model) {
      if (int rc = check_probe_model(*budget.model)) return rc;
      depth = std::max(depth, budget.model->depth);
    }
    if (depth > kSortMax) return invalid("a per-query nprobe needs nprobe (and model depth) <= 4096");
  }
  Plan pl{};
  int rc = make_plan(ix, std::min(nq, max_batch), k, depth, ranking, survivors, &pl);
  if (rc) return rc;
  if (ws_bytes < pl.total) {
    set_error("search workspace too small");
    return KATO_ENOMEM;
  }
  unsigned char *w = static_cast<unsigned char *>(ws);
  KATO_CUDA(cudaMemsetAsync(w + pl.off_stats, 0, 48 * sizeof(unsigned long long), st));
  g_launches = 0;
  for (uint32_t q0 = 0; q0 < nq; q0 += max_batch) {
    const uint32_t b = std::min(max_batch, nq - q0);
    Budget bud = budget;
    bud.cap = p;
    if (bud.nprobe_in) bud.nprobe_in += q0;
    if (bud.nprobe_out) bud.nprobe_out += q0;
    if ((rc = search_pass(ix, pl, queries + static_cast<size_t>(q0) * ix->dim, b, w,
                          out_ids + static_cast<size_t>(q0) * k,
                          out_dists + static_cast<size_t>(q0) * k, bud, st,
                          static_cast<PhaseTimer *>(timer))))
      return rc;
  }
  return KATO_OK;
}

// The probe-budget features of nq queries (phases 0-2, then the feature
// kernel), max_batch at a time.
int probe_features_search(const katoann_gpu_index *ix, const float *queries, uint32_t nq,
                          const uint32_t *rank, uint32_t depth, uint32_t max_batch, void *ws,
                          size_t ws_bytes, float *z, cudaStream_t st) {
  if (nq == 0) return KATO_OK;
  if (max_batch == 0) return invalid("max_batch must be positive");
  if (!rank) return invalid("null feature ranks");
  if (depth == 0 || depth > ix->nlist || depth > kSortMax)
    return invalid("feature depth must be 1 to min(nlist, 4096)");
  Plan pl{};
  int rc = make_plan(ix, std::min(nq, max_batch), 1, depth, KATO_RANK_FULL, 1, &pl);
  if (rc) return rc;
  if (ws_bytes < pl.total) {
    set_error("feature workspace too small");
    return KATO_ENOMEM;
  }
  unsigned char *w = static_cast<unsigned char *>(ws);
  g_launches = 0;
  for (uint32_t q0 = 0; q0 < nq; q0 += max_batch) {
    const uint32_t b = std::min(max_batch, nq - q0);
    if ((rc = coarse_pass(ix, pl, queries + static_cast<size_t>(q0) * ix->dim, b, w, depth, st,
                          nullptr)))
      return rc;
    if ((rc = probe_features(reinterpret_cast<float *>(w + pl.off_cd), ix->nlist,
                             reinterpret_cast<uint32_t *>(w + pl.off_probed), depth, rank, b,
                             z + static_cast<size_t>(q0) * KATO_PROBE_FEATURES, st)))
      return rc;
  }
  return KATO_OK;
}

uint32_t last_launches() { return g_launches; }

// --------------------------------------------------------------- autotune
// Times one search of these queries under every candidate setting of the
// ranking pass's knobs - seed rows, CTA split weight, item width - and keeps
// the fastest. The knobs change the work and its schedule, never a result.
int autotune(const katoann_gpu_index *ix, const float *queries, uint32_t nq, uint32_t k, uint32_t p,
             int ranking, uint32_t survivors, uint32_t max_batch, const Budget &budget, void *ws,
             size_t ws_bytes, cudaStream_t st, uint32_t *out) {
  if (nq == 0) return invalid("autotune needs queries");
  // the batch the search runs, once: the buffers of the results
  uint32_t *ids = nullptr;
  float *dists = nullptr;
  KATO_CUDA(cudaMalloc(&ids, static_cast<size_t>(nq) * k * 4));
  const cudaError_t e2 = cudaMalloc(&dists, static_cast<size_t>(nq) * k * 4);
  if (e2 != cudaSuccess) {
    cudaFree(ids);
    return cuda_status(e2, "autotune buffers");
  }
  cudaEvent_t a = nullptr, b = nullptr;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const uint32_t seed0 = g_seed_rows.load(), beta0 = g_tc_beta.load(), width0 = g_tc_width.load();
  float best = 1e30f;
  uint32_t bs = seed0, bb = beta0, bw = width0;
  int rc = KATO_OK;
  for (uint32_t seed : {1024u, 2048u, 4096u})
    for (uint32_t beta : {0u, 1u, 2u, 4u})
      for (uint32_t width : {0u, 32u}) {
        g_seed_rows = seed;
        g_tc_beta = beta;
        g_tc_width = width;
        int r = search(ix, queries, nq, k, p, ranking, survivors, max_batch, ws, ws_bytes, ids,
                       dists, budget, st, nullptr);
        if (r == KATO_ENOMEM) continue;  // this setting needs a larger workspace
        if (r) {
          rc = r;
          break;
        }
        cudaEventRecord(a, st);
        for (int rep = 0; rep < 3 && !r; ++rep)
          r = search(ix, queries, nq, k, p, ranking, survivors, max_batch, ws, ws_bytes, ids, dists,
                     budget, st, nullptr);
        cudaEventRecord(b, st);
        if (r || cudaEventSynchronize(b) != cudaSuccess) {
          rc = r ? r : cuda_status(cudaGetLastError(), "autotune");
          break;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best) {
          best = ms;
          bs = seed;
          bb = beta;
          bw = width;
        }
      }
  g_seed_rows = rc ? seed0 : bs;
  g_tc_beta = rc ? beta0 : bb;
  g_tc_width = rc ? width0 : bw;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(ids);
  cudaFree(dists);
  if (rc) return rc;
  out[0] = bs;
  out[1] = bb;
  out[2] = bw;
  out[3] = static_cast<uint32_t>(best / 3 * 1000.0f);
  return KATO_OK;
}

// ------------------------------------------------------------ CUDA graphs
struct SearchGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint32_t launches = 0;
};

int search_capture(const katoann_gpu_index *ix, const float *queries, uint32_t nq, uint32_t k,
                   uint32_t p, int ranking, uint32_t survivors, uint32_t max_batch, void *ws,
                   size_t ws_bytes, uint32_t *out_ids, float *out_dists, const Budget &budget,
                   cudaStream_t st, void **out) {
  *out = nullptr;
  if (!st || st == cudaStreamLegacy || st == cudaStreamPerThread)
    return invalid("graph capture needs a created stream");
  KATO_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  const int rc = search(ix, queries, nq, k, p, ranking, survivors, max_batch, ws, ws_bytes,
                        out_ids, out_dists, budget, st, nullptr);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(st, &g);  // always ends the capture
  if (rc || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return rc ? rc : cuda_status(e, "cudaStreamEndCapture");
  }
  cudaGraphExec_t ex = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&ex, g, 0);
  if (ei != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_status(ei, "cudaGraphInstantiate");
  }
  *out = new SearchGraph{g, ex, g_launches};
  return KATO_OK;
}

int graph_launch(void *h, cudaStream_t st) {
  if (!h) return invalid("null graph");
  KATO_CUDA(cudaGraphLaunch(static_cast<SearchGraph *>(h)->exec, st));
  return KATO_OK;
}

uint32_t graph_launches(const void *h) {
  return h ? static_cast<const SearchGraph *>(h)->launches : 0;
}

void graph_destroy(void *h) {
  auto *g = static_cast<SearchGraph *>(h);
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
}

void *timer_create(uint32_t max_passes) {
  auto *t = new PhaseTimer();
  t->max_passes = max_passes;
  t->ev.resize(static_cast<size_t>(max_passes) * kTimerStride);
  t->kdone.assign(max_passes, 0);
  for (auto &e : t->ev)
    if (cudaEventCreate(&e) != cudaSuccess) {
      delete t;
      return nullptr;
    }
  return t;
}

void timer_destroy(void *p) {
  auto *t = static_cast<PhaseTimer *>(p);
  if (!t) return;
  for (auto &e : t->ev) cudaEventDestroy(e);
  delete t;
}

int timer_read(void *p, float *ms, uint32_t *passes) {
  auto *t = static_cast<PhaseTimer *>(p);
  for (int i = 0; i < KATO_PHASES; ++i) ms[i] = 0.0f;
  *passes = t->used;
  for (int k = 0; k < KATO_TIMED_KERNELS; ++k) t->kms[k] = 0.0f, t->kn[k] = 0;
  if (t->used == 0) return KATO_OK;
  // the last phase event of the last pass follows every other event in it
  KATO_CUDA(cudaEventSynchronize(t->ev[(t->used - 1) * kTimerStride + KATO_PHASES]));
  for (uint32_t u = 0; u < t->used; ++u) {
    const cudaEvent_t *e = t->ev.data() + static_cast<size_t>(u) * kTimerStride;
    for (int i = 0; i < KATO_PHASES; ++i) {
      float x = 0;
      if (cudaEventElapsedTime(&x, e[i], e[i + 1]) == cudaSuccess) ms[i] += x;
    }
    for (int k = 0; k < KATO_TIMED_KERNELS; ++k) {
      float x = 0;
      if ((t->kdone[u] >> k & 1u) &&
          cudaEventElapsedTime(&x, e[KATO_PHASES + 1 + 2 * k], e[KATO_PHASES + 2 + 2 * k]) ==
              cudaSuccess) {
        t->kms[k] += x;
        ++t->kn[k];
      }
    }
    t->kdone[u] = 0;
  }
  t->used = 0;
  return KATO_OK;
}

void timer_kernels(void *p, float *ms, uint32_t *launches) {
  const auto *t = static_cast<const PhaseTimer *>(p);
  for (int k = 0; k < KATO_TIMED_KERNELS; ++k) {
    ms[k] = t->kms[k];
    launches[k] = t->kn[k];
  }
}

size_t search_workspace(const katoann_gpu_index *ix, uint32_t max_batch, uint32_t k, uint32_t p,
                        int ranking, uint32_t survivors) {
  Plan pl{};
  if (make_plan(ix, max_batch, k, p, ranking, survivors, &pl)) return 0;
  return pl.total;
}


}  // namespace kato
