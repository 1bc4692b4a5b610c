// bw_chain.cu -- single-pass replay of a linear version chain (see bw_chain.cuh).
//
// Sweep (k_chain_sweep, one CTA per state block; 128-512 threads, tiles of 512-1024
// events, a ring of 2-3 tiles, the geometry picked per workload by occupancy):
//   * the block's events [e0, e1) stream through the ring, each tile one
//     cp.async.bulk copy from global memory into shared memory completed on the
//     stage's mbarrier (bounded waits);
//   * the running key histogram of the block is an exact int32 window H[key] in
//     shared memory (plus int32 totals of 32-key chunks when the key domain is
//     larger than 4,096 keys).  A window holds events whose absolute sum stays
//     below 2^28 + 2^29, so every partial sum of it is exact in int32; before it
//     can grow past that it is folded into the block's key prefix row in global
//     memory (P[k] = sum of the folded events below key k, int64).  Tiles holding a
//     delta outside (-2^19, 2^19) bypass the window: their events go to a per-block
//     int64 key histogram with global atomics, folded into P before the next tile;
//   * a tile owns the queries whose position (number of events at or before their
//     state) falls inside it: state < state of the tile's last event.  Their local
//     answer = P[hi] - P[lo] + the window over [lo, hi) before the tile is applied,
//     plus the tile's first `pos` events inside [lo, hi); one warp per query,
//     int32 lane sums reduced with redux.sync;
//   * one warp (the last) finds the next tile's queries and their positions while
//     the others answer the current tile's: the query records come through a
//     32-record window that cp.async fills one tile ahead, and land in a
//     double-buffered shared query buffer.
// Carry (k_chain_colsum, k_chain_colfix): exclusive column scan over the blocks'
// final prefix rows in two passes (segment sums, then segment-local prefixes), in
// place: row b becomes the key prefix of the events of blocks 0 .. b-1.
// Fix-up (k_chain_fixup): every query of block b >= 1 adds row[hi] - row[lo].
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <type_traits>

#include "bw_gpu.h"
#include "bw_common.cuh"
#include "bw_chain.cuh"

namespace bw {
namespace {

constexpr int TE = kChainTile;   // largest tile (the shared-memory ring is sized per geometry)
constexpr int QB = kChainQBuf;
constexpr int kMaxWarps = kChainThreads / 32;
constexpr int kChunkShift = 5;                   // chunk totals cover 32 keys each
constexpr uint32_t kFlatKeys = 4096;             // key domains up to this size keep no chunk totals
constexpr uint32_t kWaitLimit = 1u << 22;        // mbarrier polls before a stage is declared lost
constexpr uint32_t kFoldAt = 1u << 28;           // window |delta| sum that triggers a fold
// A tile is int32-safe when every delta lies in (-2^19, 2^19): with at most 1024
// events its absolute sum is then below 2^29.

struct ChainParams {
  const uint4* ev;        // events as 16-byte records (state, key, delta lo, delta hi)
  const BwQuery* qs;
  int64_t* ans;
  const int32_t* parent;
  int64_t E, Q;
  int32_t S;
  uint32_t C;
  int32_t B;
  int32_t nch, nseg;
  int64_t* rows;          // B rows of C+1 int64: key prefixes (row[k] = sum below key k)
  int64_t* wide;          // B rows of C int64: key histogram of the block's wide tiles
  int64_t* btab;          // B x (first query, end query)
  int64_t* seg;           // nseg rows of C+1 uint64
  int32_t* status;
};

// Shared words written in one tile and read in the next are double-buffered by
// tile parity: a fast warp may already write the next tile's copy while a slow one
// still reads this tile's.
struct Misc {
  uint32_t wsum[2][kMaxWarps];   // per-warp |delta| sum of a tile's window updates
  int64_t tq[2][2];              // queries [tq0, tq1) of a tile
  uint32_t prev_state[2];        // state of the event before a tile
  int64_t tail_q0;
  unsigned long long scan[kMaxWarps];   // warp totals of the fold's key scan
};

// Dynamic shared memory of the sweep, every region 16-byte aligned.
struct SweepSmem {
  size_t ring, H, T, qbuf, qpre, bar, misc, bytes;
};
__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~size_t(15); }
// hw: bytes of a window entry (4: int32 window, 8: int64 window)
__host__ __device__ inline SweepSmem sweep_smem(uint32_t C, int nch, int te, int ns, int hw) {
  SweepSmem L;
  size_t o = 0;
  L.ring = o;  o = al16(o + (size_t)ns * te * 16);
  L.H = o;     o = al16(o + (size_t)C * hw);
  L.T = o;     o = al16(o + (size_t)nch * hw);
  L.qbuf = o;  o = al16(o + 2 * (size_t)QB * 16);   // two tiles' query records
  L.qpre = o;  o = al16(o + 32 * 12);                // prefetched window of 32 query records
  L.bar = o;   o = al16(o + (size_t)ns * 8);
  L.misc = o;  o = al16(o + sizeof(Misc));
  L.bytes = o;
  return L;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Bounded wait for phase `parity` of a stage barrier; false when it never completed.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t i = 0; i < kWaitLimit; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void set_status(int32_t* st, int32_t code) {
  if (*reinterpret_cast<volatile int32_t*>(st) == 0) atomicCAS(st, 0, code);
}

// delta in (-2^19, 2^19): its high word is the sign extension of its low word
__device__ __forceinline__ bool small_delta(const uint4& e) {
  const int32_t lo = (int32_t)e.z;
  return e.w == (uint32_t)(lo >> 31) && (uint32_t)(lo + (1 << 19)) < (1u << 20);
}

__device__ __forceinline__ uint64_t warp_sum_u64(uint64_t v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Lane share of the window sum over keys [lo, hi) (lo < hi <= C): the partial
// chunks at either end from H (fewer than 32 keys each), the whole chunks from T.
__device__ __forceinline__ int32_t probe32(const int32_t* H, const int32_t* T, uint32_t lo, uint32_t hi, int lane) {
  const uint32_t clo = (lo + 31) >> kChunkShift, chi = hi >> kChunkShift;
  int32_t s = 0;
  if (clo >= chi) {   // fewer than 64 keys
    for (uint32_t k = lo + lane; k < hi; k += 32) s += H[k];
    return s;
  }
  const uint32_t a = lo + lane, z = (chi << kChunkShift) + lane;
  if (a < (clo << kChunkShift)) s += H[a];
  if (z < hi) s += H[z];
  for (uint32_t c = clo + lane; c < chi; c += 32) s += T[c];
  return s;
}

// Lane share of the window sum over keys [lo, hi) (lo < hi <= C) without chunk
// totals: 128-bit reads of H, four keys per lane, masked to the interval.  H is
// 16-byte aligned and padded to a multiple of four keys, so the last read stays in
// the region; padding keys fall outside [lo, hi).
__device__ __forceinline__ int32_t probe_flat(const int32_t* H, uint32_t lo, uint32_t hi, int lane) {
  const uint32_t w = hi - lo;
  int32_t s = 0;
#pragma unroll 2
  for (uint32_t k = (lo & ~3u) + 4 * lane; k < hi; k += 128) {
    const int4 v = *reinterpret_cast<const int4*>(H + k);
    const uint32_t d = k - lo;
    s += (d < w ? v.x : 0) + (d + 1 < w ? v.y : 0) + (d + 2 < w ? v.z : 0) + (d + 3 < w ? v.w : 0);
  }
  return s;
}

// The int64 window's counterparts: lane shares of the sum over [lo, hi) (lo < hi <= C)
// from 32-key chunk totals plus the partial chunks, or flat 128-bit reads of two
// keys each (H 16-byte aligned and padded to an even key count).
__device__ __forceinline__ uint64_t probe_chunks64(const unsigned long long* H, const unsigned long long* T,
                                                   uint32_t lo, uint32_t hi, int lane) {
  const uint32_t clo = (lo + 31) >> kChunkShift, chi = hi >> kChunkShift;
  uint64_t s = 0;
  if (clo >= chi) {
    for (uint32_t k = lo + lane; k < hi; k += 32) s += H[k];
    return s;
  }
  const uint32_t a = lo + lane, z = (chi << kChunkShift) + lane;
  if (a < (clo << kChunkShift)) s += H[a];
  if (z < hi) s += H[z];
  for (uint32_t c = clo + lane; c < chi; c += 32) s += T[c];
  return s;
}
__device__ __forceinline__ uint64_t probe_flat64(const unsigned long long* H, uint32_t lo, uint32_t hi, int lane) {
  const uint32_t w = hi - lo;
  uint64_t s = 0;
#pragma unroll 2
  for (uint32_t k = (lo & ~1u) + 2 * lane; k < hi; k += 64) {
    const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(H + k);
    const uint32_t d = k - lo;
    s += (d < w ? v.x : 0ull) + (d + 1 < w ? v.y : 0ull);
  }
  return s;
}

// Position of a query in its tile: the number of the tile's events at or before
// its state (upper bound over the tile's sorted states).
__device__ __forceinline__ uint32_t tile_pos(const uint4* tile, int n, uint32_t qst) {
  uint32_t lo = 0, hi = (uint32_t)n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (tile[mid].x <= qst) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// First query index in [0, Q) whose state is >= x (Q when none), found by the
// whole CTA in rounds of one probe per thread.
__device__ int64_t first_query_at_or_after(const BwQuery* qs, int64_t Q, uint32_t x) {
  const int nt = blockDim.x;
  int64_t lo = 0, hi = Q;
  while (true) {
    const int64_t n = hi - lo;
    if (n <= 0) return lo;
    const int64_t step = (n + nt - 1) / nt;
    const int64_t pos = lo + (int64_t)threadIdx.x * step;
    const bool lt = pos < hi && qs[pos].state < x;
    const int cnt = __syncthreads_count(lt);
    if (step == 1) return lo + cnt;
    const int64_t nlo = cnt ? lo + (int64_t)(cnt - 1) * step + 1 : lo;
    hi = min(hi, lo + (int64_t)cnt * step);
    lo = nlo;
  }
}

// The query warp's window of the next 32 query records, copied into shared memory
// with cp.async one tile before it is read (so the copy's latency stays hidden).
__device__ __forceinline__ void qpre_issue(uint32_t* qpre, const BwQuery* qs, int64_t Q, int64_t base, int lane) {
  const int64_t i = base + lane;
  if (i < Q) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(qs + i);
#pragma unroll
    for (int j = 0; j < 3; ++j)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(qpre + 3 * lane + j)), "l"(src + j)
                   : "memory");
  } else {
    qpre[3 * lane] = 0xffffffffu;   // past the last query
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
}

// Query warp: the queries of a tile (n events, the last with state x) are those
// from qcur on with state < x.  Their records and positions in the tile go to qbuf
// (the first QB), their range to tq; qcur advances past them.  `pbase` is the first
// query of the window in flight.
__device__ void find_tile_queries(const ChainParams& p, uint32_t* qpre, int64_t& pbase, int64_t& qcur,
                                  const uint4* tile, int n, uint32_t* qbuf, int64_t* tq, int lane) {
  const uint32_t x = tile[n - 1].x;
  const int64_t tq0 = qcur;
  while (true) {
    if (pbase != qcur) {
      qpre_issue(qpre, p.qs, p.Q, qcur, lane);
      pbase = qcur;
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    const uint32_t st = qpre[3 * lane], lo = qpre[3 * lane + 1], hi = qpre[3 * lane + 2];
    const bool valid = qcur + lane < p.Q;
    const uint32_t ball = __ballot_sync(0xffffffffu, valid && st < x);
    const int k = ball == 0xffffffffu ? 32 : __ffs(~ball) - 1;
    if (lane < k) {
      const int64_t slot = qcur - tq0 + lane;
      if (slot < QB) {
        uint4 r;
        r.x = st;
        r.y = lo;
        r.z = hi;
        r.w = tile_pos(tile, n, st);
        reinterpret_cast<uint4*>(qbuf)[slot] = r;
      }
    }
    __syncwarp();   // every lane has read the window before it is refilled
    qcur += k;
    if (k < 32) break;
  }
  if (lane == 0) {
    tq[0] = tq0;
    tq[1] = qcur;
  }
  qpre_issue(qpre, p.qs, p.Q, qcur, lane);   // read at the next tile
  pbase = qcur;
}

// The same with the int64 window (no folded row: it only fills at the end).
__device__ __forceinline__ int64_t answer_one64(const ChainParams& p, const unsigned long long* H,
                                                const unsigned long long* T, const uint4* tile, uint32_t pos,
                                                uint32_t lo, uint32_t hi, int lane) {
  lo = min(lo, p.C);
  hi = min(hi, p.C);
  if (lo >= hi) return 0;
  const uint32_t w = hi - lo;
  uint64_t part = p.nch ? probe_chunks64(H, T, lo, hi, lane) : probe_flat64(H, lo, hi, lane);
#pragma unroll 4
  for (uint32_t j = lane; j < pos; j += 32) {
    const uint4 e = tile[j];
    if (e.y - lo < w) part += ((uint64_t)e.w << 32) | e.z;
  }
  return (int64_t)warp_sum_u64(part);
}

// Answer of one query by one warp, valid in lane 0: the folded key prefix row
// (P[hi] - P[lo], when it holds data), the window probe, and the tile's first
// `pos` events inside [lo, hi) (tile == nullptr: none).
__device__ __forceinline__ int64_t answer_one(const ChainParams& p, const int32_t* H, const int32_t* T,
                                              const int64_t* P, bool rows_live, bool wide_tile, const uint4* tile,
                                              uint32_t pos, uint32_t lo, uint32_t hi, int lane) {
  lo = min(lo, p.C);
  hi = min(hi, p.C);
  if (lo >= hi) return 0;
  const uint32_t w = hi - lo;
  uint64_t pv = 0;
  if (rows_live && lane < 2) pv = (uint64_t)__ldcg(P + (lane ? hi : lo));   // both ends in flight at once
  int32_t part = p.nch ? probe32(H, T, lo, hi, lane) : probe_flat(H, lo, hi, lane);
  uint64_t wide = 0;
  if (tile) {
    if (wide_tile) {
      for (uint32_t j = lane; j < pos; j += 32) {
        const uint4 e = tile[j];
        if (e.y - lo < w) wide += ((uint64_t)e.w << 32) | e.z;
      }
    } else {
#pragma unroll 4
      for (uint32_t j = lane; j < pos; j += 32) {
        const uint4 e = tile[j];
        if (e.y - lo < w) part += (int32_t)e.z;
      }
    }
  }
  uint64_t total = (uint64_t)(int64_t)(int32_t)__reduce_add_sync(0xffffffffu, (uint32_t)part);
  if (wide_tile) total += warp_sum_u64(wide);
  const uint64_t phi = __shfl_down_sync(0xffffffffu, pv, 1);
  return (int64_t)(total + phi - pv);
}

// Fold of the window (and of the wide tiles' histogram) into the block's key
// prefix row: P[k+1] += sum of H[j] + wide[j] over j <= k.  Each thread takes a
// contiguous key segment; a CTA-wide exclusive scan of the segment sums gives its
// base.  H, T and the consumed wide entries return to zero.  All threads call it.
template <int NT, typename HT>
__device__ void fold(const ChainParams& p, HT* H, HT* T, int64_t* P, int64_t* wide, bool rows_live,
                     bool wide_live, Misc* m) {
  constexpr int NW = NT / 32;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t C = p.C, per = (C + NT - 1) / NT;
  const uint32_t k0 = min(C, (uint32_t)tid * per), k1 = min(C, k0 + per);
  uint64_t s = 0;
  for (uint32_t k = k0; k < k1; ++k) {
    s += (uint64_t)(int64_t)H[k];   // sign-extends an int32 window entry
    if (wide_live) s += (uint64_t)__ldcg(wide + k);
  }
  uint64_t incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) m->scan[warp] = incl;
  __syncthreads();
  uint64_t run = incl - s;
#pragma unroll
  for (int w = 0; w < NW; ++w)
    if (w < warp) run += m->scan[w];
  for (uint32_t k = k0; k < k1; ++k) {
    run += (uint64_t)(int64_t)H[k];
    H[k] = 0;
    if (wide_live) {
      run += (uint64_t)__ldcg(wide + k);
      wide[k] = 0;
    }
    P[k + 1] = rows_live ? (int64_t)((uint64_t)__ldcg(P + k + 1) + run) : (int64_t)run;
  }
  if (tid == 0 && !rows_live) P[0] = 0;
  for (int c = tid; c < p.nch; c += NT) T[c] = 0;
  __syncthreads();
}

// Tile geometry: NT threads, EPT events per thread, TL = NT * EPT events per tile
// (<= 1024, so an int32-safe tile's absolute sum stays below 2^29); MINB CTAs per SM;
// NS tiles in the shared-memory ring.  W64: the window is int64 (two 32-bit shared
// atomics per update, exact modulo 2^64 at any delta size): no window folds, no wide
// tiles -- the mode for chains whose deltas mostly exceed the int32-safe range.
template <int NT, int EPT, int MINB, int NS, bool W64>
__global__ void __launch_bounds__(NT, MINB) k_chain_sweep(ChainParams p) {
  constexpr int NW = NT / 32, QW = NW - 1, TL = NT * EPT;
  static_assert(TL <= TE && NW <= kMaxWarps && NW >= 2, "tile geometry");
  extern __shared__ __align__(128) unsigned char sm[];
  const uint32_t C = p.C;
  using HT = typename std::conditional<W64, unsigned long long, int32_t>::type;
  const SweepSmem SL = sweep_smem(C, p.nch, TL, NS, (int)sizeof(HT));
  uint4* ring = reinterpret_cast<uint4*>(sm + SL.ring);
  HT* H = reinterpret_cast<HT*>(sm + SL.H);
  HT* T = reinterpret_cast<HT*>(sm + SL.T);
  uint32_t* qbuf = reinterpret_cast<uint32_t*>(sm + SL.qbuf);   // [2][QB] uint4, by tile parity
  uint32_t* qpre = reinterpret_cast<uint32_t*>(sm + SL.qpre);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + SL.bar);
  Misc* m = reinterpret_cast<Misc*>(sm + SL.misc);
  auto qbuf_of = [&](int t) { return qbuf + (size_t)(t & 1) * QB * 4; };

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int b = blockIdx.x;
  const int64_t e0 = (int64_t)b * p.E / p.B, e1 = (int64_t)(b + 1) * p.E / p.B;
  const int64_t ne = e1 - e0;
  const int ntiles = (int)((ne + TL - 1) / TL);
  int64_t* P = p.rows + (int64_t)b * (C + 1);
  int64_t* wrow = p.wide + (int64_t)b * C;
  auto tile_n = [&](int t) { return (int)min((int64_t)TL, ne - (int64_t)t * TL); };

  for (uint32_t i = tid; i < C; i += NT) H[i] = 0;
  for (int i = tid; i < p.nch; i += NT) T[i] = 0;
  if (tid < 2 * kMaxWarps) m->wsum[tid / kMaxWarps][tid % kMaxWarps] = 0;
  if (tid == 0) {
    for (int s = 0; s < NS; ++s) mbar_init(&bar[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    m->prev_state[0] = b > 0 ? p.ev[e0 - 1].x : 0u;
  }
  __syncthreads();
  int issued = 0;   // tiles whose copy was issued (thread 0)
  if (tid == 0) {
    for (; issued < NS && issued < ntiles; ++issued)
      bulk_load(ring + (issued % NS) * TL, p.ev + e0 + (int64_t)issued * TL, (uint32_t)tile_n(issued) * 16u,
                &bar[issued % NS]);
  }
  // input checks spread over every sweep thread: parent[v] = v - 1, and every query
  // (sorted by state, state and bounds in range) -- queries behind an out-of-order
  // one may never be reached by a tile, so they are checked here, not when consumed
  for (int64_t v = (int64_t)b * NT + tid; v < p.S; v += (int64_t)p.B * NT)
    if (p.parent[v] != (int32_t)(v - 1)) set_status(p.status, BW_STATUS_BAD_PARENT);
  for (int64_t i = (int64_t)b * NT + tid; i < p.Q; i += (int64_t)p.B * NT) {
    const uint32_t* r = reinterpret_cast<const uint32_t*>(p.qs + i);
    const uint32_t qst = r[0], lo = r[1], hi = r[2];
    if (i > 0 && qst < p.qs[i - 1].state) set_status(p.status, BW_STATUS_QUERIES_UNSORTED);
    if (qst >= (uint32_t)p.S) set_status(p.status, BW_STATUS_STATE_RANGE);
    if (lo > C || hi > C) set_status(p.status, BW_STATUS_QUERY_RANGE);
  }
  // the block's first query: position >= e0, i.e. state >= state of event e0 - 1
  const int64_t qstart = b > 0 ? first_query_at_or_after(p.qs, p.Q, m->prev_state[0]) : 0;

  int64_t qcur = qstart, pbase = qstart;
  if (warp == QW) qpre_issue(qpre, p.qs, p.Q, qcur, lane);

  uint4 cur[EPT];
  bool rows_live = false;   // the prefix row holds data (set by the first fold)
  bool wide_init = false;   // the wide histogram row has been zeroed
  bool wide_live = false;   // a wide tile was applied since the last fold
  uint32_t win = 0;         // |delta| sum in the int32 window (the same in every thread)
  int bigp = 0, lost = 0;
  uint32_t bad = 0;         // event defects seen by this thread (reported at the end)
  if (ntiles > 0) {
    if (!mbar_wait(&bar[0], 0)) {
      set_status(p.status, BW_STATUS_TIMEOUT);
      lost = 1;
    } else {
      const int n = tile_n(0);
#pragma unroll
      for (int k = 0; k < EPT; ++k) {
        const int idx = tid + k * NT;
        cur[k] = idx < n ? ring[idx] : make_uint4(0, 0, 0, 0);
        if (!W64) bigp |= !small_delta(cur[k]);
      }
      if (warp == QW) find_tile_queries(p, qpre, pbase, qcur, ring, n, qbuf_of(0), m->tq[0], lane);
    }
  }
  // end-of-tile barrier: OR of the next tile's wide flag and of lost waits (a
  // second barrier separates the two only when the first is set)
  auto tile_barrier = [&](int wide, int gone, int& big_out) -> bool {
    if (!__syncthreads_or(wide | gone)) {
      big_out = 0;
      return false;
    }
    const bool ab = __syncthreads_or(gone);
    big_out = __syncthreads_or(wide);
    return ab;
  };
  int big = 0;
  bool aborted = tile_barrier(bigp, lost, big);

  int t = 0;
  for (; t < ntiles && !aborted; ++t) {
    const int n = tile_n(t);
    const uint4* tile = ring + (t % NS) * TL;
    if (tid == 0 && t >= 1 && issued < ntiles) {
      // stage (t-1) % NS was released by the barrier that ended tile t-1
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      bulk_load(ring + (issued % NS) * TL, p.ev + e0 + (int64_t)issued * TL, (uint32_t)tile_n(issued) * 16u,
                &bar[issued % NS]);
      ++issued;
    }
    const int64_t tq0 = m->tq[t & 1][0], tq1 = m->tq[t & 1][1];
    if (t > 0) {   // window updates of the previous tile, summed over its warps
      const uint32_t v = lane < NW ? m->wsum[(t - 1) & 1][lane] : 0u;
      win += __reduce_add_sync(0xffffffffu, v);
    }
    // fold the window into the prefix row before it could overflow, and after a
    // wide tile (whose events went to the wide histogram)
    if (!W64 && (win >= kFoldAt || wide_live)) {
      fold<NT>(p, H, T, P, wrow, rows_live, wide_live, m);
      win = 0;
      rows_live = true;
      wide_live = false;
    }
    if (!W64 && big && !wide_init) {
      for (uint32_t k = tid; k < C; k += NT) wrow[k] = 0;
      wide_init = true;
      __syncthreads();
    }
    // the tile's queries, one warp each; meanwhile the query warp waits for the next
    // tile and finds its queries (into the other query buffer)
    const bool has_q = tq1 > tq0;
    bool next_found = false;
    if (has_q) {
      if (warp == QW) {
        if (t + 1 < ntiles) {
          const uint4* nt = ring + ((t + 1) % NS) * TL;
          if (!mbar_wait(&bar[(t + 1) % NS], (uint32_t)(((t + 1) / NS) & 1))) {
            set_status(p.status, BW_STATUS_TIMEOUT);
            lost = 1;
          } else {
            find_tile_queries(p, qpre, pbase, qcur, nt, tile_n(t + 1), qbuf_of(t + 1), m->tq[(t + 1) & 1], lane);
          }
        }
        next_found = true;
      }
      const uint4* qb = reinterpret_cast<const uint4*>(qbuf_of(t));
      for (int64_t i = tq0 + warp; warp < QW && i < tq1; i += QW) {
        uint32_t lo, hi, pos;
        if (i - tq0 < QB) {
          const uint4 r = qb[i - tq0];
          lo = r.y;
          hi = r.z;
          pos = r.w;
        } else {
          const uint32_t* r = reinterpret_cast<const uint32_t*>(p.qs + i);
          lo = r[1];
          hi = r[2];
          pos = tile_pos(tile, n, r[0]);
        }
        int64_t a;
        if constexpr (W64) a = answer_one64(p, H, T, tile, pos, lo, hi, lane);
        else a = answer_one(p, H, T, P, rows_live, big != 0, tile, pos, lo, hi, lane);
        if (lane == 0) p.ans[i] = a;
      }
      __syncthreads();
    }
    // apply the tile (the state before each event comes from the previous lane; lane
    // 0 reads it from the tile, or from the previous tile for the first event)
    uint32_t wsum = 0;
#pragma unroll
    for (int k = 0; k < EPT; ++k) {
      const int idx = tid + k * NT;
      const uint32_t up = __shfl_up_sync(0xffffffffu, cur[k].x, 1);
      if (idx < n) {
        const uint4 e = cur[k];
        const uint32_t prev = lane ? up : (idx ? tile[idx - 1].x : m->prev_state[t & 1]);
        bad |= (e.x < prev ? 1u : 0u) | (e.x >= (uint32_t)p.S ? 2u : 0u);
        if (e.y >= C) {
          bad |= 4u;
        } else if (W64) {
          const uint64_t d = ((uint64_t)e.w << 32) | e.z;
          shared_add_u64(reinterpret_cast<unsigned long long*>(&H[e.y]), d);
          if (p.nch) shared_add_u64(reinterpret_cast<unsigned long long*>(&T[e.y >> kChunkShift]), d);
        } else if (!big) {
          const int32_t d = (int32_t)e.z;
          atomicAdd(reinterpret_cast<int32_t*>(&H[e.y]), d);
          if (p.nch) atomicAdd(reinterpret_cast<int32_t*>(&T[e.y >> kChunkShift]), d);
          wsum += (uint32_t)(d < 0 ? -d : d);
        } else {
          atomicAdd(reinterpret_cast<unsigned long long*>(wrow + e.y), ((unsigned long long)e.w << 32) | e.z);
        }
      }
    }
    wide_live |= big != 0;
    {
      const uint32_t ws = __reduce_add_sync(0xffffffffu, wsum);
      if (lane == 0) m->wsum[t & 1][warp] = ws;
    }
    if (tid == 0) m->prev_state[(t + 1) & 1] = tile[n - 1].x;
    // next tile: wait for its copy, load this thread's events (and, when no query
    // phase ran, let the query warp find the next tile's queries)
    bigp = 0;
    if (t + 1 < ntiles) {
      const int nn = tile_n(t + 1);
      const uint4* nt = ring + ((t + 1) % NS) * TL;
      if (!mbar_wait(&bar[(t + 1) % NS], (uint32_t)(((t + 1) / NS) & 1))) {
        set_status(p.status, BW_STATUS_TIMEOUT);
        lost = 1;
      } else {
#pragma unroll
        for (int k = 0; k < EPT; ++k) {
          const int idx = tid + k * NT;
          cur[k] = idx < nn ? nt[idx] : make_uint4(0, 0, 0, 0);
          if (!W64) bigp |= !small_delta(cur[k]);
        }
        if (warp == QW && !next_found)
          find_tile_queries(p, qpre, pbase, qcur, nt, nn, qbuf_of(t + 1), m->tq[(t + 1) & 1], lane);
      }
    }
    aborted = tile_barrier(bigp, lost, big);
  }

  if (bad)
    set_status(p.status, (bad & 1u) ? BW_STATUS_EVENTS_UNSORTED
                                    : (bad & 2u) ? BW_STATUS_STATE_RANGE : BW_STATUS_EVENT_KEY_RANGE);
  // the query warp's last window copy lands before its shared memory goes away
  if (warp == QW) asm volatile("cp.async.wait_all;" ::: "memory");
  if (aborted) {
    // wait (bounded) for the copies still in flight before the CTA exits: tiles
    // from the one whose wait gave up to the last one issued
    if (tid == 0)
      for (int u = t; u < issued; ++u) mbar_wait(&bar[u % NS], (uint32_t)((u / NS) & 1));
    __syncthreads();
    return;
  }
  // final fold: the block's whole key histogram as a key prefix row
  if (warp == QW && lane == 0) m->tail_q0 = qcur;
  fold<NT>(p, H, T, P, wrow, rows_live && !W64, wide_live && !W64, m);
  // last block: the queries after its last event see every event of the chain,
  // all of it now in the prefix row
  if (b == p.B - 1) {
    for (int64_t i = m->tail_q0 + tid; i < p.Q; i += NT) {
      const uint32_t* r = reinterpret_cast<const uint32_t*>(p.qs + i);
      const uint32_t lo = min(r[1], C), hi = min(r[2], C);
      p.ans[i] = lo < hi ? (int64_t)((uint64_t)__ldcg(P + hi) - (uint64_t)__ldcg(P + lo)) : 0;
    }
    if (warp == QW) qcur = p.Q;
  }
  if (warp == QW && lane == 0) {
    p.btab[2 * b] = qstart;
    p.btab[2 * b + 1] = qcur;
  }
}

// Segment sums of the block prefix rows, column by column (column 0 is always 0).
__global__ void k_chain_colsum(ChainParams p) {
  const uint32_t k = blockIdx.y * 256 + threadIdx.x + 1;
  if (k > p.C) return;
  const int b0 = blockIdx.x * kChainSegRows, b1 = min(p.B, b0 + kChainSegRows);
  uint64_t s = 0;
  for (int b = b0; b < b1; ++b) s += (uint64_t)p.rows[(int64_t)b * (p.C + 1) + k];
  p.seg[(int64_t)blockIdx.x * (p.C + 1) + k] = (int64_t)s;
}

// Rows become exclusive column prefixes: row b = the key prefix of the carry of
// blocks 0 .. b-1.
__global__ void k_chain_colfix(ChainParams p) {
  const uint32_t k = blockIdx.y * 256 + threadIdx.x + 1;
  if (k > p.C) return;
  uint64_t run = 0;
  for (int s = 0; s < (int)blockIdx.x; ++s) run += (uint64_t)p.seg[(int64_t)s * (p.C + 1) + k];
  const int b0 = blockIdx.x * kChainSegRows, b1 = min(p.B, b0 + kChainSegRows);
  for (int b = b0; b < b1; ++b) {
    int64_t* x = p.rows + (int64_t)b * (p.C + 1) + k;
    const uint64_t v = (uint64_t)*x;
    *x = (int64_t)run;
    run += v;
  }
}

// Block b >= 1: every query of the block adds the carry inside [lo, hi).
__global__ void __launch_bounds__(kChainThreads) k_chain_fixup(ChainParams p) {
  const int b = blockIdx.x + 1;
  const int64_t* row = p.rows + (int64_t)b * (p.C + 1);
  const int64_t q0 = p.btab[2 * b], q1 = p.btab[2 * b + 1];
  for (int64_t i = q0 + threadIdx.x; i < q1; i += blockDim.x) {
    const BwQuery q = p.qs[i];
    const uint32_t lo = min(q.lo, p.C), hi = min(q.hi, p.C);
    if (lo < hi) p.ans[i] = (int64_t)((uint64_t)p.ans[i] + (uint64_t)row[hi] - (uint64_t)row[lo]);
  }
}

// Sweep geometries: threads per CTA, events per thread, CTAs per SM the kernel is
// compiled for.  Smaller CTAs give more state blocks and shorter per-tile
// barriers; larger ones amortise the query warp over more appliers.
struct Geometry {
  int threads, ept, minb, stages;
};
constexpr Geometry kGeometries[] = {{128, 4, 5, 3}, {256, 4, 3, 3}, {512, 2, 2, 3}, {256, 4, 4, 2}, {256, 3, 4, 3}};
constexpr int kNumGeometries = 5;

// BW_CHAIN_GEOMETRY=<index into kGeometries> pins the geometry (tuning runs).
// Otherwise, when the events fill every CTA with full state blocks, 256 threads
// with (in this order of preference, measured on byte-dominated chains) 3 events
// each and a three-tile ring at four CTAs per SM (three with the int64 window), 4
// events and a two-tile ring at three or more, 4 events and a three-tile ring at two
// or more; else (few, short state blocks) 512 threads x 2 events, whose wide CTAs
// finish each block soonest, with one block per SM while every block keeps at least
// 2,048 events.  Tiles always stay large: smaller
// tiles shorten the in-tile scans but cost more per tile than they save, even on
// query-dense chains (measured).
int geometry_override() {
  static const int g = [] {
    const char* v = std::getenv("BW_CHAIN_GEOMETRY");
    if (!v || !*v) return -1;
    const int i = std::atoi(v);
    return i >= 0 && i < kNumGeometries ? i : -1;
  }();
  return g;
}

std::once_flag g_attr_once;
cudaError_t g_attr_err = cudaSuccess;

}  // namespace

bool chain_selected(const BwReplayArgs* a) {
  if (!(a->flags & BW_REPLAY_CHAIN_HINT) || (a->flags & BW_REPLAY_GENERAL)) return false;
  if (a->n_keys > kChainMaxKeys || a->n_states < 1) return false;
  if (a->events && (reinterpret_cast<uintptr_t>(a->events) & 15) != 0) return false;
  return (a->flags & BW_REPLAY_CHAIN_KERNEL) || a->n_queries * 8 <= a->n_events;
}

int chain_spec(const BwReplayArgs* a, int sms, ChainSpec& s) {
  s.S = a->n_states;
  s.C = a->n_keys;
  s.E = a->n_events;
  s.Q = a->n_queries;
  // query-dense chains (more than one query per 64 events) keep chunk totals at any
  // domain size: their intervals are probed often, and a probe over chunk totals
  // reads ~width/1024 words per lane instead of ~width/128
  const bool dense = s.Q * 64 > s.E;
  s.nch = (s.C > kFlatKeys || dense) ? (int32_t)((s.C + 31) >> 5) : 0;
  s.w64 = (a->flags & BW_REPLAY_WIDE) && s.C <= kChainMaxKeys64;
  const int hw = s.w64 ? 8 : 4;
  int pin = geometry_override();
  int fit[kNumGeometries];
  size_t need[kNumGeometries];
  for (int g = 0; g < kNumGeometries; ++g) {
    const Geometry& G = kGeometries[g];
    need[g] = sweep_smem(s.C, s.nch, G.threads * G.ept, G.stages, hw).bytes;
    fit[g] = (int)(kSmemPerSM / (need[g] + 1024));
    if (fit[g] > G.minb) fit[g] = G.minb;
  }
  if (pin >= 0 && fit[pin] < 1) pin = -1;
  if (pin < 0 && fit[4] >= (s.w64 ? 3 : 4) && s.E >= (int64_t)sms * fit[4] * kChainMinBlockEvents) pin = 4;
  if (pin < 0 && fit[3] >= 3 && s.E >= (int64_t)sms * fit[3] * kChainMinBlockEvents) pin = 3;
  if (pin < 0 && fit[1] >= 2 && s.E >= (int64_t)sms * fit[1] * kChainMinBlockEvents) pin = 1;
  // too few events to fill the GPU with full blocks: the widest CTA (512 threads)
  // finishes each short block soonest (measured on the 1M-event plain chain)
  const bool few = pin < 0;
  if (few && fit[2] >= 1) pin = 2;
  int best = -1, best_threads = 0;
  for (int g = 0; g < kNumGeometries; ++g) {
    const Geometry& G = kGeometries[g];
    const size_t smem = need[g];
    const int ctas = fit[g];
    if (ctas < 1) continue;
    if (pin >= 0 ? g == pin : ctas * G.threads >= best_threads) {
      best = g;
      best_threads = ctas * G.threads;
      s.threads = G.threads;
      s.ept = G.ept;
      s.geometry = g;
      s.smem = smem;
      s.ctas_per_sm = ctas;
    }
  }
  if (best < 0) return BW_EINVAL;
  int64_t B = a->blocks > 0 ? a->blocks : (s.E + kChainMinBlockEvents - 1) / kChainMinBlockEvents;
  // few events: one block per SM when every block still gets 2,048 events or more
  if (a->blocks <= 0 && few && B < sms) B = std::min<int64_t>(sms, std::max<int64_t>(B, s.E / 2048));
  const int64_t cap = (int64_t)sms * s.ctas_per_sm;
  if (a->blocks <= 0 && B > cap) B = cap;
  if (B > s.E) B = s.E;
  if (B < 1) B = 1;
  if (B > (1 << 20)) return BW_EINVAL;
  s.B = (int32_t)B;
  s.nseg = (s.B + kChainSegRows - 1) / kChainSegRows;
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  size_t o = 256;   // status word
  s.off_btab = o;  o = al(o + (size_t)s.B * 16);
  s.off_rows = o;  o = al(o + (size_t)s.B * (s.C + 1) * 8);
  s.off_wide = o;  o = al(o + (size_t)s.B * s.C * 8);
  s.off_seg = o;   o = al(o + (size_t)s.nseg * (s.C + 1) * 8);
  s.total = o;
  return 0;
}

int chain_enqueue(const ChainSpec& s, const BwReplayArgs* a, EventSet* evs, int* kernels) {
  std::call_once(g_attr_once, [] {
    const cudaFuncAttribute A = cudaFuncAttributeMaxDynamicSharedMemorySize;
    const void* fns[] = {(const void*)k_chain_sweep<128, 4, 5, 3, false>, (const void*)k_chain_sweep<256, 4, 3, 3, false>,
                         (const void*)k_chain_sweep<512, 2, 2, 3, false>, (const void*)k_chain_sweep<256, 4, 4, 2, false>,
                         (const void*)k_chain_sweep<256, 3, 4, 3, false>, (const void*)k_chain_sweep<128, 4, 5, 3, true>,
                         (const void*)k_chain_sweep<256, 4, 3, 3, true>, (const void*)k_chain_sweep<512, 2, 2, 3, true>,
                         (const void*)k_chain_sweep<256, 4, 4, 2, true>, (const void*)k_chain_sweep<256, 3, 4, 3, true>};
    for (const void* f : fns)
      if (g_attr_err == cudaSuccess) g_attr_err = cudaFuncSetAttribute(f, A, kSmemLimit);
  });
  if (g_attr_err != cudaSuccess) return report(g_attr_err, "chain sweep attribute");
  cudaStream_t st = static_cast<cudaStream_t>(a->stream);
  char* ws = static_cast<char*>(a->workspace);
  ChainParams p;
  p.ev = reinterpret_cast<const uint4*>(a->events);
  p.qs = a->queries;
  p.ans = a->answers;
  p.parent = a->parent;
  p.E = s.E;
  p.Q = s.Q;
  p.S = s.S;
  p.C = s.C;
  p.B = s.B;
  p.nch = s.nch;
  p.nseg = s.nseg;
  p.rows = reinterpret_cast<int64_t*>(ws + s.off_rows);
  p.wide = reinterpret_cast<int64_t*>(ws + s.off_wide);
  p.btab = reinterpret_cast<int64_t*>(ws + s.off_btab);
  p.seg = reinterpret_cast<int64_t*>(ws + s.off_seg);
  p.status = reinterpret_cast<int32_t*>(ws);
  int rc = report(cudaMemsetAsync(ws, 0, 4, st), "status reset");
  if (rc) return rc;
  if (evs) {
    for (int i = 0; i <= BW_STAGE_SWEEP; ++i)
      if ((rc = report(cudaEventRecord(evs->ev[i], st), "event record"))) return rc;
  }
  switch (s.geometry * 2 + (s.w64 ? 1 : 0)) {
    case 0: k_chain_sweep<128, 4, 5, 3, false><<<s.B, 128, s.smem, st>>>(p); break;
    case 1: k_chain_sweep<128, 4, 5, 3, true><<<s.B, 128, s.smem, st>>>(p); break;
    case 2: k_chain_sweep<256, 4, 3, 3, false><<<s.B, 256, s.smem, st>>>(p); break;
    case 3: k_chain_sweep<256, 4, 3, 3, true><<<s.B, 256, s.smem, st>>>(p); break;
    case 4: k_chain_sweep<512, 2, 2, 3, false><<<s.B, 512, s.smem, st>>>(p); break;
    case 5: k_chain_sweep<512, 2, 2, 3, true><<<s.B, 512, s.smem, st>>>(p); break;
    case 6: k_chain_sweep<256, 4, 4, 2, false><<<s.B, 256, s.smem, st>>>(p); break;
    case 7: k_chain_sweep<256, 4, 4, 2, true><<<s.B, 256, s.smem, st>>>(p); break;
    case 8: k_chain_sweep<256, 3, 4, 3, false><<<s.B, 256, s.smem, st>>>(p); break;
    default: k_chain_sweep<256, 3, 4, 3, true><<<s.B, 256, s.smem, st>>>(p); break;
  }
  int k = 1;
  if ((rc = report(cudaGetLastError(), "chain sweep launch"))) return rc;
  if (evs && (rc = report(cudaEventRecord(evs->ev[BW_STAGE_SWEEP + 1], st), "event record"))) return rc;
  if (s.B > 1) {
    const dim3 g((unsigned)s.nseg, (s.C + 255) / 256);   // columns 1 .. C
    k_chain_colsum<<<g, 256, 0, st>>>(p);
    k_chain_colfix<<<g, 256, 0, st>>>(p);
    k_chain_fixup<<<s.B - 1, kChainThreads, 0, st>>>(p);
    k += 3;
    if ((rc = report(cudaGetLastError(), "chain carry launch"))) return rc;
  }
  if (evs) {
    evs->chain = 1;
    if ((rc = report(cudaEventRecord(evs->ev[BW_STAGE_COUNT + 1], st), "event record"))) return rc;
  }
  if (kernels) *kernels += k;
  return 0;
}

}  // namespace bw
