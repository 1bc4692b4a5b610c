// bw_esweep.cu -- Euler-tile sweep of the general (tree) pipeline.
//
// A state block is a range [t0, t1) of one tree's Euler steps: an enter step applies
// its state's events, the matching exit step removes them, and the queries of a
// state are answered right after its enter step.  Flattened in step order, a block
// is therefore a chain of signed events, and this sweep replays it the way the chain
// path replays a chain (bw_chain.cu), one block at a time per persistent CTA (blocks
// from the shared queue, largest first):
//
//   * two producer warps.  The planner walks the block's step descriptors (a
//     shared-memory ring refilled by cp.async up to 192 steps ahead), 64 steps per
//     batch (two per lane), and cuts the flattened sequence into tiles of up to
//     kEsTile events and kEsQB queries; it hands each batch plan to the issuer
//     through two shared plan buffers and named barriers.  The issuer turns
//     consecutive steps whose event ranges are adjacent in memory -- the enters of a
//     run of consecutive states, or the exits of such a run, which come in descending
//     state order -- into one cp.async.bulk copy into the tile's stage, completed on
//     the stage's "full" mbarrier.  Enter events fill the stage from the front in step
//     order and exit events from the back, so an event's sign is its side of the
//     stage; a query records how many enter and exit events of the tile precede it,
//     and its bounds arrive by cp.async tracked by the same barrier;
//   * sixteen consumer warps take a tile: each thread loads its two events (and, for
//     int32 windows, repacks them as signed (key, delta) pairs), each warp its
//     queries, and the stage is released on its "empty" mbarrier (int64 windows: after
//     the scans, which then read the stage itself).  One warp per
//     query: before a consumer barrier the probe of the window over [lo, hi) as it
//     stood before the tile, after it the scan of the tile's events before the query
//     plus the carried key-prefix row of the block -- overlapping the other warps'
//     updates, since the scan reads only the packed tile -- then the updates;
//   * the window is a flat histogram in shared memory: over the keys themselves when
//     the tree's key domain fits it, else over the block's key ranks one rank slice at
//     a time (popcount rank table of the prepare pass); int32 entries when the block's
//     applied |delta| sum is below 2^31 (every partial sum is then exact), int64 ones
//     otherwise; 32-entry chunk totals for windows above 4,096 entries.
//
// Per tile the consumers meet at most twice: before the probes (the previous tiles'
// updates are complete; the barrier also agrees on lost waits) and after them.  Every
// mbarrier wait is bounded; a lost wait sets BW_STATUS_TIMEOUT, every role stops
// (the planner ends the pass with an empty plan so that the issuer does too), and the
// issuer waits (bounded) for its copies in flight before the CTA exits.
#include <cuda_runtime.h>
#include <cstdint>

#include "bw_gpu.h"
#include "bw_common.cuh"
#include "bw_pipeline.cuh"

namespace bw {
namespace {

constexpr int kEsNC = 512;                 // consumer threads
constexpr int kEsNWC = kEsNC / 32;         // consumer warps
constexpr int kEsThreads = kEsNC + 64;     // plus the producer warps (planner, issuer)
constexpr int kEsEPT = 2;                  // events per consumer thread per tile
constexpr int kEsTile = kEsNC * kEsEPT;    // events per tile
constexpr int kEsStages = 3;
constexpr int kEsQB = 64;                  // queries per tile
constexpr int kEsQW = kEsQB / kEsNWC;      // queries per consumer warp per tile
constexpr uint32_t kEsFlat = 4096;         // windows up to this size keep no chunk totals
constexpr int kEsRing = 256;               // planner's descriptor ring (steps)
constexpr uint32_t kEsWaitLimit = 1u << 22;
constexpr uint32_t kFull = 0xffffffffu;

struct EsMeta {
  int32_t nf, nb, nq, last;   // front (enter) events, back (exit) events, queries, last tile of the pass
};
struct EsCtl {
  int32_t ticket, abort, pad0, pad1;
};

// Dynamic shared memory (all regions 16-byte aligned).
struct EsSmem {
  size_t H, T, bits, rl, stage, pack, q, meta, bar, ctl, ring, plan, pmeta, bytes;
};
__host__ __device__ constexpr size_t es_al(size_t x) { return (x + 15) & ~size_t(15); }
__host__ __device__ constexpr EsSmem es_smem() {
  EsSmem L{};
  size_t o = 0;
  L.H = o;     o = es_al(o + (size_t)kEsCap32 * 4);                 // int32 x cap32 == int64 x cap64
  L.T = o;     o = es_al(o + (size_t)(kEsCap32 / 32) * 4);
  L.bits = o;  o = es_al(o + (size_t)kWinWords * 8);
  L.rl = o;    o = es_al(o + ((size_t)kWinWords + 2) * 2);          // slice-local ranks, uint16
  L.stage = o; o = es_al(o + (size_t)kEsStages * kEsTile * 16);
  L.pack = o;  o = es_al(o + (size_t)kEsTile * 8);                   // the tile as signed (key, int32 delta)
  L.q = o;     o = es_al(o + (size_t)kEsStages * kEsQB * 16);
  L.meta = o;  o = es_al(o + (size_t)kEsStages * sizeof(EsMeta));
  L.bar = o;   o = es_al(o + (size_t)2 * kEsStages * 8);
  L.ctl = o;   o = es_al(o + sizeof(EsCtl));
  L.ring = o;  o = es_al(o + (size_t)kEsRing * 16);
  L.plan = o;  o = es_al(o + (size_t)2 * 64 * 16);                  // two batch plans
  L.pmeta = o; o = es_al(o + (size_t)2 * 16);
  L.bytes = o;
  return L;
}
static_assert(es_smem().bytes <= (size_t)kSmemLimit, "Euler sweep shared memory");
static_assert(kEsCap64 * 8 == kEsCap32 * 4, "int32 and int64 windows share the region");
static_assert(sizeof(StepDesc) == 16, "step descriptors are read as uint4 {e0, q0, ne, nq}");
static_assert(kEsTile <= 2047 && kEsQB <= 127, "the producer's packed counts");

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Transaction bytes a stage barrier waits for, announced before the copies are
// issued so that its transaction count never runs below zero.
__device__ __forceinline__ void mbar_expect(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// One bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned) into
// shared memory, completing on the stage barrier.
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Bounded wait for phase `parity` of a stage barrier; false when it never completed.
// After two failed polls the waiter sleeps between polls: a polling warp shares the
// shared-memory pipe with the producer's shuffles and the consumers' atomics.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t i = 0; i < kEsWaitLimit; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
    if (i >= 2) __nanosleep(32);
  }
  return false;
}
// Consumer-only barriers (named barrier 1, the producer warp never joins).
__device__ __forceinline__ void cons_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kEsNC) : "memory"); }
__device__ __forceinline__ bool cons_sync_or(bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.or.pred p, 1, %2, q;\n\tselp.u32 %0, 1, 0, p;\n}"
      : "=r"(r)
      : "r"((uint32_t)v), "n"(kEsNC)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void es_status(int32_t* st, int32_t code) {
  if (*reinterpret_cast<volatile int32_t*>(st) == 0) atomicCAS(st, 0, code);
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

// Rank of key offset x inside the slice: uint16 slice-local rank table + popcount.
__device__ __forceinline__ uint32_t es_rank(const uint64_t* bits, const uint16_t* rl, uint32_t x) {
  const uint32_t wi = x >> 6;
  return (uint32_t)rl[wi] + (uint32_t)__popcll(bits[wi] & ((1ull << (x & 63)) - 1ull));
}

// What one pass (one rank slice of one block) needs.
struct EsPass {
  int32_t t0, t1;
  uint32_t klo, khi;      // keys of the slice
  uint32_t nr;            // window entries
  int32_t nch;            // chunk totals (0: flat probes)
  bool dense, first;
  const int64_t* crow;    // carried key-prefix row (nullptr: the block starts its tree)
};

// ------------------------------------------------------------------ producer
// Two warps: the planner walks the descriptors and cuts the tiles; the issuer merges
// copy groups and issues the copies.  A batch is 64 consecutive steps, two per lane
// (lane l: steps 2l and 2l + 1).  Batch plans go from the planner to the issuer
// through two shared plan buffers, each guarded by a pair of named barriers (plan b
// written: kBarPlanFull + b; plan b read: kBarPlanFree + b; 64 threads each).
constexpr int kBarPlanFull = 2;
constexpr int kBarPlanFree = 4;
constexpr int kEsBatch = 64;
__device__ __forceinline__ void pbar_arrive(int id) { asm volatile("bar.arrive %0, 64;" ::"r"(id) : "memory"); }
__device__ __forceinline__ void pbar_sync(int id) { asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory"); }

struct EsPlanMeta {
  uint32_t nq;     // queries of the tile before the batch | after it << 16
  uint32_t flags;  // 1: the batch ends its tile, 2: it ends the pass
  uint32_t nf, nb; // the tile's front and back events after the batch
};
constexpr uint32_t kPlanTileEnd = 1, kPlanPassEnd = 2;

// The planner's cursor: step ct with its first coe events and coq queries already
// taken; the descriptors of steps below wb have been requested into the ring (slot
// u % kEsRing), 32 steps per cp.async group, up to kEsRing - kEsBatch steps ahead.
struct EsCursor {
  int32_t ct, coe, coq, wb;
};
__device__ __forceinline__ void es_ring_request(const EsParams& p, uint4* ring, EsCursor& c, int32_t t1, int lane) {
  while (c.wb < t1 && c.wb < c.ct + (kEsRing - kEsBatch)) {
    const int32_t u = c.wb + lane;
    if (u < t1) cp_async16(ring + (u & (kEsRing - 1)), p.desc + u);
    asm volatile("cp.async.commit_group;" ::: "memory");
    c.wb += 32;
  }
}
// Wait until the descriptors of steps [ct, ct + kEsBatch) have landed (the groups of
// later steps may stay in flight), then make them visible to the whole warp.
__device__ __forceinline__ void es_ring_ready(const EsCursor& c, int32_t t0) {
  const int32_t later = (c.wb - t0) / 32 - (c.ct + kEsBatch - 1 - t0) / 32 - 1;   // groups past the batch
  if (later >= 5) asm volatile("cp.async.wait_group 5;" ::: "memory");
  else if (later == 4) asm volatile("cp.async.wait_group 4;" ::: "memory");
  else if (later == 3) asm volatile("cp.async.wait_group 3;" ::: "memory");
  else if (later == 2) asm volatile("cp.async.wait_group 2;" ::: "memory");
  else if (later == 1) asm volatile("cp.async.wait_group 1;" ::: "memory");
  else asm volatile("cp.async.wait_group 0;" ::: "memory");
  __syncwarp();
}

// One step's part of a batch plan: events [src, src + te) of sign ex, queries
// [q0, q0 + tq) with their first slot xq in the batch, the front slot of an enter
// step's first event and the exit events of the tile before the step.
__device__ __forceinline__ uint4 es_rec(uint32_t src, uint32_t q0, int32_t te, bool ex, int32_t tq, int32_t xq,
                                        int32_t fpos, int32_t boff) {
  return make_uint4(src, q0, (uint32_t)te | (ex ? 1u << 11 : 0u) | ((uint32_t)tq << 12) | ((uint32_t)xq << 19),
                    (uint32_t)fpos | ((uint32_t)boff << 16));
}

// Planner: every batch of the pass, tiles cut at kEsTile events or kEsQB queries.
// On an abort it ends the pass with an empty plan so that the issuer stops too.
__device__ void es_plan(const EsParams& p, const EsPass& ps, uint4* ring, uint4* plan, EsPlanMeta* pmeta,
                        const EsCtl* ctl, int lane) {
  EsCursor c;
  c.ct = ps.t0; c.coe = 0; c.coq = 0; c.wb = ps.t0;
  const int32_t t1 = ps.t1;
  int32_t nf = 0, nb = 0, nq = 0;   // the tile so far: front (enter) events, back (exit) events, queries
  uint32_t pb = 0;                  // batches planned in this pass
  for (;;) {
    const bool stop = *reinterpret_cast<const volatile int32_t*>(&ctl->abort) != 0;
    uint4 rec0 = make_uint4(0, 0, 0, 0), rec1 = rec0;
    uint32_t flags = 0, nq0 = (uint32_t)nq;
    if (stop) {
      flags = kPlanTileEnd | kPlanPassEnd;
    } else {
      es_ring_request(p, ring, c, t1, lane);
      es_ring_ready(c, ps.t0);
      const int32_t u0 = c.ct + 2 * lane, u1 = u0 + 1;
      const bool v0 = u0 < t1, v1 = u1 < t1;
      const uint4 d0 = ring[u0 & (kEsRing - 1)], d1 = ring[u1 & (kEsRing - 1)];   // StepDesc {e0, q0, ne, nq}
      const bool ex0 = (int32_t)d0.w < 0, ex1 = (int32_t)d1.w < 0;
      int32_t ne0 = v0 ? (int32_t)d0.z : 0, qn0 = v0 && (int32_t)d0.w > 0 ? (int32_t)d0.w : 0;
      const int32_t ne1 = v1 ? (int32_t)d1.z : 0, qn1 = v1 && (int32_t)d1.w > 0 ? (int32_t)d1.w : 0;
      uint32_t src0 = d0.x, qa0 = d0.y;
      if (lane == 0) {
        ne0 -= c.coe; src0 += (uint32_t)c.coe;
        qn0 -= c.coq; qa0 += (uint32_t)c.coq;
      }
      // counts clamped below the tile limits (a step that fits has exact counts; the
      // first one that does not is the only one cut), summed per lane (saturating: a
      // lane past the cut is never used), then scanned over the lanes
      const int32_t c0 = min(ne0, kEsTile + 1), c1 = min(ne1, kEsTile + 1);
      const int32_t cq0 = min(qn0, kEsQB + 1), cq1 = min(qn1, kEsQB + 1);
      const uint32_t pe = (uint32_t)min(c0 + c1, 2047), pq = (uint32_t)min(cq0 + cq1, 127);
      const uint32_t pxv = (uint32_t)min((ex0 ? c0 : 0) + (ex1 ? c1 : 0), 2047);
      uint32_t sa = pe | (pq << 16), sx = pxv;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, sa, o), yx = __shfl_up_sync(kFull, sx, o);
        if (lane >= o) { sa += y; sx += yx; }
      }
      const int32_t xe = (int32_t)(sa & 0xffffu) - (int32_t)pe;   // events before the lane's pair
      const int32_t xq = (int32_t)(sa >> 16) - (int32_t)pq;       // queries before it
      const int32_t xx = (int32_t)sx - (int32_t)pxv;              // exit events before it
      const int32_t room_e = kEsTile - nf - nb, room_q = kEsQB - nq;
      const bool f0 = v0 && xe + c0 <= room_e && xq + cq0 <= room_q;
      const bool f1 = f0 && v1 && xe + c0 + c1 <= room_e && xq + cq0 + cq1 <= room_q;
      // K: the first step of the batch that is not taken whole (64: none)
      const uint32_t m1 = __ballot_sync(kFull, !f1);
      int K = 64;
      if (m1) {
        const int L = __ffs(m1) - 1;
        K = 2 * L + (__shfl_sync(kFull, f0 ? 1 : 0, L) ? 1 : 0);
      }
      int32_t te0 = 0, tq0 = 0, te1 = 0, tq1 = 0;
      const int s0i = 2 * lane, s1i = s0i + 1;
      if (s0i < K) {
        te0 = ne0; tq0 = qn0;
      } else if (s0i == K && v0) {
        te0 = min(ne0, room_e - xe);
        tq0 = te0 == ne0 ? min(qn0, room_q - xq) : 0;
      }
      if (s1i < K) {
        te1 = ne1; tq1 = qn1;
      } else if (s1i == K && v1) {
        te1 = min(ne1, room_e - xe - c0);
        tq1 = te1 == ne1 ? min(qn1, room_q - xq - cq0) : 0;
      }
      const int32_t fpos0 = nf + (xe - xx), boff0 = nb + xx;
      const int32_t fpos1 = fpos0 + (ex0 ? 0 : te0), boff1 = boff0 + (ex0 ? te0 : 0);
      rec0 = es_rec(src0, qa0, te0, ex0, tq0, xq, fpos0, boff0);
      rec1 = es_rec(d1.x, d1.y, te1, ex1, tq1, xq + tq0, fpos1, boff1);
      const uint32_t tt = (uint32_t)(te0 + te1) | ((uint32_t)(tq0 + tq1) << 16);   // <= kEsTile, kEsQB
      const uint32_t sum = __reduce_add_sync(kFull, tt);
      const uint32_t xsum = __reduce_add_sync(kFull, (uint32_t)((ex0 ? te0 : 0) + (ex1 ? te1 : 0)));
      nb += (int32_t)xsum;
      nf += (int32_t)(sum & 0xffffu) - (int32_t)xsum;
      nq += (int32_t)(sum >> 16);
      if (K == 64) {
        c.ct += 64; c.coe = 0; c.coq = 0;
      } else if (c.ct + K >= t1) {
        c.ct = t1; c.coe = 0; c.coq = 0;
      } else {
        const uint32_t kt = __shfl_sync(kFull, (K & 1) ? ((uint32_t)te1 | ((uint32_t)tq1 << 16))
                                                       : ((uint32_t)te0 | ((uint32_t)tq0 << 16)), K >> 1);
        c.coe = (K == 0 ? c.coe : 0) + (int32_t)(kt & 0xffffu);
        c.coq = (K == 0 ? c.coq : 0) + (int32_t)(kt >> 16);
        c.ct += K;
      }
      if (c.ct >= t1) flags = kPlanTileEnd | kPlanPassEnd;
      else if (nf + nb >= kEsTile || nq >= kEsQB) flags = kPlanTileEnd;
    }
    const int b = (int)(pb & 1u);
    if (pb >= 2) pbar_sync(kBarPlanFree + b);   // the issuer has read this buffer's last plan
    plan[b * kEsBatch + 2 * lane] = rec0;
    plan[b * kEsBatch + 2 * lane + 1] = rec1;
    if (lane == 0) {
      EsPlanMeta m;
      m.nq = nq0 | ((uint32_t)nq << 16); m.flags = flags; m.nf = (uint32_t)nf; m.nb = (uint32_t)nb;
      pmeta[b] = m;
    }
    pbar_arrive(kBarPlanFull + b);
    ++pb;
    if (flags & kPlanTileEnd) { nf = 0; nb = 0; nq = 0; }
    if (flags & kPlanPassEnd) break;
  }
  // balance the free barriers of the last (up to) two plans
  for (uint32_t q = pb > 2 ? pb - 2 : 0; q < pb; ++q) pbar_sync(kBarPlanFree + (int)(q & 1u));
  asm volatile("cp.async.wait_all;" ::: "memory");   // ring copies of this pass landed
}

// Next copy-group break after batch position i = 2 * lane + w (0..63; 64 if none):
// break bits b0 (even positions, one per lane) and b1 (odd positions).
__device__ __forceinline__ int es_next_break(uint32_t b0, uint32_t b1, int lane, int w) {
  const uint32_t hi0 = lane + 1 < 32 ? (b0 & (kFull << (lane + 1))) : 0u;                 // even positions > 2 lane
  const uint32_t hi1 = w == 0 ? (b1 & (kFull << lane)) : (lane + 1 < 32 ? (b1 & (kFull << (lane + 1))) : 0u);
  const int e = hi0 ? 2 * (__ffs(hi0) - 1) : 64, o = hi1 ? 2 * (__ffs(hi1) - 1) + 1 : 64;
  return e < o ? e : o;
}

// Issuer: turns the plans of a pass into stage copies, query records and stage
// metadata, one tile per stage.  `cnt` counts tiles (the consumers' sequence).
// Returns false when a wait for a free stage was lost (it still reads every plan).
__device__ bool es_issue(const EsParams& p, unsigned char* sm, const uint4* plan, const EsPlanMeta* pmeta,
                         uint32_t& cnt, int lane) {
  constexpr EsSmem L = es_smem();
  uint4* stages = reinterpret_cast<uint4*>(sm + L.stage);
  uint4* qls = reinterpret_cast<uint4*>(sm + L.q);
  EsMeta* metas = reinterpret_cast<EsMeta*>(sm + L.meta);
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + L.bar);
  uint64_t* empty = full + kEsStages;
  EsCtl* ctl = reinterpret_cast<EsCtl*>(sm + L.ctl);
  bool ok = true, fresh = true, qcopies = false;
  uint32_t pb = 0;
  for (;;) {
    const int st = (int)(cnt % kEsStages);
    if (fresh && ok) {   // first batch of a tile: the consumers released the stage
      ok = !*reinterpret_cast<volatile int32_t*>(&ctl->abort) && mbar_wait(&empty[st], ((cnt / kEsStages) & 1u) ^ 1u);
      if (!ok && lane == 0) {
        es_status(p.status, BW_STATUS_TIMEOUT);
        ctl->abort = 1;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      fresh = false;
    }
    const int b = (int)(pb & 1u);
    pbar_sync(kBarPlanFull + b);
    const uint4 r0 = plan[b * kEsBatch + 2 * lane], r1 = plan[b * kEsBatch + 2 * lane + 1];
    const EsPlanMeta m = pmeta[b];
    pbar_arrive(kBarPlanFree + b);
    ++pb;
    if (ok) {
      uint4* sg = stages + (size_t)st * kEsTile;
      uint4* ql = qls + (size_t)st * kEsQB;
      uint64_t* fb = &full[st];
      const uint32_t te0 = r0.z & 0x7ffu, te1 = r1.z & 0x7ffu;
      const bool ex0 = (r0.z >> 11) & 1u, ex1 = (r1.z >> 11) & 1u;
      const uint32_t a0 = r0.x, z0 = a0 + te0, a1 = r1.x, z1 = a1 + te1;
      // copy groups in step order: a step joins the previous step's group when both
      // take events of the same sign from adjacent ranges (ascending: a run of enters;
      // descending: a run of exits, whose order inside the group does not matter -- no
      // query sits between exits).  An enter group lands at [fpos, fpos + n) in step
      // order, an exit group at [kEsTile - boff - n, kEsTile - boff).
      const uint32_t pa = __shfl_up_sync(kFull, a1, 1), pz = __shfl_up_sync(kFull, z1, 1);
      const uint32_t ptx = __shfl_up_sync(kFull, te1 | (ex1 ? 0x80000000u : 0u), 1);
      const bool mg0 = lane > 0 && te0 > 0 && (ptx & 0x7fffffffu) != 0 && (ptx >> 31) == (ex0 ? 1u : 0u) &&
                       (pz == a0 || (ex0 && z0 == pa));
      const bool mg1 = te1 > 0 && te0 > 0 && ex0 == ex1 && (z0 == a1 || (ex1 && z1 == a0));
      const bool h0 = te0 > 0 && !mg0, h1 = te1 > 0 && !mg1;
      const uint32_t b0 = __ballot_sync(kFull, h0 || te0 == 0), b1 = __ballot_sync(kFull, h1 || te1 == 0);
      // the last member of each head's group: the step before the next break
      const int l0 = es_next_break(b0, b1, lane, 0) - 1, l1 = es_next_break(b0, b1, lane, 1) - 1;
      const uint32_t x0a = __shfl_sync(kFull, a0, l0 >> 1), x0b = __shfl_sync(kFull, a1, l0 >> 1);
      const uint32_t y0a = __shfl_sync(kFull, z0, l0 >> 1), y0b = __shfl_sync(kFull, z1, l0 >> 1);
      const uint32_t x1a = __shfl_sync(kFull, a0, l1 >> 1), x1b = __shfl_sync(kFull, a1, l1 >> 1);
      const uint32_t y1a = __shfl_sync(kFull, z0, l1 >> 1), y1b = __shfl_sync(kFull, z1, l1 >> 1);
      const uint32_t la0 = (l0 & 1) ? x0b : x0a, lz0 = (l0 & 1) ? y0b : y0a;
      const uint32_t la1 = (l1 & 1) ? x1b : x1a, lz1 = (l1 & 1) ? y1b : y1a;
      const uint32_t bytes = __reduce_add_sync(kFull, te0 + te1) * 16u;
      if (lane == 0 && bytes) mbar_expect(fb, bytes);   // the batch's bytes, before its copies
      __syncwarp();
      if (h0) {
        const uint32_t s0 = a0 < la0 ? a0 : la0, s1 = z0 > lz0 ? z0 : lz0, n = s1 - s0;
        const int32_t slot = ex0 ? kEsTile - (int32_t)(r0.w >> 16) - (int32_t)n : (int32_t)(r0.w & 0xffffu);
        bulk_copy(sg + slot, p.ev + s0, n * 16u, fb);
      }
      if (h1) {
        const uint32_t s0 = a1 < la1 ? a1 : la1, s1 = z1 > lz1 ? z1 : lz1, n = s1 - s0;
        const int32_t slot = ex1 ? kEsTile - (int32_t)(r1.w >> 16) - (int32_t)n : (int32_t)(r1.w & 0xffffu);
        bulk_copy(sg + slot, p.ev + s0, n * 16u, fb);
      }
      // queries of an enter step: after all of its events; bounds by cp.async
#pragma unroll
      for (int w = 0; w < 2; ++w) {
        const uint4 rr = w ? r1 : r0;
        const uint32_t te = rr.z & 0x7ffu, tq = (rr.z >> 12) & 0x7fu, xq = rr.z >> 19;
        for (uint32_t r = 0; r < tq; ++r) {
          const uint32_t* qr = reinterpret_cast<const uint32_t*>(p.qs + (rr.y + r));
          uint4* e = ql + ((m.nq & 0xffffu) + xq + r);
          cp_async4(&e->x, qr + 1);
          cp_async4(&e->y, qr + 2);
          e->z = ((rr.w & 0xffffu) + te) | (rr.w & 0xffff0000u);
          e->w = rr.y + r;
          qcopies = true;
        }
      }
      if (m.flags & kPlanTileEnd) {
        if (lane == 0) {
          EsMeta* mt = metas + st;
          mt->nf = (int32_t)m.nf;
          mt->nb = (int32_t)m.nb;
          mt->nq = (int32_t)(m.nq >> 16);
          mt->last = (m.flags & kPlanPassEnd) ? 1 : 0;
        }
        // the stage completes when this lane's query copies have landed (the arrive
        // adds one pending arrival now and removes it when the copies complete)
        if (qcopies) asm volatile("cp.async.mbarrier.arrive.shared::cta.b64 [%0];" ::"r"(smem_u32(fb)) : "memory");
        qcopies = false;
        __threadfence_block();
        __syncwarp();
        if (lane == 0) mbar_arrive(fb);
      }
    }
    if (m.flags & kPlanTileEnd) {
      if (ok) ++cnt;
      fresh = true;
    }
    if (m.flags & kPlanPassEnd) return ok;
  }
}

// ------------------------------------------------------------------ consumers
// Lane share of the window sum over entries [ra, rb) (ra < rb <= nr): partial chunks
// from H, whole chunks from T; or flat 128-bit reads (H padded to whole uint4s).
template <typename HT>
__device__ __forceinline__ HT es_probe(const HT* H, const HT* T, int32_t nch, uint32_t ra, uint32_t rb, int lane) {
  HT s = 0;
  if (nch) {
    const uint32_t clo = (ra + 31) >> 5, chi = rb >> 5;
    if (clo >= chi) {
      for (uint32_t k = ra + lane; k < rb; k += 32) s += H[k];
      return s;
    }
    const uint32_t x = ra + lane, y = (chi << 5) + lane;
    if (x < (clo << 5)) s += H[x];
    if (y < rb) s += H[y];
    for (uint32_t c = clo + lane; c < chi; c += 32) s += T[c];
    return s;
  }
  constexpr uint32_t per = 16 / sizeof(HT);
  const uint32_t w = rb - ra;
  for (uint32_t k = (ra & ~(per - 1)) + per * lane; k < rb; k += 32 * per) {
    const uint32_t d = k - ra;
    if constexpr (sizeof(HT) == 4) {
      const int4 v = *reinterpret_cast<const int4*>(H + k);
      s += (d < w ? (HT)v.x : 0) + (d + 1 < w ? (HT)v.y : 0) + (d + 2 < w ? (HT)v.z : 0) + (d + 3 < w ? (HT)v.w : 0);
    } else {
      const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(H + k);
      s += (d < w ? (HT)v.x : 0) + (d + 1 < w ? (HT)v.y : 0);
    }
  }
  return s;
}

// Lane share of the delta sum of stage events [j0, j1) with keys in [a, a + w).
template <typename HT>
__device__ __forceinline__ HT es_scan(const uint4* tile, uint32_t j0, uint32_t j1, uint32_t a, uint32_t w, int lane) {
  HT s = 0;
#pragma unroll 4
  for (uint32_t j = j0 + lane; j < j1; j += 32) {
    const uint4 e = tile[j];
    if (e.y - a < w) {
      if constexpr (sizeof(HT) == 4) s += (HT)e.z;
      else s += ((HT)e.w << 32) | e.z;
    }
  }
  return s;
}

// Lane share of the signed delta sum of packed events [j0, j1) with keys in [a, a + w).
__device__ __forceinline__ int32_t es_scan_packed(const uint2* pk, uint32_t j0, uint32_t j1, uint32_t a, uint32_t w,
                                                  int lane) {
  int32_t s = 0;
#pragma unroll 4
  for (uint32_t j = j0 + lane; j < j1; j += 32) {
    const uint2 e = pk[j];
    if (e.x - a < w) s += (int32_t)e.y;
  }
  return s;
}

// One pass of the consumers over the tiles of a pass.  Returns false on a lost wait.
template <typename HT>
__device__ bool es_consume(const EsParams& p, const EsPass& ps, unsigned char* sm, uint32_t& cnt, uint32_t& bad) {
  constexpr EsSmem L = es_smem();
  HT* H = reinterpret_cast<HT*>(sm + L.H);
  HT* T = reinterpret_cast<HT*>(sm + L.T);
  const uint64_t* bits = reinterpret_cast<const uint64_t*>(sm + L.bits);
  const uint16_t* rl = reinterpret_cast<const uint16_t*>(sm + L.rl);
  const uint4* stages = reinterpret_cast<const uint4*>(sm + L.stage);
  uint2* packed = reinterpret_cast<uint2*>(sm + L.pack);
  const uint4* qls = reinterpret_cast<const uint4*>(sm + L.q);
  const EsMeta* metas = reinterpret_cast<const EsMeta*>(sm + L.meta);
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + L.bar);
  uint64_t* empty = full + kEsStages;
  EsCtl* ctl = reinterpret_cast<EsCtl*>(sm + L.ctl);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t klo = ps.klo, khi = ps.khi;
  auto rank_of = [&](uint32_t k) -> uint32_t {   // window entry of a bound inside [klo, khi]
    if (ps.dense) return k;
    return k >= khi ? ps.nr : es_rank(bits, rl, k - klo);
  };
  for (;;) {
    const int s = (int)(cnt % kEsStages);
    const uint32_t ph = (cnt / kEsStages) & 1u;
    // warp 0 polls the stage barrier; the others wait at the consumer barrier, which
    // also agrees on lost waits and completes the previous tiles' updates
    const bool ok = warp == 0 ? mbar_wait(&full[s], ph) : true;
    if (cons_sync_or(!ok || *reinterpret_cast<volatile int32_t*>(&ctl->abort) != 0)) {
      if (tid == 0) {
        es_status(p.status, BW_STATUS_TIMEOUT);
        ctl->abort = 1;
      }
      return false;
    }
    if (warp != 0) mbar_wait(&full[s], ph);   // complete: this thread's acquire of the stage
    const EsMeta m = metas[s];
    const uint4* tile = stages + (size_t)s * kEsTile;
    const int32_t back = kEsTile - m.nb;      // first exit slot
    uint4 it[kEsEPT];
#pragma unroll
    for (int k = 0; k < kEsEPT; ++k) {
      const int j = tid + k * kEsNC;
      it[k] = (j < m.nf || j >= back) ? tile[j] : make_uint4(0, 0, 0, 0);
    }
    // this warp's query records (the stage may be refilled once every warp released it)
    uint4 qr[kEsQW];
#pragma unroll
    for (int r = 0; r < kEsQW; ++r) {
      const int qi = warp + r * kEsNWC;
      qr[r] = qi < m.nq ? qls[(size_t)s * kEsQB + qi] : make_uint4(0, 0, 0, 0);
    }
    // int32 windows: the tile as signed (key, delta) pairs for the in-tile scans, so
    // the stage is released before them (int64 windows scan the stage itself)
    if constexpr (sizeof(HT) == 4) {
      if (m.nq > 0) {
#pragma unroll
        for (int k = 0; k < kEsEPT; ++k) {
          const int j = tid + k * kEsNC;
          if (j < m.nf || j >= back) packed[j] = make_uint2(it[k].y, j >= back ? 0u - it[k].z : it[k].z);
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
    }
    if (m.nq > 0) {
      // probes of this warp's queries against the window before the tile; lane shares
      // stay in registers across the barrier
      HT part[kEsQW];
#pragma unroll
      for (int r = 0; r < kEsQW; ++r) {
        part[r] = 0;
        const int qi = warp + r * kEsNWC;
        if (qi < m.nq) {
          const uint4 q = qr[r];
          const uint32_t lo = q.x, hi = q.y;
          const uint32_t a = lo > klo ? lo : klo, z = hi < khi ? hi : khi;
          if (a < z) {
            const uint32_t ra = rank_of(a), rb = rank_of(z);
            if (ra < rb) part[r] = es_probe<HT>(H, T, ps.nch, ra, rb, lane);
          }
        }
      }
      cons_sync();   // probes done: the window may change
      // scans of the tile's events before each query (stage reads only), then answers
#pragma unroll
      for (int r = 0; r < kEsQW; ++r) {
        const int qi = warp + r * kEsNWC;
        if (qi < m.nq) {
          const uint4 q = qr[r];
          const uint32_t lo = q.x, hi = q.y, pe = q.z & 0xffffu, px = q.z >> 16;
          const uint32_t a = lo > klo ? lo : klo, z = hi < khi ? hi : khi;
          // both ends of the carried row, in flight during the scan
          uint64_t carry = 0;
          if (ps.first && ps.crow && lo < hi && lane < 2) carry = (uint64_t)__ldcg(ps.crow + (lane ? hi : lo));
          HT v = part[r];
          if (a < z) {
            if constexpr (sizeof(HT) == 4) {
              v += es_scan_packed(packed, 0, pe, a, z - a, lane) +
                   es_scan_packed(packed, (uint32_t)(kEsTile - (int32_t)px), (uint32_t)kEsTile, a, z - a, lane);
            } else {
              v += es_scan<HT>(tile, 0, pe, a, z - a, lane);
              v -= es_scan<HT>(tile, (uint32_t)(kEsTile - (int32_t)px), (uint32_t)kEsTile, a, z - a, lane);
            }
          }
          uint64_t total;
          if constexpr (sizeof(HT) == 4) {
            total = (uint64_t)(int64_t)(int32_t)__reduce_add_sync(kFull, (uint32_t)v);
          } else {
            uint64_t x = v;
#pragma unroll
            for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(kFull, x, o);
            total = x;
          }
          const uint64_t chi = __shfl_down_sync(kFull, carry, 1);
          if (lane == 0) {
            int64_t* out = p.answers + q.w;
            if (lo >= hi) {
              if (ps.first) *out = 0;
            } else {
              total += chi - carry;
              *out = ps.first ? (int64_t)total : (int64_t)((uint64_t)*out + total);
            }
          }
        }
      }
    }
    if constexpr (sizeof(HT) == 8) {
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);   // this warp no longer reads the stage
    }
    // apply: front slots add, back slots subtract
#pragma unroll
    for (int k = 0; k < kEsEPT; ++k) {
      const int j = tid + k * kEsNC;
      const bool neg = j >= back;
      if (j < m.nf || neg) {
        const uint4 e = it[k];
        if (e.y >= klo && e.y < khi) {
          const uint32_t r = ps.dense ? e.y : es_rank(bits, rl, e.y - klo);
          if (r >= ps.nr) { bad = 1; continue; }
          if constexpr (sizeof(HT) == 4) {
            const int32_t v = (int32_t)e.z, d = neg ? -v : v;
            atomicAdd(reinterpret_cast<int32_t*>(H) + r, d);
            if (ps.nch) atomicAdd(reinterpret_cast<int32_t*>(T) + (r >> 5), d);
          } else {
            const uint64_t v = ((uint64_t)e.w << 32) | e.z, d = neg ? (uint64_t)0 - v : v;
            shared_add_u64(reinterpret_cast<unsigned long long*>(H) + r, d);
            if (ps.nch) shared_add_u64(reinterpret_cast<unsigned long long*>(T) + (r >> 5), d);
          }
        }
      }
    }
    ++cnt;
    if (m.last) return true;
  }
}

// Window setup of a pass: zeroed entries and chunk totals, the slice's bitmap words
// and slice-local ranks.  Consumers only; ends with a consumer barrier.
template <typename HT>
__device__ void es_setup(const EsParams& p, const EsPass& ps, const BlockTab& bt, const Slice& s, int32_t b,
                         unsigned char* sm) {
  constexpr EsSmem L = es_smem();
  HT* H = reinterpret_cast<HT*>(sm + L.H);
  HT* T = reinterpret_cast<HT*>(sm + L.T);
  uint64_t* bits = reinterpret_cast<uint64_t*>(sm + L.bits);
  uint16_t* rl = reinterpret_cast<uint16_t*>(sm + L.rl);
  const int tid = threadIdx.x;
  constexpr uint32_t per = 16 / sizeof(HT);
  const uint32_t n16 = (ps.nr + per - 1) / per;   // whole uint4s (flat probes read up to there)
  uint4* H4 = reinterpret_cast<uint4*>(H);
  for (uint32_t i = tid; i < n16; i += kEsNC) H4[i] = make_uint4(0, 0, 0, 0);
  for (int32_t i = tid; i < ps.nch; i += kEsNC) T[i] = 0;
  if (!ps.dense) {
    const uint64_t* gbits = p.bits + bt.bits_off;
    const uint32_t* grl = p.rlut + bt.bits_off + b;
    const int32_t nwd = s.word_hi - s.word_lo;
    for (int32_t i = tid; i < nwd; i += kEsNC) {
      bits[i] = gbits[s.word_lo + i];
      rl[i] = (uint16_t)(grl[s.word_lo + i] - s.rank_lo);
    }
  }
  cons_sync();
}

__global__ void __launch_bounds__(kEsThreads, 1) k_esweep(EsParams p) {
  extern __shared__ __align__(128) unsigned char sm[];
  constexpr EsSmem L = es_smem();
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + L.bar);
  uint64_t* empty = full + kEsStages;
  EsCtl* ctl = reinterpret_cast<EsCtl*>(sm + L.ctl);
  uint4* ring = reinterpret_cast<uint4*>(sm + L.ring);
  uint4* plan = reinterpret_cast<uint4*>(sm + L.plan);
  EsPlanMeta* pmeta = reinterpret_cast<EsPlanMeta*>(sm + L.pmeta);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool producer = warp >= kEsNWC;   // planner (kEsNWC) and issuer (kEsNWC + 1)
  if (tid == 0) {
    for (int s = 0; s < kEsStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kEsNWC);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    ctl->abort = 0;
  }
  uint32_t cnt = 0;       // tiles this role has produced / consumed (the same sequence)
  uint32_t bad = 0;
  bool aborted = false;
  for (;;) {
    __syncthreads();
    if (tid == 0) ctl->ticket = (*reinterpret_cast<volatile int32_t*>(p.status) || ctl->abort) ? p.B
                                                                                                : atomicAdd(p.ticket, 1);
    __syncthreads();
    const int32_t i = ctl->ticket;
    if (i >= p.B) break;
    const int32_t b = p.order ? p.order[i] : i;
    const BlockTab bt = p.blocks[b];
    if (bt.t0 >= bt.t1) continue;
    const bool w64 = p.bmode[b] == 0;
    const uint32_t C = bt.C;
    EsPass ps;
    ps.t0 = bt.t0; ps.t1 = bt.t1;
    ps.dense = C <= (w64 ? p.cap64 : p.cap32);
    ps.crow = bt.carry_in >= 0 ? p.carry + bt.carry_in : nullptr;
    const Slice* bsl = p.slices + (size_t)b * kMaxSlices;
    const int32_t nsl = ps.dense ? 1 : p.nslices[b];
    // slices without keys change no answer: skipped, except that one pass (the first
    // slice with keys, else slice 0) writes every answer
    int32_t first_si = 0;
    if (!ps.dense) {
      while (first_si < nsl && bsl[first_si].n == 0) ++first_si;
      if (first_si == nsl) first_si = 0;
    }
    for (int32_t si = 0; si < nsl && !aborted; ++si) {
      Slice s;
      if (ps.dense) {
        s.word_lo = 0; s.word_hi = (int32_t)((C + 63) >> 6); s.rank_lo = 0; s.n = C;
      } else {
        s = bsl[si];
        if (s.n == 0 && si != first_si) continue;
      }
      ps.klo = ps.dense ? 0u : (uint32_t)s.word_lo << 6;
      ps.khi = ps.dense ? C : (uint32_t)min((uint64_t)s.word_hi << 6, (uint64_t)C);
      ps.nr = ps.dense ? C : s.n;
      ps.nch = ps.nr > kEsFlat ? (int32_t)((ps.nr + 31) >> 5) : 0;
      ps.first = si == first_si;
      if (warp == kEsNWC) {
        es_plan(p, ps, ring, plan, pmeta, ctl, lane);
      } else if (producer) {
        if (!es_issue(p, sm, plan, pmeta, cnt, lane)) aborted = true;
      } else {
        bool ok;
        if (w64) {
          es_setup<uint64_t>(p, ps, bt, s, b, sm);
          ok = es_consume<uint64_t>(p, ps, sm, cnt, bad);
        } else {
          es_setup<int32_t>(p, ps, bt, s, b, sm);
          ok = es_consume<int32_t>(p, ps, sm, cnt, bad);
        }
        if (!ok) aborted = true;
      }
      __syncthreads();   // the pass is over in both roles (the window is reset next)
      if (ctl->abort) aborted = true;
    }
    if (aborted) break;
  }
  if (bad) es_status(p.status, BW_STATUS_EVENT_KEY_RANGE);
  if (aborted) {
    __syncthreads();
    // copies still in flight land before the CTA exits.  A stage is refilled only
    // after its previous tile was consumed (so that tile's copies had landed): only
    // the producer's last kEsStages tiles can still be in flight, and each stage
    // barrier's phase is that of its last tile.  The producer waits (bounded) for them.
    if (warp == kEsNWC + 1 && lane == 0) {
      for (uint32_t u = cnt > (uint32_t)kEsStages ? cnt - kEsStages : 0u; u < cnt; ++u)
        mbar_wait(&full[u % kEsStages], (u / kEsStages) & 1u);
    }
  }
}

}  // namespace

int esweep_attrs() {
  return (int)cudaFuncSetAttribute(k_esweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)es_smem().bytes);
}

int esweep_launch(const EsParams& p, int grid, cudaStream_t st) {
  k_esweep<<<grid, kEsThreads, es_smem().bytes, st>>>(p);
  return (int)cudaGetLastError();
}

}  // namespace bw
