// bw_pipeline.cu -- GB300 (sm_103a) version-forest replay pipeline.
//
// Stages, all enqueued on one stream with no host round trip (kernels and one
// memset only, so the whole pipeline can be captured in a CUDA graph):
//
//   1. ingest    k_offsets       per-state [begin,end) ranges of the state-grouped
//                                event and query arrays, with input validation
//   2. linearise k_lin_*         Euler tour of every tree (enter(v) applies v's
//                                events, exit(v) removes them: the reference's
//                                preorder apply/undo, batch_engine_v7.hpp:1021-1059,
//                                laid out flat).  The continuation child v+1 is
//                                visited first, so the tour of a run of chained
//                                states is a run of consecutive arcs; list ranking
//                                runs over those runs ("segments") only.
//   3. blocks    k_blocks        equal-work cut of every tree's steps into state
//                                blocks (batch_engine_v7.hpp:707-722 cuts equal
//                                state counts of one chain; here the cut follows
//                                events + queries and never spans two trees)
//   4. prepare   k_prepare<0>    per block: key bitmap + popcount rank table
//                                (the CSR rank-LUT of sparse_engine.hpp:70-102),
//                                smem-sized key slices and the node width;
//                k_prepare<1>    unless the block ends its tree, its net key deltas
//                                as a dense key-prefix row
//   5. carry     k_carry_*       inclusive column scan of each tree's rows: the
//                                key prefix at every block start
//                                (batch_engine_v7.hpp:936-945, on the device)
//   6. sweep     k_sweep         persistent CTAs take blocks from a queue and
//                                replay each from a zero local prefix structure in
//                                shared memory; answer = carry(hi) - carry(lo) +
//                                local(hi) - local(lo) (batch_engine_v7.hpp:849-961)
//
// All arithmetic is int64 with two's-complement wrap (done in uint64), so any
// summation order gives the reference's bits.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <numeric>
#include <vector>

#include "bw_gpu.h"
#include "bw_common.cuh"
#include "bw_pipeline.cuh"

namespace bw {

int report(cudaError_t e, const char* what) {
  if (e != cudaSuccess) std::fprintf(stderr, "bw_replay: %s failed: %s\n", what, cudaGetErrorString(e));
  return (int)e;
}

__device__ __forceinline__ void set_status(int32_t* st, int32_t code) { atomicCAS(st, 0, code); }

// Largest t in [0, T) with off[t] <= x (off ascending; empty trees are skipped).
template <typename Off>
__device__ __forceinline__ int32_t find_tree(const Off* off, int32_t T, int64_t x) {
  int32_t lo = 0, hi = T - 1;
  while (lo < hi) {
    const int32_t mid = (lo + hi + 1) >> 1;
    if ((int64_t)off[mid] <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__host__ __device__ __forceinline__ int32_t words_of(uint32_t C) { return (int32_t)(((uint64_t)C + 63) >> 6); }

// ------------------------------------------------------------------ 0. init
// Status and queue tickets, per-tree last query steps, and for a single tree its
// table row (from scalars, so no host-to-device copy is needed per launch).
__global__ void k_init(int32_t* misc, TreeTabs tt, int32_t T, int one_tree, int32_t S, int64_t E, int64_t Q,
                       uint32_t C, int32_t nb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 64) misc[i] = 0;
  for (int t = i; t < T; t += gridDim.x * blockDim.x) tt.last_q[t] = 0;
  if (one_tree && i == 0) {
    tt.soff[0] = 0; tt.soff[1] = S;
    tt.eoff[0] = 0; tt.eoff[1] = E;
    tt.qoff[0] = 0; tt.qoff[1] = Q;
    tt.C[0] = C;
    tt.boff[0] = 0; tt.boff[1] = nb;
    tt.bits[0] = 0; tt.carry[0] = 0; tt.gsum[0] = 0;
  }
}

__global__ void k_fill_i64(int64_t* p, int64_t n, int64_t v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

// ------------------------------------------------------------------ 1. ingest
// Per-global-state [off[s], off[s+1]) ranges of a state-grouped array of records
// whose first field is the tree-local u32 state.  Item i belongs to the tree whose
// item range holds i; its global state is the tree's first state + the local one.
// Checks grouping within each tree and key / interval ranges against the tree's
// domain.
// Contiguous item range of this warp (whole multiples of 32), so lanes take
// consecutive items and each lane's tree only moves forward: one tree search per
// lane and range instead of one per item.
__device__ __forceinline__ void warp_range(int64_t n, int64_t& lo, int64_t& hi) {
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int64_t per = (((n + warps - 1) / warps) + 31) & ~(int64_t)31;
  lo = imin64(n, w * per);
  hi = imin64(n, lo + per);
}
template <typename Off>
__device__ __forceinline__ int32_t tree_forward(const Off* off, int32_t T, int32_t t, int64_t x) {
  while (t + 1 < T && (int64_t)off[t + 1] <= x) ++t;
  return t;
}

template <bool kEvents>
__global__ void k_offsets(const void* items, int64_t n, TreeTabs tt, int32_t T, int32_t S, int64_t* off,
                          int32_t* status) {
  const int64_t* toff = kEvents ? tt.eoff : tt.qoff;
  const BwEvent* ev = static_cast<const BwEvent*>(items);
  const BwQuery* qs = static_cast<const BwQuery*>(items);
  const int lane = threadIdx.x & 31;
  int64_t lo, hi;
  warp_range(n, lo, hi);
  if (lo >= hi) return;
  // global state of a tree-local state s of tree t (-2: out of its tree, reported by its own lane)
  auto gstate_of = [&](int32_t t, uint32_t s) -> int64_t {
    const int32_t s0 = tt.soff[t], ns = tt.soff[t + 1] - s0;
    return s < (uint32_t)ns ? (int64_t)s0 + s : -2;
  };
  auto gstate = [&](int32_t t, int64_t i) -> int64_t { return gstate_of(t, kEvents ? ev[i].state : qs[i].state); };
  // an item's (state, key) or (state, lo, hi), loaded one iteration ahead so a
  // warp keeps two record loads in flight
  struct Rec { uint32_t s, a, b; };
  auto load = [&](int64_t i) -> Rec {
    Rec r;
    if (kEvents) {
      const uint2 v = __ldg(reinterpret_cast<const uint2*>(ev + i));   // state, key
      r.s = v.x; r.a = v.y; r.b = 0;
    } else {
      r.s = qs[i].state; r.a = qs[i].lo; r.b = qs[i].hi;
    }
    return r;
  };
  int64_t gcarry = -1;   // global state of the item before this lane 0's item
  if (lo > 0) {
    int64_t gp = 0;
    if (lane == 0) gp = gstate(T > 1 ? find_tree(toff, T, lo - 1) : 0, lo - 1);
    gcarry = __shfl_sync(0xffffffffu, gp, 0);
  }
  int32_t t = T > 1 ? find_tree(toff, T, imin64(lo + lane, n - 1)) : 0;
  Rec nx = lo + lane < hi ? load(lo + lane) : Rec{0, 0, 0};
  for (int64_t i0 = lo; i0 < hi; i0 += 32) {
    const int64_t i = i0 + lane;
    const bool valid = i < hi;
    const Rec rc = nx;
    if (i + 32 < hi) nx = load(i + 32);
    int64_t g = -2;
    if (valid) {
      if (T > 1) t = tree_forward(toff, T, t, i);
      const uint32_t C = tt.C[t];
      if (kEvents) {
        if (rc.a >= C) set_status(status, BW_STATUS_EVENT_KEY_RANGE);
      } else {
        if (rc.a > C || rc.b > C) set_status(status, BW_STATUS_QUERY_RANGE);
      }
      g = gstate_of(t, rc.s);
      if (g == -2) set_status(status, BW_STATUS_STATE_RANGE);
    }
    int64_t gprev = __shfl_up_sync(0xffffffffu, g, 1);
    if (lane == 0) gprev = gcarry;
    gcarry = __shfl_sync(0xffffffffu, g, 31);
    if (!valid || g == -2 || gprev == -2) continue;
    if (gprev > g) {   // an earlier tree's states are below every state of this tree
      set_status(status, kEvents ? BW_STATUS_EVENTS_UNSORTED : BW_STATUS_QUERIES_UNSORTED);
      continue;
    }
    // off[x] = i for every global state x in (gprev, g]
    for (int64_t x = gprev + 1; x <= g; ++x) off[x] = i;
    if (i == n - 1)
      for (int64_t x = g + 1; x <= S; ++x) off[x] = n;
  }
}

// ------------------------------------------------------------------ 2. linearise
// Global parents and fork lists.  The continuation child v+1 of v (parent v+1 = v)
// is always visited first and is not listed; every other child c of p ("fork") is
// pushed on p's list by atomic exchange.  Child order does not change any answer
// (a state's answer only depends on its root path), only the step order.
__global__ void k_lin_children(const int32_t* parent, int32_t S, TreeTabs tt, int32_t T, int32_t* gpar,
                               int32_t* fork_head, int32_t* next_sib, int chain_only, int32_t* status) {
  int64_t lo, hi;
  warp_range(S, lo, hi);
  int32_t t = T > 1 && lo < hi ? find_tree(tt.soff, T, imin64(lo + (threadIdx.x & 31), S - 1)) : 0;
  for (int32_t v = (int32_t)lo + (threadIdx.x & 31); v < hi; v += 32) {
    if (T > 1) t = tree_forward(tt.soff, T, t, v);
    const int32_t s0 = tt.soff[t], l = v - s0;
    const int32_t p = parent[v];
    int32_t gp = -1;
    if (l == 0) {
      if (p != -1) set_status(status, BW_STATUS_BAD_PARENT);
    } else if (p < 0 || p >= l) {
      set_status(status, BW_STATUS_BAD_PARENT);
    } else {
      gp = s0 + p;
    }
    if (gpar) gpar[v] = gp;
    if (l > 0 && gp >= 0 && gp != v - 1) {
      if (chain_only) set_status(status, BW_STATUS_BAD_PARENT);
      next_sib[v] = atomicExch(&fork_head[gp], v);
    } else {
      next_sib[v] = -1;
    }
  }
}

// Segment heads.  enter(v) follows enter(v-1) exactly when v continues v-1; exit(v)
// follows exit(v+1) exactly when v+1 continues v and v has no forks.  An arc that
// follows another way heads a segment: a maximal run of consecutive arcs (enter
// segments go up the state ids, exit segments down).  cnt[v] packs the two head
// flags (enter | exit << 32) for an inclusive scan.
__global__ void k_lin_flags(const int32_t* gpar, const int32_t* fork_head, int32_t S, int64_t* cnt,
                            const int32_t* status) {
  if (*status) return;
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < S; v += gridDim.x * blockDim.x) {
    const bool cont = v + 1 < S && gpar[v + 1] == v;
    const bool eh = !(v > 0 && gpar[v] == v - 1);
    const bool xh = !(cont && fork_head[v] < 0);
    cnt[v] = (int64_t)(eh ? 1 : 0) | ((int64_t)(xh ? 1 : 0) << 32);
  }
}

__global__ void k_lin_heads(const int64_t* cnt, int32_t S, int32_t* ehead, int32_t* xhead, const int32_t* status) {
  if (*status) return;
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < S; v += gridDim.x * blockDim.x) {
    const uint64_t c = (uint64_t)cnt[v], cp = v ? (uint64_t)cnt[v - 1] : 0ull;
    const uint32_t e = (uint32_t)c, x = (uint32_t)(c >> 32);
    if (e != (uint32_t)cp) ehead[e - 1] = v;
    if (x != (uint32_t)(cp >> 32)) xhead[x - 1] = v;
  }
}

__device__ __forceinline__ uint64_t pack_rank(int32_t next, uint32_t dist) {
  return ((uint64_t)(uint32_t)next << 32) | dist;
}

// Segment list: enter segments 0..He-1 (run [ehead[i], ehead[i+1]) of chained
// states), exit segments He..He+Hx-1 (exits of states (xhead[j-1], xhead[j]],
// taken downwards).  Each segment's successor is the segment headed by the arc that
// follows its tail arc in the Euler tour; every tree's list ends at the exit of its
// root.  r = (successor, length) for weighted list ranking.
__global__ void k_lin_rank_init(const int64_t* cnt, const int32_t* ehead, const int32_t* xhead, const int32_t* gpar,
                                const int32_t* fork_head, const int32_t* next_sib, int32_t S, uint64_t* r,
                                const int32_t* status) {
  if (*status) return;
  const uint64_t tot = (uint64_t)cnt[S - 1];
  const int64_t He = (uint32_t)tot, H = He + (int64_t)(tot >> 32);
  auto eid = [&](int32_t w) { return (int32_t)((uint32_t)cnt[w]) - 1; };
  auto xid = [&](int32_t w) { return (int32_t)(He + (int64_t)((uint64_t)cnt[w] >> 32) - 1); };
  for (int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; id < H; id += (int64_t)gridDim.x * blockDim.x) {
    int32_t succ, len;
    if (id < He) {
      const int32_t h = ehead[id];
      const int32_t tl = (id + 1 < He ? ehead[id + 1] : S) - 1;
      len = tl - h + 1;
      const int32_t f = fork_head[tl];
      succ = f >= 0 ? eid(f) : xid(tl);
    } else {
      const int64_t x = id - He;
      const int32_t u = xhead[x];
      const int32_t lo = x > 0 ? xhead[x - 1] + 1 : 0;
      len = u - lo + 1;
      const int32_t p = gpar[lo];
      if (p < 0) {
        succ = -1;                                  // exit of a tree root: end of its tour
      } else if (p == lo - 1) {
        const int32_t f = fork_head[p];             // lo continues p: p's forks come next
        succ = f >= 0 ? eid(f) : xid(p);
      } else {
        const int32_t ns = next_sib[lo];            // lo is a fork: its next sibling
        succ = ns >= 0 ? eid(ns) : xid(p);
      }
    }
    r[id] = pack_rank(succ, (uint32_t)len);
  }
}

// One Wyllie pointer-jumping round, in place: dist(x) += dist(next(x)),
// next(x) = next(next(x)).  A (next, dist) pair is one 64-bit word, so a read sees a
// consistent pair even while its owner updates it (jumping further ahead keeps
// dist(x) = the lengths from x up to next(x)).  Round r records whether any pointer
// is still live; a round after one that found none returns at once.
__global__ void k_lin_round(uint64_t* __restrict__ r, const int64_t* cnt, int32_t S, int32_t* live, int32_t round,
                            const int32_t* status) {
  if (*status) return;
  if (round > 0 && live[round - 1] == 0) return;
  const uint64_t tot = (uint64_t)cnt[S - 1];
  const int64_t H = (int64_t)(uint32_t)tot + (int64_t)(tot >> 32);
  bool any = false;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < H; x += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t a = r[x];
    const int32_t nx = (int32_t)(a >> 32);
    if (nx < 0) continue;
    const uint64_t b = r[nx];
    r[x] = (b & 0xFFFFFFFF00000000ull) | (uint32_t)((uint32_t)a + (uint32_t)b);
    any |= (int32_t)(b >> 32) >= 0;
  }
  if (__syncthreads_or(any) && threadIdx.x == 0) live[round] = 1;
}

// Step sequence (each step's enter/exit partner), per-step descriptors and work, and each tree's last
// step that answers a query.  Tree t's tour occupies steps [2 s0, 2 s0 + 2 ns): the
// head arc of a segment sits at 2 s0 + 2 ns - dist, the other arcs follow it.
__global__ void k_lin_steps(const uint64_t* r, const int64_t* cnt, const int32_t* ehead, const int32_t* xhead,
                            int32_t S, TreeTabs tt, int32_t T, const int64_t* eoff, const int64_t* qoff,
                            int32_t* partner, StepDesc* desc, int64_t* work, const int32_t* status) {
  if (*status) return;
  const int64_t He = (uint32_t)(uint64_t)cnt[S - 1];
  int64_t lo, hi;
  warp_range(S, lo, hi);
  int32_t t = T > 1 && lo < hi ? find_tree(tt.soff, T, imin64(lo + (threadIdx.x & 31), S - 1)) : 0;
  // the state's counters and ranges, loaded one iteration ahead
  struct Pre { uint64_t c, cp; int64_t e0, e1, q0, q1; };
  auto load = [&](int32_t v) -> Pre {
    Pre x;
    x.c = (uint64_t)cnt[v]; x.cp = v ? (uint64_t)cnt[v - 1] : 0ull;
    x.e0 = eoff[v]; x.e1 = eoff[v + 1]; x.q0 = qoff[v]; x.q1 = qoff[v + 1];
    return x;
  };
  Pre nx{0, 0, 0, 0, 0, 0};
  if (lo + (threadIdx.x & 31) < hi) nx = load((int32_t)lo + (threadIdx.x & 31));
  for (int32_t v = (int32_t)lo + (threadIdx.x & 31); v < hi; v += 32) {
    const Pre pr = nx;
    if (v + 32 < hi) nx = load(v + 32);
    if (T > 1) t = tree_forward(tt.soff, T, t, v);
    const int32_t s0 = tt.soff[t], ns = tt.soff[t + 1] - s0;
    const int64_t base = 2 * (int64_t)s0 + 2 * (int64_t)ns;
    const uint64_t c = pr.c, cp = pr.cp;
    const int64_t eid = (int64_t)(uint32_t)c - 1;
    const int64_t xh = (int64_t)(c >> 32) - (int64_t)(cp >> 32);
    const int64_t xid = (int64_t)(c >> 32) - xh;       // exit heads below v
    const int64_t pe = base - (int64_t)(uint32_t)r[eid] + (v - ehead[eid]);
    const int64_t px = base - (int64_t)(uint32_t)r[He + xid] + (xhead[xid] - v);
    const int64_t e0 = pr.e0, q0 = pr.q0;
    const int32_t ne = (int32_t)(pr.e1 - e0), nq = (int32_t)(pr.q1 - q0);
    partner[pe] = (int32_t)px;
    partner[px] = (int32_t)pe;
    StepDesc d;
    d.e0 = (uint32_t)e0; d.q0 = (uint32_t)q0; d.ne = ne; d.nq = nq;
    desc[pe] = d;
    d.q0 = 0; d.nq = -1;
    desc[px] = d;
    work[pe] = kStepCost + ne + (nq > 0 ? kQueryStepCost + kQueryCost * nq : 0);
    work[px] = kStepCost + ne;
    if (nq > 0) atomicMax(&tt.last_q[t], (int32_t)pe + 1);
  }
}

// ------------------------------------------------------------------ 3. blocks
// Block b of tree t (index i of nb) covers the steps of the tree's trimmed range
// [a, z) (z = one past its last query step: later steps cannot change an answer)
// whose inclusive work prefix lies in (i W / nb, (i + 1) W / nb].
__global__ void k_blocks(const int64_t* work, TreeTabs tt, int32_t T, int32_t B, BlockTab* bt, const int32_t* status) {
  const int32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int32_t t = T > 1 ? find_tree(tt.boff, T, b) : 0;
  const int32_t idx = b - tt.boff[t], nb = tt.boff[t + 1] - tt.boff[t];
  const uint32_t C = tt.C[t];
  const int32_t nw = words_of(C);
  BlockTab x;
  x.tree = t; x.idx = idx; x.C = C; x.nwords = nw;
  x.bits_off = tt.bits[t] + (int64_t)idx * nw;
  x.carry_in = idx >= 1 ? tt.carry[t] + (int64_t)(idx - 1) * ((int64_t)C + 1) : -1;
  x.carry_out = idx < nb - 1 ? tt.carry[t] + (int64_t)idx * ((int64_t)C + 1) : -1;
  x.t0 = x.t1 = 0;
  if (!*status) {
    const int64_t s0 = tt.soff[t], ns = tt.soff[t + 1] - s0;
    const int64_t a = 2 * s0, zf = a + 2 * ns;
    const int32_t lq = tt.last_q[t];
    const int64_t z = lq > 0 ? (lq < zf ? lq : zf) : a;
    const int64_t base = a > 0 ? work[a - 1] : 0;
    const int64_t W = z > a ? work[z - 1] - base : 0;
    auto cut = [&](int32_t i) -> int64_t {
      if (i <= 0) return a;
      if (i >= nb) return z;
      const int64_t lim = base + (int64_t)(((__int128)W * i) / nb);
      int64_t lo = a, hi = z;  // first step with work > lim
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (work[mid] <= lim) lo = mid + 1; else hi = mid;
      }
      return lo;
    };
    x.t0 = (int32_t)cut(idx);
    x.t1 = (int32_t)cut(idx + 1);
  }
  bt[b] = x;
}

// ------------------------------------------------------------------ 4. prepare
struct PrepParams {
  const BwEvent* ev;
  const StepDesc* desc;
  const int32_t* partner;  // per step: the step of the same node's enter/exit
  const BlockTab* blocks;
  const int32_t* order;    // queue order of the blocks (NULL: identity)
  int32_t B;
  int32_t ww;              // rank-table window in bitmap words (<= kWinWords)
  uint32_t cap32, cap64;   // slice rank capacity with int32 / int64 sweep nodes
  uint64_t* bits;
  uint32_t* rlut;
  Slice* slices;
  int32_t* nslices;
  int64_t* carry;
  int32_t* status;
  int32_t* bmode;
  int32_t* ticket;
};

// Visit the (key, signed delta) of the block's steps that matter: mode 0 (key
// set) skips exits of nodes entered in the block (their keys come with the
// enter, flagged by `twice` since the sweep applies them twice); mode 1 (net
// deltas) also skips enters of nodes that exit in the block, since the two cancel.
// Each warp takes 32 consecutive steps at a time (lane l decodes step l), flattens
// their kept events with a warp scan, and lanes take consecutive flattened events,
// so steps with few events still fill the warp.  Loop bounds are warp-uniform and f
// is called by all 32 lanes (valid marks real events), so f may use warp-collective
// operations.
template <typename F>
__device__ __forceinline__ void for_block_events(const PrepParams& p, int32_t t0, int32_t t1, int mode, F&& f) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  // this lane's step of the next group, loaded one group ahead
  StepDesc nd;
  int32_t npt = 0;
  nd.e0 = 0; nd.q0 = 0; nd.ne = 0; nd.nq = 0;
  if (t0 + 32 * warp + lane < t1) {
    nd = p.desc[t0 + 32 * warp + lane];
    npt = p.partner[t0 + 32 * warp + lane];
  }
  for (int32_t c = t0 + 32 * warp; c < t1; c += 32 * nw) {
    const int32_t t = c + lane;
    const StepDesc d = nd;
    const int32_t pt = npt;   // the node's other step (exit of an enter, enter of an exit)
    if (t + 32 * nw < t1) {
      nd = p.desc[t + 32 * nw];
      npt = p.partner[t + 32 * nw];
    }
    int32_t cnt = 0;
    uint32_t e0 = 0;
    bool neg = false, twice = false;
    if (t < t1) {
      neg = d.nq < 0;
      twice = !neg && pt < t1;
      bool keep = true;
      if (neg) keep = pt < t0;                   // entered in this block: keys known, deltas cancel
      else if (mode == 1 && twice) keep = false; // leaves within this block: net zero
      if (keep) { cnt = d.ne; e0 = d.e0; }
    }
    int32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const int32_t total = __shfl_sync(0xffffffffu, incl, 31);
    for (int32_t g0 = 0; g0 < total; g0 += 32) {
      const int32_t g = g0 + lane;
      int32_t lo = 0, hi = 31;   // first lane whose inclusive count exceeds g
#pragma unroll
      for (int it = 0; it < 5; ++it) {
        const int32_t mid = (lo + hi) >> 1;
        const int32_t v = __shfl_sync(0xffffffffu, incl, mid);
        if (v > g) hi = mid; else lo = mid + 1;
      }
      const int32_t src = lo;
      const int32_t s_incl = __shfl_sync(0xffffffffu, incl, src);
      const int32_t s_cnt = __shfl_sync(0xffffffffu, cnt, src);
      const uint32_t s_e0 = __shfl_sync(0xffffffffu, e0, src);
      const bool s_neg = __shfl_sync(0xffffffffu, neg ? 1 : 0, src) != 0;
      const bool s_twice = __shfl_sync(0xffffffffu, twice ? 1 : 0, src) != 0;
      const bool valid = g < total;
      uint32_t k = 0;
      uint64_t v = 0;
      if (valid) {
        const BwEvent e = p.ev[(int64_t)s_e0 + (g - (s_incl - s_cnt))];
        k = e.key;
        v = s_neg ? (uint64_t)0 - (uint64_t)e.delta : (uint64_t)e.delta;
      }
      f(k, v, valid, s_twice);
    }
  }
}

// Pass A of block b: per window of the key domain, the bitmap of the keys the
// block's events touch, its popcount rank table, the greedy slices the sweep's
// rank capacity allows, and the block's node mode (int32 when the applied |delta|
// sum stays below 2^31).
__device__ void prepare_block_a(const PrepParams& p, int32_t b, unsigned char* smem) {
  const BlockTab bt = p.blocks[b];
  const int32_t nwords = bt.nwords;
  const uint32_t C = bt.C;
  uint64_t* sbits = reinterpret_cast<uint64_t*>(smem);                    // ww words
  uint32_t* srl = reinterpret_cast<uint32_t*>(sbits + p.ww);              // ww + 2
  __shared__ int32_t s_nsl;
  __shared__ int32_t s_mode;

  const int32_t t0 = bt.t0, t1 = bt.t1;
  uint64_t* gbits = p.bits + bt.bits_off;
  uint32_t* grl = p.rlut + bt.bits_off + b;
  Slice* gsl = p.slices + (size_t)b * kMaxSlices;
  if (threadIdx.x == 0) s_nsl = 0;
  uint32_t rank_base = 0;
  uint64_t mass = 0;  // per-thread partial of the block's applied |delta| sum

  // ---- pass A: per window, key bitmap -> rank table -> slices
  for (int32_t w0 = 0; w0 < nwords; w0 += p.ww) {
    const int32_t ww = min(p.ww, nwords - w0);
    for (int i = threadIdx.x; i < ww; i += blockDim.x) sbits[i] = 0;
    __syncthreads();
    const uint32_t klo = (uint32_t)w0 << 6;
    const uint32_t khi = (uint32_t)imin64((int64_t)(w0 + ww) << 6, (int64_t)C);
    for_block_events(p, t0, t1, 0, [&](uint32_t k, uint64_t v, bool valid, bool twice) {
      if (valid && k >= klo && k < khi) shared_set_bit(sbits, k - klo);
      if (valid && w0 == 0) {
        // |delta| summed over every application the sweep makes (saturating)
        const uint64_t a = (v >> 63) ? (uint64_t)0 - v : v;
        const uint64_t m = (a > (1ull << 33) ? (1ull << 33) : a) << (twice ? 1 : 0);
        mass = mass + m > (1ull << 40) ? (1ull << 40) : mass + m;   // 512 partials stay < 2^49
      }
    });
    if (w0 == 0) {
      uint64_t tot = 0;
      block_exclusive_scan<uint64_t>(mass, &tot);   // block total
      if (threadIdx.x == 0) s_mode = tot < (1ull << 31) ? 1 : 0;
    }
    __syncthreads();
    const uint32_t cap = s_mode ? p.cap32 : p.cap64;
    const uint32_t wtot = block_exclusive_scan_popc(sbits, srl, ww);   // srl[0..ww]
    for (int i = threadIdx.x; i < ww; i += blockDim.x) {
      gbits[w0 + i] = sbits[i];
      grl[w0 + i] = rank_base + srl[i];
    }
    if (threadIdx.x == 0) {
      // greedy slices over the window's words: close a slice before it exceeds cap
      // (its end: the last word boundary whose rank stays within cap of the slice
      // start, by binary search over the nondecreasing rank table; at least one word)
      int32_t ns = s_nsl;
      int32_t lo = 0;
      while (lo < ww) {
        int32_t hi = lo + 1, top = ww;
        while (hi < top) {
          const int32_t mid = (hi + top + 1) >> 1;
          if (srl[mid] - srl[lo] <= cap) hi = mid; else top = mid - 1;
        }
        if (ns < kMaxSlices) {
          Slice s;
          s.word_lo = w0 + lo; s.word_hi = w0 + hi;
          s.rank_lo = rank_base + srl[lo]; s.n = srl[hi] - srl[lo];
          gsl[ns] = s;
        }
        ++ns;
        lo = hi;
      }
      s_nsl = ns;
    }
    rank_base += wtot;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    grl[nwords] = rank_base;
    if (s_nsl > kMaxSlices) set_status(p.status, BW_STATUS_TOO_MANY_SLICES);
    p.nslices[b] = min(s_nsl, kMaxSlices);
    p.bmode[b] = s_mode;
  }
  __syncthreads();
}

// Pass B of block b (only blocks that hand a carry on, i.e. all but the last
// block of each tree): per slice of pass A, the block's net key deltas gathered
// in a shared histogram over the slice's ranks, written out as the dense
// key-prefix row carry[carry_out .. carry_out + C].
__device__ void prepare_block_b(const PrepParams& p, int32_t b, unsigned char* smem) {
  const BlockTab bt = p.blocks[b];
  const uint32_t C = bt.C;
  uint64_t* sbits = reinterpret_cast<uint64_t*>(smem);                    // ww words
  uint32_t* srl = reinterpret_cast<uint32_t*>(sbits + p.ww);              // ww + 2
  // histogram: int32 per rank when the block's nodes are int32 (exact, same
  // bound), int64 otherwise; both fit the same bytes (cap32 ~ 2 * cap64)
  unsigned char* hist_raw = reinterpret_cast<unsigned char*>(srl + p.ww + 2 + (p.ww & 1));  // 8-byte aligned
  __shared__ uint64_t s_wsum[kPrepThreads / 32];
  const int32_t t0 = bt.t0, t1 = bt.t1;
  const uint64_t* gbits = p.bits + bt.bits_off;
  const uint32_t* grl = p.rlut + bt.bits_off + b;
  const Slice* gsl = p.slices + (size_t)b * kMaxSlices;
  const int32_t nsl = p.nslices[b];
  int64_t* row = p.carry + bt.carry_out;
  const bool h32 = p.bmode[b] != 0;
  unsigned* hist32 = reinterpret_cast<unsigned*>(hist_raw);
  unsigned long long* hist64 = reinterpret_cast<unsigned long long*>(hist_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  uint64_t base = 0;  // key prefix at the start of the slice (same in every thread)
  for (int32_t si = 0; si < nsl; ++si) {
    const Slice s = gsl[si];
    const int32_t nwd = s.word_hi - s.word_lo;
    for (int i = threadIdx.x; i < nwd; i += blockDim.x) {
      sbits[i] = gbits[s.word_lo + i];
      srl[i] = grl[s.word_lo + i] - s.rank_lo;
    }
    for (uint32_t i = threadIdx.x; i <= s.n; i += blockDim.x) {
      if (h32) hist32[i] = 0; else hist64[i] = 0;
    }
    __syncthreads();
    const uint32_t klo = (uint32_t)s.word_lo << 6;
    const uint32_t khi = (uint32_t)imin64((int64_t)s.word_hi << 6, (int64_t)C);
    if (s.n) {
      for_block_events(p, t0, t1, 1, [&](uint32_t k, uint64_t d, bool valid, bool) {
        if (valid && k >= klo && k < khi) {
          const uint32_t r = local_rank(sbits, srl, k - klo);
          if (h32) atomicAdd(hist32 + r, (unsigned)d);
          else shared_add_u64(hist64 + r, d);
        }
      });
    }
    __syncthreads();
    auto hval = [&](uint32_t r) -> uint64_t {
      return h32 ? (uint64_t)(int64_t)(int32_t)hist32[r] : (uint64_t)hist64[r];
    };
    // each warp writes a contiguous key range; its start value is the sum of the
    // histogram over the ranks before the range (block scan of warp sums)
    const uint32_t nk = khi - klo;
    const uint32_t span = ((nk + nw - 1) / nw + 31) & ~31u;
    const uint32_t ka = klo + imin64((int64_t)warp * span, nk), kb = klo + imin64((int64_t)(warp + 1) * span, nk);
    const uint32_t ra = ka < khi ? local_rank(sbits, srl, ka - klo) : s.n;
    const uint32_t rb = kb < khi ? local_rank(sbits, srl, kb - klo) : s.n;
    uint64_t part = 0;
    for (uint32_t r = ra + lane; r < rb; r += 32) part += hval(r);
#pragma unroll
    for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0) s_wsum[warp] = part;
    __syncthreads();
    uint64_t start = base, total = 0;
    for (int w = 0; w < nw; ++w) {
      const uint64_t x = s_wsum[w];
      if (w < warp) start += x;
      total += x;
    }
    for (uint32_t k0 = ka; k0 < kb; k0 += 32) {
      const uint32_t k = k0 + lane;
      uint64_t val = 0;
      if (k < kb) {
        const uint32_t x = k - klo;
        if ((sbits[x >> 6] >> (x & 63)) & 1ull) val = hval(local_rank(sbits, srl, x));
      }
      uint64_t incl = val;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      if (k < kb) row[k] = (int64_t)(start + incl - val);
      start += __shfl_sync(0xffffffffu, incl, 31);
    }
    base += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) row[C] = (int64_t)base;
}

// Persistent: CTAs take blocks from the queue until it is empty.  Pass A needs
// only the bitmap window (several CTAs per SM); pass B also holds the slice
// histogram, so it runs as its own kernel over the blocks that hand a carry on.
template <int Pass>
__global__ void __launch_bounds__(kPrepThreads, Pass == 0 ? 3 : 2) k_prepare(PrepParams p) {
  if (*p.status) return;  // bounds/descriptors are not trustworthy after an input error
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int32_t s_ticket;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_ticket = atomicAdd(p.ticket, 1);
    __syncthreads();
    const int32_t i = s_ticket;
    if (i >= p.B) break;
    const int32_t b = p.order ? p.order[i] : i;
    if (Pass == 0) prepare_block_a(p, b, smem);
    else if (p.blocks[b].carry_out >= 0) prepare_block_b(p, b, smem);
  }
}

// ------------------------------------------------------------------ 5. carry
// Tree t with nb blocks has nb - 1 rows (the net key-prefix rows of its blocks
// 0..nb-2); in place they become inclusive prefix sums, so row i is the key prefix
// of the state vector at the start of block i + 1.  Rows are processed in groups
// of kCarryGroup with every (group, column) pair its own thread: group sums, then
// each group adds the sums of the groups before it and scans its rows.
struct CarryParams {
  int64_t* carry;
  int64_t* gsum;
  const CarryUnit* units;  // NULL: one tree, unit u = (0, u / chunks1, u % chunks1)
  int32_t chunks1;
  TreeTabs tt;
  const int32_t* status;
};

__device__ __forceinline__ CarryUnit carry_unit(const CarryParams& p, int32_t u) {
  if (p.units) return p.units[u];
  CarryUnit c;
  c.tree = 0; c.group = u / p.chunks1; c.chunk = u % p.chunks1; c.pad = 0;
  return c;
}

__global__ void k_carry_groups(CarryParams p) {
  if (*p.status) return;
  const CarryUnit cu = carry_unit(p, blockIdx.x);
  const int32_t t = cu.tree;
  const int64_t width = (int64_t)p.tt.C[t] + 1;
  const int64_t k = (int64_t)cu.chunk * kCarryChunk + threadIdx.x;
  const int32_t rows = p.tt.boff[t + 1] - p.tt.boff[t] - 1;
  // a tree with one row group has no group sums (and no space reserved for them)
  if (k >= width || rows <= kCarryGroup) return;
  const int32_t r0 = cu.group * kCarryGroup, n = min(kCarryGroup, rows - r0);
  const int64_t* src = p.carry + p.tt.carry[t] + (int64_t)r0 * width + k;
  uint64_t v[kCarryGroup];
#pragma unroll
  for (int i = 0; i < kCarryGroup; ++i) v[i] = i < n ? (uint64_t)src[(size_t)i * width] : 0;
  uint64_t sum = 0;
#pragma unroll
  for (int i = 0; i < kCarryGroup; ++i) sum += v[i];
  p.gsum[p.tt.gsum[t] + (int64_t)cu.group * width + k] = (int64_t)sum;
}

__global__ void k_carry_apply(CarryParams p) {
  if (*p.status) return;
  const CarryUnit cu = carry_unit(p, blockIdx.x);
  const int32_t t = cu.tree;
  const int64_t width = (int64_t)p.tt.C[t] + 1;
  const int64_t k = (int64_t)cu.chunk * kCarryChunk + threadIdx.x;
  if (k >= width) return;
  const int32_t rows = p.tt.boff[t + 1] - p.tt.boff[t] - 1;
  const int32_t r0 = cu.group * kCarryGroup, n = min(kCarryGroup, rows - r0);
  int64_t* dst = p.carry + p.tt.carry[t] + (int64_t)r0 * width + k;
  uint64_t v[kCarryGroup];
#pragma unroll
  for (int i = 0; i < kCarryGroup; ++i) v[i] = i < n ? (uint64_t)dst[(size_t)i * width] : 0;
  uint64_t run = 0;
  for (int32_t g = 0; g < cu.group; ++g) run += (uint64_t)p.gsum[p.tt.gsum[t] + (int64_t)g * width + k];
#pragma unroll
  for (int i = 0; i < kCarryGroup; ++i) {
    run += v[i];
    if (i < n) dst[(size_t)i * width] = (int64_t)run;
  }
}

// ------------------------------------------------------------------ 6. sweep
struct SweepParams {
  const BwEvent* ev;
  const BwQuery* qs;
  const StepDesc* desc;
  const BlockTab* blocks;
  const int32_t* order;   // queue order (NULL: identity)
  int32_t B;
  const uint64_t* bits;
  const uint32_t* rlut;
  const Slice* slices;
  const int32_t* nslices;
  const int64_t* carry;
  int64_t* answers;
  const int32_t* status;
  const int32_t* bmode;   // per block: 1 = int32 Fenwick nodes are exact, 0 = int64
  int32_t* ticket;
};

// The sweep keeps the block-local prefix structure in shared memory as chunks of
// kChunk ranks with chunk totals T[h], in one of two forms.  Fenwick chunks (a tree
// inside every chunk, per-warp copies of the exclusive prefix of the totals rebuilt
// before a probe phase): an update touches <= kChunkLevels nodes of its chunk, a probe
// is one thread.  Flat chunks (each rank's own value, totals in up to 8 side-by-side
// copies): an update is two atomics, a probe is one warp summing the partial chunks at
// both ends of its range and the totals between them.
//
// Steps are replayed in tiles of up to Cfg::kTileSteps consecutive steps whose events
// and queries, flattened in step order, fit the tile's staging slots.  Own-slot tiles:
// thread i stages, with cp.async, flattened events i + kThreads m and its query slots
// of the next tile while it replays the current one and waits only for its own copies.
// Cooperative tiles: warps copy 32-step groups and a barrier publishes the tile.
// Specialised tiles: one warp cuts and stages tiles two ahead for the others.  A tile
// within the single-probe limits is replayed offline (one barrier, every query probed
// on the state at the tile start plus its correction over the tile's earlier events,
// a barrier, the tile's updates); otherwise per query step (its updates, a barrier,
// its probes, a barrier).  Step descriptors and their event/query prefix sums come
// from a shared ring refilled Cfg::kRingFill steps at a time.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }
// Commit this thread's uncommitted copies and wait for all of its copies.
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Point update of one chunk: the Fenwick nodes above local index l (l in
// 1..kChunk, stopping below the chunk top, at most kChunkLevels nodes) and the
// chunk total.  int64 nodes use exact 32-bit-pair atomics with all low-word
// atomics issued before any high-word one (one shared-atomic round trip);
// int32 nodes (and the int32 chunk total beside them: every partial sum of a
// block whose applied |delta| sum is below 2^31 fits) take plain 32-bit atomics
// with no return value.
template <typename Node>
__device__ __forceinline__ void chunk_add(Node* f, Node* tot, uint32_t l, uint64_t v) {
  const unsigned lo = (unsigned)v, hi = (unsigned)(v >> 32);
  unsigned* tw = reinterpret_cast<unsigned*>(tot);
  if constexpr (sizeof(Node) == 4) {
    uint32_t x = l;
#pragma unroll
    for (int lv = 0; lv < kChunkLevels; ++lv) {
      if (x < (uint32_t)kChunk) atomicAdd(reinterpret_cast<unsigned*>(f) + x, lo);
      x += x & (0u - x);
    }
    atomicAdd(tw, lo);
  } else {
    unsigned* fw = reinterpret_cast<unsigned*>(f);
    unsigned old[kChunkLevels];
    uint32_t x = l;
#pragma unroll
    for (int lv = 0; lv < kChunkLevels; ++lv) {
      if (x < (uint32_t)kChunk) old[lv] = atomicAdd(fw + 2 * x, lo);
      x += x & (0u - x);
    }
    const unsigned oldt = atomicAdd(tw, lo);
    x = l;
#pragma unroll
    for (int lv = 0; lv < kChunkLevels; ++lv) {
      if (x < (uint32_t)kChunk) {
        const unsigned h = hi + ((old[lv] + lo) < old[lv] ? 1u : 0u);
        if (h) atomicAdd(fw + 2 * x + 1, h);
      }
      x += x & (0u - x);
    }
    const unsigned ht = hi + ((oldt + lo) < oldt ? 1u : 0u);
    if (ht) atomicAdd(tw + 1, ht);
  }
}

// Flat chunk update: the rank's own value and the chunk total (both of the
// node type, so int32 blocks make two no-return atomics).
template <typename Node>
__device__ __forceinline__ void flat_add(Node* f, Node* tot, uint32_t i, uint64_t v) {
  if constexpr (sizeof(Node) == 4) {
    atomicAdd(reinterpret_cast<unsigned*>(f) + i, (unsigned)v);
    atomicAdd(reinterpret_cast<unsigned*>(tot), (unsigned)v);
  } else {
    shared_add_u64(reinterpret_cast<unsigned long long*>(f) + i, v);
    shared_add_u64(reinterpret_cast<unsigned long long*>(tot), v);
  }
}

template <typename Node>
__device__ __forceinline__ uint64_t node_value(Node x) {
  if constexpr (sizeof(Node) == 4) return (uint64_t)(int64_t)(int32_t)x;
  else return (uint64_t)x;
}

// Prefix of ranks < r: coarse prefix of the chunk plus the in-chunk Fenwick nodes
// (<= kChunkLevels, indices known up front so the loads issue together).
template <typename Node>
__device__ __forceinline__ uint64_t chunk_prefix(const Node* fine, const unsigned long long* P, uint32_t r) {
  const uint32_t h = r >> kChunkBits;
  const Node* f = fine + (size_t)h * kChunkStride;
  uint64_t v = P[h];
  uint32_t x = r & (kChunk - 1u);
#pragma unroll
  for (int it = 0; it < kChunkLevels; ++it) {
    if (x) v += node_value(f[x]);
    x &= x - 1;
  }
  return v;
}

// Prefix (keys < k) of the slice's contribution.
template <typename Node>
__device__ __forceinline__ uint64_t slice_prefix2(const Node* fine, const unsigned long long* P, uint32_t n,
                                                  const uint64_t* bits, const uint32_t* rl, uint32_t klo,
                                                  uint32_t khi, uint32_t k) {
  if (k <= klo) return 0;
  const uint32_t r = k >= khi ? n : local_rank(bits, rl, k - klo);
  return chunk_prefix(fine, P, r);
}

// A tile: steps [s, e) whose events (up to kTileEv, in step order) and queries (up
// to kTileQ) are staged together; bit i of qm[i / 64] marks step s + i as a query
// step (tiles span at most 128 steps).
struct Tile {
  int32_t s, e;
  uint64_t qm[2];
  __device__ __forceinline__ bool any_query() const { return (qm[0] | qm[1]) != 0; }
  __device__ __forceinline__ void clear() { qm[0] = qm[1] = 0; }
};
// Query steps of a tile in order: the next one's offset from the tile start (the
// masks must not both be empty), and removing it.
__device__ __forceinline__ int32_t next_query_step(const uint64_t* qm) {
  return qm[0] ? __ffsll((long long)qm[0]) - 1 : 64 + __ffsll((long long)qm[1]) - 1;
}
__device__ __forceinline__ void pop_query_step(uint64_t* qm) {
  if (qm[0]) qm[0] &= qm[0] - 1; else qm[1] &= qm[1] - 1;
}

template <typename Node, typename Cfg>
__device__ __forceinline__ void sweep_block(const SweepParams& p, const SweepLayout& L, unsigned char* smem,
                                            int32_t b) {
  const BlockTab bt = p.blocks[b];
  uint64_t* sbits = reinterpret_cast<uint64_t*>(smem);
  uint32_t* srl = reinterpret_cast<uint32_t*>(smem + L.off_rl);
  Node* fine = reinterpret_cast<Node*>(smem + L.off_fine);
  Node* T = reinterpret_cast<Node*>(smem + L.off_T);   // chunk totals
  StepDesc* ring = reinterpret_cast<StepDesc*>(smem + L.off_ring);
  StepDesc* pdesc = reinterpret_cast<StepDesc*>(smem + L.off_pdesc);   // [Cfg::kRingFill] next refill
  int64_t* epre = reinterpret_cast<int64_t*>(smem + L.off_epre);   // events before step, per ring slot
  int64_t* qpre = reinterpret_cast<int64_t*>(smem + L.off_qpre);   // queries before step, per ring slot
  BwEvent* evbuf = reinterpret_cast<BwEvent*>(smem + L.off_ev);     // [2][Cfg::kTileEv]
  uint8_t* emeta = smem + L.off_emeta;                               // [2][Cfg::kTileEv] step << 1 | exit
  uint8_t* qmeta = smem + L.off_qmeta;                               // [2][Cfg::kTileQ] step
  unsigned long long* corr = reinterpret_cast<unsigned long long*>(smem + L.off_corr);  // [kOfflineQ]
  unsigned char* qbuf = smem + L.off_q;                              // [2][Cfg::kTileQ] x 12 B
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // flattened queries g = qslot + 256 m belong to this thread: consecutive queries
  // go to different warps, so a tile's few queries are probed by different warps
  const int qslot = lane * Cfg::kWarps + warp;
  unsigned long long* Pw = reinterpret_cast<unsigned long long*>(smem + L.off_P) + (size_t)warp * (kMaxChunks + 1);
  constexpr int32_t M = Cfg::kRing - 1;

  const int32_t t0 = bt.t0, t1 = bt.t1;
  if (t0 >= t1) return;
  const int32_t nsl = p.nslices[b];
  const uint64_t* gbits = p.bits + bt.bits_off;
  const uint32_t* grl = p.rlut + bt.bits_off + b;
  const int64_t* crow = bt.carry_in >= 0 ? p.carry + bt.carry_in : nullptr;

  // Slices without keys change no answer: they are skipped, except that one pass
  // (the first slice with keys, else slice 0) writes every answer.
  const Slice* bsl = p.slices + (size_t)b * kMaxSlices;
  int32_t first_si = 0;
  while (first_si < nsl && bsl[first_si].n == 0) ++first_si;
  if (first_si == nsl) first_si = 0;
  for (int32_t si = 0; si < nsl; ++si) {
    const Slice s = bsl[si];
    if (s.n == 0 && si != first_si) continue;
    const int32_t nwd = s.word_hi - s.word_lo;
    const uint32_t klo = (uint32_t)s.word_lo << 6;
    const uint32_t khi = (uint32_t)imin64((int64_t)s.word_hi << 6, (int64_t)bt.C);
    const uint32_t nch = (s.n + kChunk - 1) / kChunk;
    // Flat chunks keep R copies of each chunk total side by side (copy lane % R), so
    // the lanes of a warp updating the same chunk of a small slice hit different
    // words; R is the largest power of two <= 8 whose copies fit the totals' space.
    uint32_t R = 1;
    if constexpr (Cfg::kFlat) {
      const uint32_t cap = (uint32_t)((size_t)L.nch32 * 8 / sizeof(Node));
      while (R < 8 && nch > 0 && 2 * R * nch <= cap) R *= 2;
    }
    const bool first = si == first_si;
    const bool carried = first && crow != nullptr;
    for (int i = tid; i < nwd; i += Cfg::kThreads) {
      sbits[i] = gbits[s.word_lo + i];
      srl[i] = grl[s.word_lo + i] - s.rank_lo;
    }
    for (uint32_t i = tid; i < nch * kChunkStride; i += Cfg::kThreads) fine[i] = 0;
    for (uint32_t i = tid; i < nch * R; i += Cfg::kThreads) T[i] = 0;
    for (int i = tid; i < kOfflineQ; i += Cfg::kThreads) corr[i] = 0;

    // Step ring: descriptors and event/query prefixes of steps [filled - Cfg::kRing, filled);
    // steps past t1 read as empty.  A refill overwrites the oldest Cfg::kRingFill slots;
    // the last warp (FW) loads them and scans their counts (the running totals live in
    // that warp).
    int32_t filled = t0;
    int64_t run_e = 0, run_q = 0;
    constexpr int FW = Cfg::kWarps - 1;
    // Warp FW copies the descriptors of the next refill into shared memory (cp.async,
    // one refill ahead; the copies join the warp's next commit group), so a refill
    // costs a scan and shared stores, not a global load.
    constexpr int PER = Cfg::kRingFill / 32;
    auto prefetch = [&](int32_t from) {
      for (int i = lane; i < Cfg::kRingFill; i += 32) {
        const int32_t t = from + i;
        if (t < t1) {
          cp_async16(pdesc + i, p.desc + t);
        } else {
          StepDesc z;
          z.e0 = 0; z.q0 = 0; z.ne = 0; z.nq = 0;
          pdesc[i] = z;
        }
      }
    };
    if (warp == FW) prefetch(t0);
    // Warp FW's part of a refill (the caller keeps readers of the overwritten slots
    // and of the new ones on the right sides of barriers).
    auto refill = [&]() {
      if (warp == FW) {
        cp_async_wait_all();   // this warp's descriptor copies (and its own tile copies)
        __syncwarp();
        // lane takes descriptors [lane * PER, (lane + 1) * PER): sums, warp scan, then
        // a second pass over the staged copies writes the ring slots and prefixes
        const StepDesc* mine = pdesc + lane * PER;
        int64_t le = 0, lq = 0;
#pragma unroll
        for (int j = 0; j < PER; ++j) {
          const int32_t ne = mine[j].ne, nq = mine[j].nq;
          le += ne;
          lq += nq > 0 ? nq : 0;
        }
        int64_t ie = le, iq = lq;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int64_t ye = __shfl_up_sync(0xffffffffu, ie, o), yq = __shfl_up_sync(0xffffffffu, iq, o);
          if (lane >= o) { ie += ye; iq += yq; }
        }
        int64_t xe = run_e + ie - le, xq = run_q + iq - lq;
#pragma unroll 2
        for (int j = 0; j < PER; ++j) {
          const StepDesc d = mine[j];
          const int32_t sl = (filled + lane * PER + j) & M;
          ring[sl] = d;
          epre[sl] = xe;
          qpre[sl] = xq;
          xe += d.ne;
          xq += d.nq > 0 ? d.nq : 0;
        }
        run_e += __shfl_sync(0xffffffffu, ie, 31);
        run_q += __shfl_sync(0xffffffffu, iq, 31);
        __syncwarp();   // every lane has read the staged descriptors
        prefetch(filled + Cfg::kRingFill);
        __syncwarp();   // the new slots are visible to the warp's other lanes
      }
      filled += Cfg::kRingFill;
    };
    auto fill = [&]() {
      __syncthreads();
      refill();
      __syncthreads();
    };
    // Tile from step s: as many whole steps (<= kTileSteps) as fit kTileEv events and
    // kTileQ queries, at least one.  The fit is monotone in the end step, so each
    // warp counts it with one ballot per 32 candidate ends; every warp computes the
    // same tile.
    auto make_tile = [&](int32_t st) -> Tile {
      constexpr int NB = (Cfg::kTileSteps + 31) / 32;
      const int32_t emax = min(st + Cfg::kTileSteps, t1);
      const int64_t le = epre[st & M] + Cfg::kTileEv, lq = qpre[st & M] + Cfg::kTileQ;
      int32_t e = st;
      int64_t qe[NB];   // query prefix after step st + 32 j + lane
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        const int32_t ea = st + 1 + 32 * j + lane;
        qe[j] = qpre[ea & M];
        bool ok = ea <= emax && epre[ea & M] <= le && qe[j] <= lq;
        if constexpr (Cfg::kFlat) {
          // and within the single-probe limits (queries x events), so that a tile is
          // replayed with one probe phase unless one step alone exceeds them
          if (ok) {
            const int64_t nqx = qpre[ea & M] - qpre[st & M], nex = epre[ea & M] - epre[st & M];
            ok = nqx <= kOfflineQ && nqx * nex <= kOfflinePairs;
          }
        }
        e += __popc(__ballot_sync(0xffffffffu, ok));
      }
      if (e == st) e = st + 1;
      Tile x;
      x.s = st;
      x.e = e;
      x.clear();
      // step u answers queries exactly when the query prefix grows across it
      int64_t before = qpre[st & M];
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        int64_t qb = __shfl_up_sync(0xffffffffu, qe[j], 1);
        if (lane == 0) qb = before;
        before = __shfl_sync(0xffffffffu, qe[j], 31);
        const bool q = st + 32 * j + lane < x.e && qe[j] > qb;
        x.qm[j >> 1] |= (uint64_t)__ballot_sync(0xffffffffu, q) << (32 * (j & 1));
      }
      return x;
    };
    // Stage a tile cooperatively: the first half of the warps copy (cp.async) the
    // events and the second half the queries of 32-step groups.  Lane l decodes step
    // l of the group; small steps are copied lane by lane, large ones by lanes taking
    // consecutive flattened items.  Each item's step (and exit flag) is written beside
    // it.  A barrier after the copies land makes the tile visible.
    auto stage = [&](const Tile& x, int buf) {
      const bool evw = warp < Cfg::kWarps / 2;
      const int wgrp = evw ? warp : warp - Cfg::kWarps / 2;
      const int64_t p0 = evw ? epre[x.s & M] : qpre[x.s & M];
      const int64_t cap = evw ? Cfg::kTileEv : Cfg::kTileQ;
      BwEvent* eb = evbuf + (size_t)buf * Cfg::kTileEv;
      uint8_t* em = emeta + (size_t)buf * Cfg::kTileEv;
      unsigned char* qb = qbuf + (size_t)buf * Cfg::kTileQ * 12;
      uint8_t* qm = qmeta + (size_t)buf * Cfg::kTileQ;
      constexpr int HW = Cfg::kWarps / 2;   // warps per half (events / queries)
      for (int32_t c = x.s, gi = 0; c < x.e; c += 32, ++gi) {
        const int32_t st = c + lane;
        int32_t cnt = 0;
        int64_t src = 0, f = 0;
        uint8_t meta = 0;
        if (st < x.e) {
          const StepDesc d = ring[st & M];
          f = (evw ? epre[st & M] : qpre[st & M]) - p0;
          const int64_t n = evw ? d.ne : (d.nq > 0 ? d.nq : 0);
          cnt = (int32_t)imin64(n, cap - f > 0 ? cap - f : 0);
          src = evw ? (int64_t)d.e0 : (int64_t)d.q0;
          meta = evw ? (uint8_t)(((st - x.s) << 1) | (d.nq < 0 ? 1 : 0)) : (uint8_t)(st - x.s);
        }
        int32_t most = cnt;
#pragma unroll
        for (int o = 16; o; o >>= 1) most = max(most, __shfl_xor_sync(0xffffffffu, most, o));
        auto put = [&](int64_t fpos, int64_t from, uint8_t mt) {
          if (evw) {
            cp_async16(eb + fpos, p.ev + from);
            em[fpos] = mt;
          } else {
            const uint32_t* q = reinterpret_cast<const uint32_t*>(p.qs + from);
            unsigned char* dq = qb + (size_t)fpos * 12;
            cp_async4(dq, q);
            cp_async4(dq + 4, q + 1);
            cp_async4(dq + 8, q + 2);
            qm[fpos] = mt;
          }
        };
        if (most <= 16) {
          // small steps: one warp of the half takes the group, lane l copies its step
          if (gi % HW == wgrp)
            for (int32_t i = 0; i < most; ++i)
              if (i < cnt) put(f + i, src + i, meta);
        } else {
          // large steps: the half's warps split the group's flattened items; a
          // lane finds its item's step by a shuffle search over the inclusive counts
          int32_t incl = cnt;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
          }
          const int32_t total = __shfl_sync(0xffffffffu, incl, 31);
          for (int32_t g0 = 32 * wgrp; g0 < total; g0 += 32 * HW) {
            const int32_t g = g0 + lane;
            int32_t lo = 0, hi = 31;   // first lane whose inclusive count exceeds g
#pragma unroll
            for (int it = 0; it < 5; ++it) {
              const int32_t mid = (lo + hi) >> 1;
              if (__shfl_sync(0xffffffffu, incl, mid) > g) hi = mid; else lo = mid + 1;
            }
            const int32_t s_incl = __shfl_sync(0xffffffffu, incl, lo), s_cnt = __shfl_sync(0xffffffffu, cnt, lo);
            const int64_t s_src = __shfl_sync(0xffffffffu, src, lo), s_f = __shfl_sync(0xffffffffu, f, lo);
            const uint8_t s_meta = (uint8_t)__shfl_sync(0xffffffffu, (uint32_t)meta, lo);
            if (g < total) {
              const int32_t off = g - (s_incl - s_cnt);
              put(s_f + off, s_src + off, s_meta);
            }
          }
        }
      }
      cp_async_commit();
    };
    // Stage a tile with one warp (the staging warp of a specialised tile): events,
    // then queries, 32 steps at a time; lane l decodes step l of the group, small
    // steps are copied lane by lane, large ones by lanes taking consecutive flattened
    // items.  The caller commits the copies.
    auto stage_warp = [&](const Tile& x, int buf) {
      BwEvent* eb = evbuf + (size_t)buf * Cfg::kTileEv;
      uint8_t* em = emeta + (size_t)buf * Cfg::kTileEv;
      unsigned char* qb = qbuf + (size_t)buf * Cfg::kTileQ * 12;
      uint8_t* qmt = qmeta + (size_t)buf * Cfg::kTileQ;
#pragma unroll 1
      for (int pass = 0; pass < 2; ++pass) {
        const bool evw = pass == 0;
        const int64_t p0 = evw ? epre[x.s & M] : qpre[x.s & M];
        const int64_t cap = evw ? Cfg::kTileEv : Cfg::kTileQ;
        if ((evw ? epre[x.e & M] : qpre[x.e & M]) == p0) continue;   // nothing of this kind
        for (int32_t c = x.s; c < x.e; c += 32) {
          const int32_t st = c + lane;
          int32_t cnt = 0;
          int64_t src = 0, f = 0;
          uint8_t meta = 0;
          if (st < x.e) {
            const StepDesc d = ring[st & M];
            f = (evw ? epre[st & M] : qpre[st & M]) - p0;
            const int64_t n = evw ? d.ne : (d.nq > 0 ? d.nq : 0);
            cnt = (int32_t)imin64(n, cap - f > 0 ? cap - f : 0);
            src = evw ? (int64_t)d.e0 : (int64_t)d.q0;
            meta = evw ? (uint8_t)(((st - x.s) << 1) | (d.nq < 0 ? 1 : 0)) : (uint8_t)(st - x.s);
          }
          int32_t most = cnt;
#pragma unroll
          for (int o = 16; o; o >>= 1) most = max(most, __shfl_xor_sync(0xffffffffu, most, o));
          auto put = [&](int64_t fpos, int64_t from, uint8_t mt) {
            if (evw) {
              cp_async16(eb + fpos, p.ev + from);
              em[fpos] = mt;
            } else {
              const uint32_t* q = reinterpret_cast<const uint32_t*>(p.qs + from);
              unsigned char* dq = qb + (size_t)fpos * 12;
              cp_async4(dq, q);
              cp_async4(dq + 4, q + 1);
              cp_async4(dq + 8, q + 2);
              qmt[fpos] = mt;
            }
          };
          if (most <= 16) {
            for (int32_t i = 0; i < most; ++i)
              if (i < cnt) put(f + i, src + i, meta);
          } else {
            int32_t incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
              const int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
              if (lane >= o) incl += y;
            }
            const int32_t total = __shfl_sync(0xffffffffu, incl, 31);
            for (int32_t g0 = 0; g0 < total; g0 += 32) {
              const int32_t g = g0 + lane;
              int32_t lo = 0, hi = 31;   // first lane whose inclusive count exceeds g
#pragma unroll
              for (int it = 0; it < 5; ++it) {
                const int32_t mid = (lo + hi) >> 1;
                if (__shfl_sync(0xffffffffu, incl, mid) > g) hi = mid; else lo = mid + 1;
              }
              const int32_t s_incl = __shfl_sync(0xffffffffu, incl, lo), s_cnt = __shfl_sync(0xffffffffu, cnt, lo);
              const int64_t s_src = __shfl_sync(0xffffffffu, src, lo), s_f = __shfl_sync(0xffffffffu, f, lo);
              const uint8_t s_meta = (uint8_t)__shfl_sync(0xffffffffu, (uint32_t)meta, lo);
              if (g < total) {
                const int32_t off = g - (s_incl - s_cnt);
                put(s_f + off, s_src + off, s_meta);
              }
            }
          }
        }
      }
    };
    auto apply = [&](uint32_t k, uint64_t v, bool neg) {
      if (k >= klo && k < khi) {
        if (neg) v = (uint64_t)0 - v;
        const uint32_t r = local_rank(sbits, srl, k - klo);
        if constexpr (Cfg::kFlat)
          flat_add<Node>(fine + (size_t)(r >> kChunkBits) * kChunkStride, T + (r >> kChunkBits) * R + (lane & (R - 1)),
                         r & (kChunk - 1u), v);
        else
          chunk_add<Node>(fine + (size_t)(r >> kChunkBits) * kChunkStride, T + (r >> kChunkBits),
                          (r & (kChunk - 1u)) + 1u, v);
      }
    };
    bool dirty = true;   // chunk totals changed since the warps' prefix copies were built
    auto rebuild = [&]() {
      // this warp's copy of the exclusive prefix of the chunk totals
      const uint32_t per = ((nch + 31) / 32) | 1u;  // odd: lanes hit different banks
      const uint32_t lo = lane * per;
      uint64_t tv[kRebuildPer];
      uint64_t sum = 0;
#pragma unroll
      for (int i = 0; i < kRebuildPer; ++i) {
        tv[i] = ((uint32_t)i < per && lo + i < nch) ? node_value(T[lo + i]) : 0;
        sum += tv[i];
      }
      uint64_t xx = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, xx, o);
        if (lane >= o) xx += y;
      }
      uint64_t run = xx - sum;
#pragma unroll
      for (int i = 0; i < kRebuildPer; ++i) {
        if ((uint32_t)i < per && lo + i < nch) Pw[lo + i] = run;
        run += tv[i];
      }
      if (lane == 31) Pw[nch] = xx;
      __syncwarp();
    };
    auto finish = [&](uint32_t lo, uint32_t hi, uint64_t acc, int64_t j) {
      int64_t* out = p.answers + j;
      if (hi <= lo) {
        if (first) *out = 0;
        return;
      }
      acc += slice_prefix2(fine, Pw, s.n, sbits, srl, klo, khi, hi);
      acc -= slice_prefix2(fine, Pw, s.n, sbits, srl, klo, khi, lo);
      *out = first ? (int64_t)acc : (int64_t)((uint64_t)*out + acc);
    };
    // Flat chunks: this lane's share of the sum over the slice ranks of keys in
    // [lo, hi): every 32nd value of the partial chunks at both ends and every 32nd
    // chunk total between them (read straight from the shared chunk totals, so no
    // prefix copy has to be rebuilt after updates).
    auto key_rank = [&](uint32_t k) -> uint32_t {
      return k <= klo ? 0u : (k >= khi ? s.n : local_rank(sbits, srl, k - klo));
    };
    // Lane partial sums are kept in the node type: an int32 block's every partial
    // sum fits int32 (its applied |delta| sum is below 2^31), so 32-bit wrapping
    // arithmetic and one warp reduction give the exact value, sign-extended after.
    auto flat_range = [&](uint32_t lo, uint32_t hi) -> Node {
      const uint32_t ra = key_rank(lo), rb = key_rank(hi);
      if (rb <= ra) return 0;
      const uint32_t ha = ra >> kChunkBits, hb = (rb - 1u) >> kChunkBits;
      const uint32_t ia = ra & (kChunk - 1u), ib = ((rb - 1u) & (kChunk - 1u)) + 1u;   // [ia, kChunk) of ha, [0, ib) of hb
      const Node* fa = fine + (size_t)ha * kChunkStride;
      // fixed trip counts with predicated loads, so all of a lane's loads issue together
      const uint32_t enda = ha == hb ? ib : (uint32_t)kChunk;
      Node v = 0;
#pragma unroll
      for (int t = 0; t < kChunk / 32; ++t) {
        const uint32_t i = ia + lane + 32u * t;
        v += i < enda ? fa[i] : Node(0);
      }
      if (ha != hb) {
        const Node* fb = fine + (size_t)hb * kChunkStride;
#pragma unroll
        for (int t = 0; t < kChunk / 32; ++t) {
          const uint32_t i = lane + 32u * t;
          v += i < ib ? fb[i] : Node(0);
        }
        // the copies of the chunks strictly between: T[(ha + 1) R, hb R), at most
        // the totals' space (2 kMaxChunks int32 words)
        const uint32_t c1 = hb * R;
#pragma unroll
        for (int t = 0; t < 2 * kMaxChunks / 32; ++t) {
          const uint32_t c = (ha + 1u) * R + lane + 32u * t;
          v += c < c1 ? T[c] : Node(0);
        }
      }
      return v;
    };
    auto warp_sum = [&](Node v) -> uint64_t {
      if constexpr (sizeof(Node) == 4) {
        return (uint64_t)(int64_t)(int32_t)__reduce_add_sync(0xffffffffu, v);
      } else {
        uint64_t d = v;
#pragma unroll
        for (int o = 16; o; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        return d;
      }
    };
    // Answer the queries of the lanes with `mine` (warp-uniform call): Fenwick chunks
    // let each owner finish alone; flat chunks sum the chunk's values with the warp.
    auto finish_warp = [&](bool mine, uint32_t lo, uint32_t hi, uint64_t acc, int64_t j) {
      if constexpr (!Cfg::kFlat) {
        if (mine) finish(lo, hi, acc, j);
      } else {
        uint32_t owners = __ballot_sync(0xffffffffu, mine);
        while (owners) {
          const int src = __ffs(owners) - 1;
          owners &= owners - 1;
          const uint32_t l = __shfl_sync(0xffffffffu, lo, src), h = __shfl_sync(0xffffffffu, hi, src);
          const uint64_t d = warp_sum(h > l ? flat_range(l, h) : Node(0));
          if (lane == src) {
            int64_t* out = p.answers + j;
            if (hi <= lo) {
              if (first) *out = 0;
            } else {
              const uint64_t a = acc + d;
              *out = first ? (int64_t)a : (int64_t)((uint64_t)*out + a);
            }
          }
        }
      }
    };
    // Replay a staged, visible tile.  Thread t applies flattened events t + 256 m;
    // the tile's queries g = qslot + 256 m belong to this thread.  Segment mode:
    // segments of steps ending at each query step; the updates of a segment, a
    // barrier, the probes of its query step, a barrier.  Offline mode (few queries x
    // events): every query of the tile probed against the state at the tile start
    // plus the tile's events of its own and earlier steps (summed by the owner's
    // warp), a barrier, then all of the tile's updates.  Updates after the last probe
    // of a tile run without a barrier.
    auto process = [&](const Tile& x, int buf) {
      const int64_t pe0 = epre[x.s & M], ne = epre[x.e & M] - pe0;
      const int64_t pq0 = qpre[x.s & M], nq = qpre[x.e & M] - pq0;
      const int64_t ns_e = imin64(ne, Cfg::kTileEv), ns_q = imin64(nq, Cfg::kTileQ);
      const BwEvent* eb = evbuf + (size_t)buf * Cfg::kTileEv;
      const uint8_t* em = emeta + (size_t)buf * Cfg::kTileEv;
      const unsigned char* qb = qbuf + (size_t)buf * Cfg::kTileQ * 12;
      const uint8_t* qmt = qmeta + (size_t)buf * Cfg::kTileQ;
      uint64_t c_lo[Cfg::kQPer], c_hi[Cfg::kQPer];
#pragma unroll
      for (int m = 0; m < Cfg::kQPer; ++m) {
        c_lo[m] = c_hi[m] = 0;
        const int64_t g = qslot + m * Cfg::kThreads;
        if (carried && g < ns_q) {
          const uint32_t* q = reinterpret_cast<const uint32_t*>(qb + (size_t)g * 12);
          if (q[2] > q[1]) {
            c_lo[m] = (uint64_t)__ldg(crow + q[1]);
            c_hi[m] = (uint64_t)__ldg(crow + q[2]);
          }
        }
      }
      // answers index of the staged query g of tile step u
      auto qindex = [&](int32_t urel, int64_t g) -> int64_t {
        const int32_t u = x.s + urel;
        return (int64_t)ring[u & M].q0 + (pq0 + g - qpre[u & M]);
      };
      if (x.any_query() && ne <= Cfg::kTileEv && nq <= kOfflineQ && nq * ne <= kOfflinePairs) {
        if (!Cfg::kFlat && dirty) {
          rebuild();
          dirty = false;
        }
        {
          // the tile's event/query pairs: query g's events are cut into `parts` ranges
          // of whole 32-event chunks, one warp per (query, range), summed into corr[g]
          const int32_t nchunk = (int32_t)((ne + 31) / 32);
          const int32_t parts = max(1, min(nchunk, Cfg::kWarps / max(1, (int32_t)nq)));
          const int32_t per = (nchunk + parts - 1) / parts;
          for (int32_t it = warp; it < (int32_t)nq * parts; it += Cfg::kWarps) {
            const int32_t g = it / parts, part = it - g * parts;
            const uint32_t* q = reinterpret_cast<const uint32_t*>(qb + (size_t)g * 12);
            const uint32_t lo = q[1], hi = q[2];
            const int32_t urel = qmt[g];
            const uint32_t a_lo = lo > klo ? lo : klo, a_hi = hi < khi ? hi : khi;
            if (!s.n || a_lo >= a_hi) continue;
            uint64_t v = 0;
            const int64_t i1 = imin64(ne, (int64_t)(part + 1) * per * 32);
#pragma unroll 4
            for (int64_t i = (int64_t)part * per * 32 + lane; i < i1; i += 32) {
              const uint8_t mt = em[i];
              const BwEvent e = eb[i];
              if ((int32_t)(mt >> 1) <= urel && e.key >= a_lo && e.key < a_hi)
                v += (mt & 1) ? (uint64_t)0 - (uint64_t)e.delta : (uint64_t)e.delta;
            }
#pragma unroll
            for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0 && v) shared_add_u64(corr + g, v);
          }
        }
        __syncthreads();   // every pair summed
#pragma unroll
        for (int m = 0; m < Cfg::kQPer; ++m) {
          const int64_t g = qslot + m * Cfg::kThreads;
          const bool mine = g < nq;
          uint32_t lo = 0, hi = 0;
          uint64_t acc = 0;
          int64_t j = 0;
          if (mine) {
            const uint32_t* q = reinterpret_cast<const uint32_t*>(qb + (size_t)g * 12);
            lo = q[1]; hi = q[2];
            acc = (uint64_t)corr[g] + (c_hi[m] - c_lo[m]);
            j = qindex((int32_t)qmt[g], g);
            corr[g] = 0;
          }
          finish_warp(mine, lo, hi, acc, j);
        }
        __syncthreads();   // probes done before this tile's updates
        if (s.n) {
#pragma unroll
          for (int m = 0; m < Cfg::kEvPer; ++m) {
            const int64_t g = tid + m * Cfg::kThreads;
            if (g < ne) {
              const BwEvent e = eb[g];
              apply(e.key, (uint64_t)e.delta, em[g] & 1);
            }
          }
        }
        if (ne > 0) dirty = true;
        return;
      }
      uint32_t done = 0;         // staged slots tid + 256 m applied so far
      int32_t a = x.s;           // first step of the current segment
      uint64_t qm[2] = {x.qm[0], x.qm[1]};
      for (;;) {
        const bool has_q = (qm[0] | qm[1]) != 0;
        const int32_t u = has_q ? x.s + next_query_step(qm) : x.e - 1;
        const int32_t urel = u - x.s;
        if (s.n) {
#pragma unroll
          for (int m = 0; m < Cfg::kEvPer; ++m) {
            const int64_t g = tid + m * Cfg::kThreads;
            if (!(done >> m & 1u) && g < ns_e) {
              const uint8_t mt = em[g];
              if ((int32_t)(mt >> 1) <= urel) {
                const BwEvent e = eb[g];
                apply(e.key, (uint64_t)e.delta, mt & 1);
                done |= 1u << m;
              }
            }
          }
          if (ne > Cfg::kTileEv && a == x.s) {  // one step with more events than a tile stages
            const StepDesc d = ring[x.s & M];
            for (int64_t g = Cfg::kTileEv + tid; g < ne; g += Cfg::kThreads) {
              const BwEvent e = p.ev[(int64_t)d.e0 + g];
              apply(e.key, (uint64_t)e.delta, d.nq < 0);
            }
          }
        }
        if (epre[(u + 1) & M] > epre[a & M]) dirty = true;
        if (!has_q) break;
        __syncthreads();  // every update of steps <= u is applied
        if (!Cfg::kFlat && dirty) {
          rebuild();
          dirty = false;
        }
#pragma unroll
        for (int m = 0; m < Cfg::kQPer; ++m) {
          const int64_t g = qslot + m * Cfg::kThreads;
          const bool mine = g < ns_q && (int32_t)qmt[g] == urel;
          uint32_t lo = 0, hi = 0;
          if (mine) {
            const uint32_t* q = reinterpret_cast<const uint32_t*>(qb + (size_t)g * 12);
            lo = q[1]; hi = q[2];
          }
          finish_warp(mine, lo, hi, c_hi[m] - c_lo[m], mine ? qindex(urel, g) : 0);
        }
        if (nq > Cfg::kTileQ) {  // one step with more queries than a tile stages
          const int64_t qbase = qindex(urel, 0);
          for (int64_t g0 = Cfg::kTileQ + (tid & ~31); g0 < nq; g0 += Cfg::kThreads) {   // warp-uniform
            const int64_t g = g0 + lane;
            const bool mine = g < nq;
            BwQuery qq;
            qq.lo = qq.hi = 0;
            uint64_t acc = 0;
            if (mine) {
              qq = p.qs[qbase + g];
              if (carried && qq.hi > qq.lo) acc = (uint64_t)__ldg(crow + qq.hi) - (uint64_t)__ldg(crow + qq.lo);
            }
            finish_warp(mine, qq.lo, qq.hi, acc, qbase + g);
          }
        }
        __syncthreads();  // probes done before the next updates
        pop_query_step(qm);
        a = u + 1;
      }
    };

    // Each staged item's step: the last step of the tile starting at or before the
    // item's flattened position, found for all of the thread's items at once by
    // binary lifting over the low words of the prefixes (a position inside a tile
    // is below 2^32, so 32-bit differences are exact).
    auto stage_own = [&](const Tile& x, int buf, int32_t* own_e, int32_t* own_q) {
      const int64_t pe0 = epre[x.s & M], ne = epre[x.e & M] - pe0;
      const int64_t pq0 = qpre[x.s & M], nq = qpre[x.e & M] - pq0;
      const uint32_t* elo = reinterpret_cast<const uint32_t*>(epre);   // low word of slot i at 2 i
      const uint32_t* qlo = reinterpret_cast<const uint32_t*>(qpre);
      const uint32_t pe0l = (uint32_t)pe0, pq0l = (uint32_t)pq0;
      int32_t se[Cfg::kEvPer], sq[Cfg::kQPer];
      bool wq[Cfg::kQPer];   // this warp holds a query slot of the tile (few warps do)
#pragma unroll
      for (int m = 0; m < Cfg::kEvPer; ++m) se[m] = x.s;
#pragma unroll
      for (int m = 0; m < Cfg::kQPer; ++m) {
        sq[m] = x.s;
        wq[m] = __any_sync(0xffffffffu, (int64_t)(qslot + m * Cfg::kThreads) < nq);
      }
#pragma unroll
      for (int b = Cfg::kTileSteps / 2; b; b >>= 1) {
#pragma unroll
        for (int m = 0; m < Cfg::kEvPer; ++m) {
          const int32_t c = se[m] + b;
          if (c < x.e && elo[2 * (c & M)] - pe0l <= (uint32_t)(tid + m * Cfg::kThreads)) se[m] = c;
        }
#pragma unroll
        for (int m = 0; m < Cfg::kQPer; ++m) {
          const int32_t c = sq[m] + b;
          if (wq[m] && c < x.e && qlo[2 * (c & M)] - pq0l <= (uint32_t)(qslot + m * Cfg::kThreads)) sq[m] = c;
        }
      }
#pragma unroll
      for (int m = 0; m < Cfg::kEvPer; ++m) {
        const int64_t g = tid + m * Cfg::kThreads;
        own_e[m] = -1;
        if (g < ne) {
          const int32_t lo = se[m];
          const StepDesc d = ring[lo & M];
          cp_async16(evbuf + (size_t)buf * Cfg::kTileEv + g, p.ev + (int64_t)d.e0 + (pe0 + g - epre[lo & M]));
          own_e[m] = ((lo - x.s) << 1) | (d.nq < 0 ? 1 : 0);
        }
      }
#pragma unroll
      for (int m = 0; m < Cfg::kQPer; ++m) {
        const int64_t g = qslot + m * Cfg::kThreads;
        own_q[m] = -1;
        if (g < nq) {
          const int32_t lo = sq[m];
          const StepDesc d = ring[lo & M];
          const uint32_t* src = reinterpret_cast<const uint32_t*>(p.qs + (int64_t)d.q0 + (pq0 + g - qpre[lo & M]));
          unsigned char* dq = qbuf + ((size_t)buf * Cfg::kTileQ + g) * 12;
          cp_async4(dq, src);
          cp_async4(dq + 4, src + 1);
          cp_async4(dq + 8, src + 2);
          own_q[m] = lo - x.s;
          qmeta[(size_t)buf * Cfg::kTileQ + g] = (uint8_t)(lo - x.s);
        }
      }
      cp_async_commit();
    };
    // need: ring steps the next make_tile reads (filled must exceed it); the offline
    // path refills the ring between its two barriers (the overwritten slots hold
    // steps before x.s, which needs Cfg::kRing >= 3 * kTileSteps + kRingFill).
    // An offline tile also cuts the tile that starts at `next_end` (the end of the
    // tile staged next) in its probe phase (warp FW, after the refill) and hands it
    // over through shared memory.
    Tile* pre_tile = reinterpret_cast<Tile*>(smem + L.off_tiles);
    bool have_pre = false;
    auto process_own = [&](const Tile& x, int buf, const int32_t* own_e, const int32_t* own_q, int32_t next_end) {
      const int32_t need = next_end < t1 ? min(next_end + Cfg::kTileSteps, t1) : -1;
      const int64_t pe0 = epre[x.s & M], ne = epre[x.e & M] - pe0;
      const int64_t pq0 = qpre[x.s & M], nq = qpre[x.e & M] - pq0;
      const BwEvent* eb = evbuf + (size_t)buf * Cfg::kTileEv;
      const unsigned char* qb = qbuf + (size_t)buf * Cfg::kTileQ * 12;
      // Exit events are negated in place by their own stager once its copies have
      // landed, so scans and updates read signed deltas (other threads read them only
      // after the tile's first barrier).
      {
        BwEvent* ebw = evbuf + (size_t)buf * Cfg::kTileEv;
#pragma unroll
        for (int m = 0; m < Cfg::kEvPer; ++m)
          if (own_e[m] >= 0 && (own_e[m] & 1)) {
            int64_t* dp = &ebw[tid + m * Cfg::kThreads].delta;
            *dp = (int64_t)((uint64_t)0 - (uint64_t)*dp);
          }
      }
      uint64_t c_lo[Cfg::kQPer], c_hi[Cfg::kQPer];
#pragma unroll
      for (int m = 0; m < Cfg::kQPer; ++m) {
        c_lo[m] = c_hi[m] = 0;
        if (carried && own_q[m] >= 0) {
          const uint32_t* q = reinterpret_cast<const uint32_t*>(qb + (size_t)(qslot + m * Cfg::kThreads) * 12);
          if (q[2] > q[1]) {
            c_lo[m] = (uint64_t)__ldg(crow + q[1]);
            c_hi[m] = (uint64_t)__ldg(crow + q[2]);
          }
        }
      }
      // answers index of the staged query g of tile step u
      auto qindex = [&](int32_t urel, int64_t g) -> int64_t {
        const int32_t u = x.s + urel;
        return (int64_t)ring[u & M].q0 + (pq0 + g - qpre[u & M]);
      };
      if (x.any_query() && ne <= Cfg::kTileEv && nq <= kOfflineQ && nq * ne <= kOfflinePairs) {
        __syncthreads();   // earlier updates applied; this tile's staged events visible
        if (!Cfg::kFlat && dirty) {
          rebuild();
          dirty = false;
        }
        // Each query's owner warp sums, in one pass with its probe, the tile's events of
        // the query's own and earlier steps (a prefix of the staged events) whose key
        // lies in both [lo, hi) and the slice.  Flat chunks fold the probe's partial
        // sums into the same warp reduction; Fenwick chunks hand the correction to the
        // owner lane, which probes alone.
#pragma unroll
        for (int m = 0; m < Cfg::kQPer; ++m) {
          const bool mine = own_q[m] >= 0;
          const int64_t g = qslot + m * Cfg::kThreads;
          uint32_t lo = 0, hi = 0;
          if (mine) {
            const uint32_t* q = reinterpret_cast<const uint32_t*>(qb + (size_t)g * 12);
            lo = q[1]; hi = q[2];
          }
          uint64_t corr_own = 0;
          uint32_t owners = __ballot_sync(0xffffffffu, mine && hi > lo);
          while (owners) {
            const int src = __ffs(owners) - 1;
            owners &= owners - 1;
            const uint32_t l = __shfl_sync(0xffffffffu, lo, src), h = __shfl_sync(0xffffffffu, hi, src);
            const int32_t ur = __shfl_sync(0xffffffffu, own_q[m], src);
            const uint32_t a_lo = l > klo ? l : klo, a_hi = h < khi ? h : khi;
            Node d = 0;
            if (s.n && a_lo < a_hi) {
              const int32_t nev = (int32_t)(epre[(x.s + ur + 1) & M] - pe0);   // events of steps <= ur
#pragma unroll 4
              for (int32_t i = lane; i < nev; i += 32) {
                const BwEvent e = eb[i];   // signed (exits negated)
                if (e.key >= a_lo && e.key < a_hi) d += (Node)e.delta;
              }
            }
            if constexpr (Cfg::kFlat) d += flat_range(l, h);
            const uint64_t dsum = warp_sum(d);
            if (lane == src) corr_own = dsum;
          }
          if (mine) {
            const int64_t j = qindex(own_q[m], g);
            int64_t* out = p.answers + j;
            // (the ring refill below leaves the slots of x's steps alone)
            if (hi <= lo) {
              if (first) *out = 0;
            } else if constexpr (Cfg::kFlat) {
              const uint64_t a = corr_own + (c_hi[m] - c_lo[m]);
              *out = first ? (int64_t)a : (int64_t)((uint64_t)*out + a);
            } else {
              finish(lo, hi, corr_own + (c_hi[m] - c_lo[m]), j);
            }
          }
        }
        if (need >= filled) refill();
        if (next_end < t1) {
          if (warp == FW) {
            const Tile nt = make_tile(next_end);
            if (lane == 0) *pre_tile = nt;
          }
          have_pre = true;
        }
        __syncthreads();   // probes done before this tile's updates; refilled ring visible
        if (s.n) {
#pragma unroll
          for (int m = 0; m < Cfg::kEvPer; ++m) {
            if (own_e[m] >= 0) {
              const BwEvent e = eb[tid + m * Cfg::kThreads];
              apply(e.key, (uint64_t)e.delta, false);
            }
          }
        }
        if (ne > 0) dirty = true;
        return;
      }
      uint32_t done = 0;         // own staged events applied so far
      int32_t a = x.s;           // first step of the current segment
      uint64_t qm[2] = {x.qm[0], x.qm[1]};
      for (;;) {
        const bool has_q = (qm[0] | qm[1]) != 0;
        const int32_t u = has_q ? x.s + next_query_step(qm) : x.e - 1;
        const int32_t urel = u - x.s;
        if (s.n) {
#pragma unroll
          for (int m = 0; m < Cfg::kEvPer; ++m) {
            if (!(done >> m & 1u) && own_e[m] >= 0 && (own_e[m] >> 1) <= urel) {
              const BwEvent e = eb[tid + m * Cfg::kThreads];
              apply(e.key, (uint64_t)e.delta, false);
              done |= 1u << m;
            }
          }
          if (ne > Cfg::kTileEv && a == x.s) {  // one step with more events than a tile stages
            const StepDesc d = ring[x.s & M];
            for (int64_t g = Cfg::kTileEv + tid; g < ne; g += Cfg::kThreads) {
              const BwEvent e = p.ev[(int64_t)d.e0 + g];
              apply(e.key, (uint64_t)e.delta, d.nq < 0);
            }
          }
        }
        if (epre[(u + 1) & M] > epre[a & M]) dirty = true;
        if (!has_q) break;
        __syncthreads();  // every update of steps <= u is applied
        if (!Cfg::kFlat && dirty) {
          rebuild();
          dirty = false;
        }
#pragma unroll
        for (int m = 0; m < Cfg::kQPer; ++m) {
          const bool mine = own_q[m] == urel;
          uint32_t lo = 0, hi = 0;
          if (mine) {
            const uint32_t* q = reinterpret_cast<const uint32_t*>(qb + (size_t)(qslot + m * Cfg::kThreads) * 12);
            lo = q[1]; hi = q[2];
          }
          finish_warp(mine, lo, hi, c_hi[m] - c_lo[m], mine ? qindex(urel, qslot + m * Cfg::kThreads) : 0);
        }
        if (nq > Cfg::kTileQ) {  // one step with more queries than a tile stages
          const int64_t qbase = qindex(urel, 0);
          for (int64_t g0 = Cfg::kTileQ + (tid & ~31); g0 < nq; g0 += Cfg::kThreads) {   // warp-uniform
            const int64_t g = g0 + lane;
            const bool mine = g < nq;
            BwQuery qq;
            qq.lo = qq.hi = 0;
            uint64_t acc = 0;
            if (mine) {
              qq = p.qs[qbase + g];
              if (carried && qq.hi > qq.lo) acc = (uint64_t)__ldg(crow + qq.hi) - (uint64_t)__ldg(crow + qq.lo);
            }
            finish_warp(mine, qq.lo, qq.hi, acc, qbase + g);
          }
        }
        __syncthreads();  // probes done before the next updates
        pop_query_step(qm);
        a = u + 1;
      }
    };

    // Specialised tiles: the consumer warps (all but the staging warp FW) replay a
    // tile staged by FW; consumer-only barriers are named barrier 1.
    constexpr int kCW = Cfg::kWarps - 1, kCons = kCW * 32;
    constexpr int kEvPerC = (Cfg::kTileEv + kCons - 1) / kCons, kQPerC = (Cfg::kTileQ + kCons - 1) / kCons;
    auto cbar = [&]() { asm volatile("bar.sync 1, %0;\n" ::"n"(kCons) : "memory"); };
    auto process_spec = [&](const Tile& x, int buf) {
      const int64_t pe0 = epre[x.s & M], ne = epre[x.e & M] - pe0;
      const int64_t pq0 = qpre[x.s & M], nq = qpre[x.e & M] - pq0;
      const int64_t ns_e = imin64(ne, Cfg::kTileEv), ns_q = imin64(nq, Cfg::kTileQ);
      const BwEvent* eb = evbuf + (size_t)buf * Cfg::kTileEv;
      const uint8_t* em = emeta + (size_t)buf * Cfg::kTileEv;
      const unsigned char* qb = qbuf + (size_t)buf * Cfg::kTileQ * 12;
      const uint8_t* qmt = qmeta + (size_t)buf * Cfg::kTileQ;
      const int cslot = lane * kCW + warp;   // consecutive queries go to different warps
      auto qindex = [&](int32_t urel, int64_t g) -> int64_t {
        const int32_t u = x.s + urel;
        return (int64_t)ring[u & M].q0 + (pq0 + g - qpre[u & M]);
      };
      if (x.any_query() && ne <= Cfg::kTileEv && nq <= kOfflineQ && nq * ne <= kOfflinePairs) {
        // one probe phase on the state at the tile start: each query's owner warp sums
        // the tile's events of the query's own and earlier steps inside [lo, hi) and
        // the slice together with the probe's partial sums, in one warp reduction
#pragma unroll
        for (int m = 0; m < kQPerC; ++m) {
          const int64_t g = cslot + m * kCons;
          const bool mine = g < nq;
          uint32_t lo = 0, hi = 0;
          int32_t urel = 0;
          uint64_t c_lo = 0, c_hi = 0;
          if (mine) {
            const uint32_t* q = reinterpret_cast<const uint32_t*>(qb + (size_t)g * 12);
            lo = q[1]; hi = q[2];
            urel = qmt[g];
            if (carried && hi > lo) {
              c_lo = (uint64_t)__ldg(crow + lo);
              c_hi = (uint64_t)__ldg(crow + hi);
            }
          }
          uint64_t corr_own = 0;
          uint32_t owners = __ballot_sync(0xffffffffu, mine && hi > lo);
          while (owners) {
            const int src = __ffs(owners) - 1;
            owners &= owners - 1;
            const uint32_t l = __shfl_sync(0xffffffffu, lo, src), h = __shfl_sync(0xffffffffu, hi, src);
            const int32_t ur = __shfl_sync(0xffffffffu, urel, src);
            const uint32_t a_lo = l > klo ? l : klo, a_hi = h < khi ? h : khi;
            Node d = 0;
            if (s.n && a_lo < a_hi) {
              const int32_t nev = (int32_t)(epre[(x.s + ur + 1) & M] - pe0);   // events of steps <= ur
#pragma unroll 4
              for (int32_t i = lane; i < nev; i += 32) {
                const BwEvent e = eb[i];
                if (e.key >= a_lo && e.key < a_hi) d += (em[i] & 1) ? Node(0) - (Node)e.delta : (Node)e.delta;
              }
            }
            d += flat_range(l, h);
            const uint64_t dsum = warp_sum(d);
            if (lane == src) corr_own = dsum;
          }
          if (mine) {
            int64_t* out = p.answers + qindex(urel, g);
            if (hi <= lo) {
              if (first) *out = 0;
            } else {
              const uint64_t v = corr_own + (c_hi - c_lo);
              *out = first ? (int64_t)v : (int64_t)((uint64_t)*out + v);
            }
          }
        }
        cbar();   // probes done before this tile's updates
        if (s.n) {
#pragma unroll
          for (int m = 0; m < kEvPerC; ++m) {
            const int64_t g = tid + m * kCons;
            if (g < ne) {
              const BwEvent e = eb[g];
              apply(e.key, (uint64_t)e.delta, em[g] & 1);
            }
          }
        }
        return;
      }
      // Segments of steps ending at each query step: the updates of a segment, a
      // barrier, the probes of its query step, a barrier (a tile with no query
      // applies all of its events with no barrier).
      uint32_t done = 0;
      int32_t a = x.s;
      uint64_t qm[2] = {x.qm[0], x.qm[1]};
      for (;;) {
        const bool has_q = (qm[0] | qm[1]) != 0;
        const int32_t u = has_q ? x.s + next_query_step(qm) : x.e - 1;
        const int32_t urel = u - x.s;
        if (s.n) {
#pragma unroll
          for (int m = 0; m < kEvPerC; ++m) {
            const int64_t g = tid + m * kCons;
            if (!(done >> m & 1u) && g < ns_e) {
              const uint8_t mt = em[g];
              if ((int32_t)(mt >> 1) <= urel) {
                const BwEvent e = eb[g];
                apply(e.key, (uint64_t)e.delta, mt & 1);
                done |= 1u << m;
              }
            }
          }
          if (ne > Cfg::kTileEv && a == x.s) {  // one step with more events than a tile stages
            const StepDesc d = ring[x.s & M];
            for (int64_t g = Cfg::kTileEv + tid; g < ne; g += kCons) {
              const BwEvent e = p.ev[(int64_t)d.e0 + g];
              apply(e.key, (uint64_t)e.delta, d.nq < 0);
            }
          }
        }
        if (!has_q) break;
        cbar();  // every update of steps <= u is applied
#pragma unroll
        for (int m = 0; m < kQPerC; ++m) {
          const int64_t g = cslot + m * kCons;
          const bool mine = g < ns_q && (int32_t)qmt[g] == urel;
          uint32_t lo = 0, hi = 0;
          uint64_t acc = 0;
          if (mine) {
            const uint32_t* q = reinterpret_cast<const uint32_t*>(qb + (size_t)g * 12);
            lo = q[1]; hi = q[2];
            if (carried && hi > lo) acc = (uint64_t)__ldg(crow + hi) - (uint64_t)__ldg(crow + lo);
          }
          finish_warp(mine, lo, hi, acc, mine ? qindex(urel, g) : 0);
        }
        if (nq > Cfg::kTileQ) {  // one step with more queries than a tile stages
          const int64_t qbase = qindex(urel, 0);
          for (int64_t g0 = Cfg::kTileQ + (tid & ~31); g0 < nq; g0 += kCons) {   // warp-uniform
            const int64_t g = g0 + lane;
            const bool mine = g < nq;
            BwQuery qq;
            qq.lo = qq.hi = 0;
            uint64_t acc = 0;
            if (mine) {
              qq = p.qs[qbase + g];
              if (carried && qq.hi > qq.lo) acc = (uint64_t)__ldg(crow + qq.hi) - (uint64_t)__ldg(crow + qq.lo);
            }
            finish_warp(mine, qq.lo, qq.hi, acc, qbase + g);
          }
        }
        cbar();  // probes done before the next updates
        pop_query_step(qm);
        a = u + 1;
      }
    };

    if constexpr (Cfg::kSpec) {
      // Warp FW cuts and stages tile k + 2 while the consumers replay tile k; one CTA
      // barrier per tile hands tile k over (FW has waited for its copies; the
      // consumers have finished tile k - 1, whose buffer FW refills next).
      Tile* tq = reinterpret_cast<Tile*>(smem + L.off_tiles);   // [3] tiles in flight
      Tile last;
      last.s = last.e = t1;
      last.clear();
      if (warp == FW) {
        while (min(t0 + Cfg::kTileSteps, t1) + 1 > filled) refill();
        const Tile a0 = make_tile(t0);
        stage_warp(a0, 0);
        cp_async_commit();
        if (a0.e < t1) {
          while (min(a0.e + Cfg::kTileSteps, t1) + 1 > filled) refill();
          last = make_tile(a0.e);
          stage_warp(last, 1);
        }
        cp_async_commit();
        if (lane == 0) {
          tq[0] = a0;
          tq[1] = last;
        }
      }
      for (int32_t k = 0;; ++k) {
        if (warp == FW) cp_async_wait<1>();   // tile k's copies landed (tile k + 1's may be in flight)
        __syncthreads();                       // tile k visible; tile k - 1 replayed
        const Tile x = tq[k % 3];
        if (x.s >= t1) break;
        if (warp == FW) {
          Tile n;
          n.s = n.e = t1;
          n.clear();
          if (last.e < t1) {
            while (min(last.e + Cfg::kTileSteps, t1) + 1 > filled) refill();
            n = make_tile(last.e);
            stage_warp(n, (k + 2) % 3);
          }
          cp_async_commit();
          if (lane == 0) tq[(k + 2) % 3] = n;
          last = n;
        } else {
          process_spec(x, k % 3);
        }
      }
    } else if constexpr (Cfg::kCoop) {
      while (min(t0 + Cfg::kTileSteps, t1) + 1 > filled) fill();
      Tile cur = make_tile(t0);
      stage(cur, 0);
      int buf = 0;
      for (;;) {
        cp_async_wait<0>();
        __syncthreads();   // the current tile is staged and visible; the other buffer is free
        const int32_t ns = cur.e;
        Tile nxt;
        nxt.s = nxt.e = t1;
        nxt.clear();
        if (ns < t1) {
          while (min(ns + Cfg::kTileSteps, t1) + 1 > filled) fill();
          nxt = make_tile(ns);
          stage(nxt, buf ^ 1);
        }
        process(cur, buf);
        if (ns >= t1) break;
        cur = nxt;
        buf ^= 1;
      }
    } else {
      while (min(t0 + Cfg::kTileSteps, t1) + 1 > filled) fill();
      Tile cur = make_tile(t0);
      int32_t cur_e[Cfg::kEvPer], cur_q[Cfg::kQPer];
      stage_own(cur, 0, cur_e, cur_q);
      int buf = 0;
      for (;;) {
        const int32_t ns = cur.e;
        Tile nxt;
        int32_t nxt_e[Cfg::kEvPer], nxt_q[Cfg::kQPer];
        if (ns < t1) {
          while (min(ns + Cfg::kTileSteps, t1) + 1 > filled) fill();
          nxt = have_pre ? *pre_tile : make_tile(ns);
          stage_own(nxt, buf ^ 1, nxt_e, nxt_q);
        } else {
          nxt.s = nxt.e = t1;
          nxt.clear();
          cp_async_commit();
        }
        cp_async_wait<1>();   // this thread's copies of the current tile have landed
        have_pre = false;
        process_own(cur, buf, cur_e, cur_q, nxt.e);
        if (ns >= t1) break;
        cur = nxt;
  #pragma unroll
        for (int m = 0; m < Cfg::kEvPer; ++m) cur_e[m] = nxt_e[m];
  #pragma unroll
        for (int m = 0; m < Cfg::kQPer; ++m) cur_q[m] = nxt_q[m];
        buf ^= 1;
      }
    }
    cp_async_wait<0>();
    __syncthreads();
  }
}

template <typename Cfg>
__global__ void __launch_bounds__(Cfg::kThreads, Cfg::kMinBlocks) k_sweep(SweepParams p, SweepLayout L) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int32_t s_ticket;
  if (*p.status) return;  // never index with descriptors of rejected input
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_ticket = atomicAdd(p.ticket, 1);
    __syncthreads();
    const int32_t i = s_ticket;
    if (i >= p.B) break;
    const int32_t b = p.order ? p.order[i] : i;
    if (p.bmode[b]) sweep_block<unsigned, Cfg>(p, L, smem, b);
    else sweep_block<unsigned long long, Cfg>(p, L, smem, b);
  }
}

// ------------------------------------------------------------------ host side
static inline size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

static size_t sweep_budget(int ctas_per_sm) { return (size_t)(kSmemPerSM / ctas_per_sm) - 3072; }

// Default sweep: the Euler-tile sweep for forests (measured fastest on batched
// uneven trees), else by the query/event ratio.
static void finish_spec(PipeSpec& s, const Tuning& tune, bool forest) {
  s.tile = tune.tile >= kTileNarrowId && tune.tile <= kTileMaxId ? tune.tile
           : forest ? kTileEulerId : (s.Q * 8 >= s.E ? kTileNarrowId : kTileWideId);
  if (s.tile >= kTileNarrow512Id) s.ctas_per_sm = 1;   // a 512-thread CTA takes the SM's registers
  const int32_t nw = words_of(s.Cmax);
  const size_t bud = sweep_budget(s.ctas_per_sm);
  switch (s.tile) {
    case kTileWideId: s.SL = sweep_layout<TileWide>(nw, bud); break;
    case kTileEulerId:
      // the prepare pass cuts slices for the Euler sweep's window with the capacities
      // of the TileNarrow512 layout (both fit the Euler sweep's window)
      s.SL = sweep_layout<TileNarrow512>(nw, bud);
      s.SL.cap32 = std::min<uint32_t>(s.SL.cap32, kEsCap32);
      s.SL.cap64 = std::min<uint32_t>(s.SL.cap64, kEsCap64);
      break;
    case kTileNarrow512Id: s.SL = sweep_layout<TileNarrow512>(nw, bud); break;
    case kTileWide512Id: s.SL = sweep_layout<TileWide512>(nw, bud); break;
    case kTileSpec512Id: s.SL = sweep_layout<TileSpec512>(nw, bud); break;
    default: s.SL = sweep_layout<TileNarrow>(nw, bud); break;
  }
  if (tune.slice_ranks > 0) {
    const uint32_t cap = (uint32_t)tune.slice_ranks;
    if (s.SL.cap32 > cap) s.SL.cap32 = cap;
    if (s.SL.cap64 > cap) s.SL.cap64 = cap;
  }
}

int pipe_spec_one(int32_t S, uint32_t C, int64_t E, int64_t Q, int32_t blocks, bool chain, const Tuning& tune,
                  int sms, PipeSpec& s) {
  if (S < 1 || S >= (1 << 30) || C < 1 || E < 0 || Q < 0 || E >= ((int64_t)1 << 32) ||
      Q >= ((int64_t)1 << 32))
    return BW_EINVAL;
  s = PipeSpec();
  s.T = 1; s.S = S; s.E = E; s.Q = Q; s.Cmax = C; s.Smax = S; s.sms = sms; s.chain_hint = chain;
  const int64_t work = est_work(S, E, Q);
  int64_t B;
  if (blocks > 0) {
    B = blocks;
  } else {
    B = 2 * (int64_t)sms;                            // two sweep CTAs per SM hide each other's latency
    if (tune.block_work > 0) B = (work + tune.block_work - 1) / tune.block_work;
    const int64_t min_work = 65536;                  // below this a block is launch-dominated
    if (work / min_work < B) B = work / min_work;
    const double carry_budget = 4.0e9;               // bytes of dense carry rows
    const int64_t by_mem = (int64_t)(carry_budget / (8.0 * ((double)C + 1.0)));
    if (by_mem < B) B = by_mem;
    if (B < 1) B = 1;
  }
  if (B > (1 << 24)) return BW_EINVAL;
  s.B = (int32_t)B;
  s.nb1 = s.B;
  const int64_t width = (int64_t)C + 1;
  s.bits_words = B * (int64_t)words_of(C);
  const int64_t rows = B - 1;
  const int64_t groups = (rows + kCarryGroup - 1) / kCarryGroup;
  s.carry_words = rows * width;
  s.group_pass = groups > 1;
  s.gsum_words = groups > 1 ? groups * width : 0;
  s.n_units = (int32_t)(groups * ((width + kCarryChunk - 1) / kCarryChunk));
  s.ctas_per_sm = tune.ctas_per_sm > 0 ? tune.ctas_per_sm : (B >= 2 * sms ? 2 : 1);
  finish_spec(s, tune, false);
  return 0;
}

int pipe_spec_forest(int32_t T, const int64_t* soff, const int64_t* eoff, const int64_t* qoff, const uint32_t* C,
                     const Tuning& tune, int sms, PipeSpec& s) {
  if (T < 1 || !soff || !eoff || !qoff || !C) return BW_EINVAL;
  if (soff[0] != 0 || eoff[0] != 0 || qoff[0] != 0) return BW_EINVAL;
  for (int32_t t = 0; t < T; ++t)
    if (soff[t + 1] <= soff[t] || eoff[t + 1] < eoff[t] || qoff[t + 1] < qoff[t] || C[t] < 1) return BW_EINVAL;
  if (soff[T] >= (1 << 30) || eoff[T] >= ((int64_t)1 << 32) || qoff[T] >= ((int64_t)1 << 32)) return BW_EINVAL;
  s = PipeSpec();
  s.T = T; s.S = (int32_t)soff[T]; s.E = eoff[T]; s.Q = qoff[T]; s.sms = sms;
  std::vector<int64_t> W(T);
  int64_t Wtot = 0;
  for (int32_t t = 0; t < T; ++t) {
    const int64_t ns = soff[t + 1] - soff[t];
    W[t] = est_work(ns, eoff[t + 1] - eoff[t], qoff[t + 1] - qoff[t]);
    Wtot += W[t];
    s.Cmax = std::max(s.Cmax, C[t]);
    s.Smax = std::max<int32_t>(s.Smax, (int32_t)ns);
  }
  s.ctas_per_sm = tune.ctas_per_sm > 0 ? tune.ctas_per_sm : 2;
  finish_spec(s, tune, true);   // the sweep layout depends only on the domains and the tuning
  int64_t target = tune.block_work > 0 ? tune.block_work
                                       : std::max<int64_t>(65536, Wtot / (4 * (int64_t)s.ctas_per_sm * sms));
  std::vector<int32_t> nb(T);
  for (;;) {                       // the block work doubles until the carry rows fit
    int64_t carry = 0, blocks = 0;
    for (int32_t t = 0; t < T; ++t) {
      nb[t] = (int32_t)std::max<int64_t>(1, (W[t] + target - 1) / target);
      carry += (int64_t)(nb[t] - 1) * ((int64_t)C[t] + 1);
      blocks += nb[t];
    }
    if (carry * 8 <= (int64_t)4e9 && blocks < (1 << 24)) break;  // dense carry rows within 4 GB
    target *= 2;
  }
  s.h_soff.resize(T + 1); s.h_eoff.assign(eoff, eoff + T + 1); s.h_qoff.assign(qoff, qoff + T + 1);
  s.h_C.assign(C, C + T);
  s.h_boff.resize(T + 1); s.h_bits.resize(T); s.h_carry.resize(T); s.h_gsum.resize(T);
  int64_t bits = 0, carry = 0, gsum = 0;
  int32_t boff = 0;
  for (int32_t t = 0; t < T; ++t) {
    s.h_soff[t] = (int32_t)soff[t];
    s.h_boff[t] = boff;
    s.h_bits[t] = bits;
    s.h_carry[t] = carry;
    s.h_gsum[t] = gsum;
    const int64_t width = (int64_t)C[t] + 1, rows = nb[t] - 1;
    const int64_t groups = (rows + kCarryGroup - 1) / kCarryGroup;
    const int64_t chunks = (width + kCarryChunk - 1) / kCarryChunk;
    for (int64_t g = 0; g < groups; ++g)
      for (int64_t c = 0; c < chunks; ++c) s.h_units.push_back(CarryUnit{t, (int32_t)g, (int32_t)c, 0});
    if (groups > 1) { s.group_pass = true; gsum += groups * width; }
    boff += nb[t];
    bits += (int64_t)nb[t] * words_of(C[t]);
    carry += rows * width;
  }
  s.h_soff[T] = (int32_t)soff[T];
  s.h_boff[T] = boff;
  s.B = boff;
  s.bits_words = bits;
  s.carry_words = carry;
  s.gsum_words = gsum;
  if (s.h_units.size() >= (size_t)1 << 31) return BW_EINVAL;
  s.n_units = (int32_t)s.h_units.size();
  // queue order: largest estimated block time first (longest-processing-time first).
  // A block is swept once per rank slice, so its work counts once per slice its
  // distinct keys are expected to need (at most its events, at most the domain).
  s.h_order.resize(s.B);
  std::vector<int64_t> bw(s.B);
  const int64_t cap = std::max<int64_t>(1, (int64_t)s.SL.cap32);
  for (int32_t t = 0; t < T; ++t) {
    const int64_t keys = std::min<int64_t>((int64_t)C[t], (eoff[t + 1] - eoff[t]) / nb[t] + 1);
    const int64_t slices = (keys + cap - 1) / cap;
    for (int32_t i = 0; i < nb[t]; ++i) bw[s.h_boff[t] + i] = W[t] / nb[t] * slices;
  }
  std::iota(s.h_order.begin(), s.h_order.end(), 0);
  std::stable_sort(s.h_order.begin(), s.h_order.end(), [&](int32_t a, int32_t b) { return bw[a] > bw[b]; });
  return 0;
}

void pipe_layout(const PipeSpec& s, Layout& L) {
  const size_t S = (size_t)s.S, S2 = 2 * S, T = (size_t)s.T, B = (size_t)s.B;
  size_t o = 0;
  auto take = [&](int i, size_t bytes) { L.off[i] = o; o = align_up(o + bytes); };
  take(W_TSOFF, (T + 1) * 4);
  take(W_TEOFF, (T + 1) * 8);
  take(W_TQOFF, (T + 1) * 8);
  take(W_TC, T * 4);
  take(W_TBOFF, (T + 1) * 4);
  take(W_TBITS, T * 8);
  take(W_TCARRY, T * 8);
  take(W_TGSUM, T * 8);
  take(W_LASTQ, T * 4);
  const bool forest = !s.h_soff.empty();   // tables uploaded by pipe_bind (else written per launch)
  take(W_UNITS, forest ? (size_t)s.n_units * sizeof(CarryUnit) : 0);
  take(W_ORDER, forest ? B * 4 : 0);
  take(W_MISC, 256);
  take(W_EOFF, (S + 1) * 8);
  take(W_QOFF, (S + 1) * 8);
  take(W_GPAR, s.T > 1 ? S * 4 : 0);
  take(W_FORK, S * 4);
  take(W_NEXT, S * 4);
  take(W_CNT, S * 8);
  take(W_EHEAD, S * 4);
  take(W_XHEAD, S * 4);
  take(W_RANKA, S2 * 8);
  take(W_RANKB, 0);               // (list ranking runs in place)
  take(W_STEPS, S2 * 4);
  take(W_DESC, S2 * sizeof(StepDesc));
  take(W_TIN, 0);                 // (enter/exit partners replace tin/tout)
  take(W_TOUT, 0);
  take(W_WORK, S2 * 8);
  take(W_SCAN, scan_tmp_bytes(S2));
  take(W_BLOCKS, B * sizeof(BlockTab));
  take(W_BMODE, B * 4);
  take(W_BITS, (size_t)s.bits_words * 8);
  take(W_RLUT, ((size_t)s.bits_words + B) * 4);
  take(W_SLICES, B * kMaxSlices * sizeof(Slice));
  take(W_NSLICES, B * 4);
  take(W_CARRY, (size_t)s.carry_words * 8);
  take(W_GSUM, (size_t)s.gsum_words * 8);
  L.total = o;
}

static TreeTabs tree_tabs(const Layout& L, char* ws) {
  TreeTabs tt;
  tt.soff = reinterpret_cast<int32_t*>(ws + L.off[W_TSOFF]);
  tt.eoff = reinterpret_cast<int64_t*>(ws + L.off[W_TEOFF]);
  tt.qoff = reinterpret_cast<int64_t*>(ws + L.off[W_TQOFF]);
  tt.C = reinterpret_cast<uint32_t*>(ws + L.off[W_TC]);
  tt.boff = reinterpret_cast<int32_t*>(ws + L.off[W_TBOFF]);
  tt.bits = reinterpret_cast<int64_t*>(ws + L.off[W_TBITS]);
  tt.carry = reinterpret_cast<int64_t*>(ws + L.off[W_TCARRY]);
  tt.gsum = reinterpret_cast<int64_t*>(ws + L.off[W_TGSUM]);
  tt.last_q = reinterpret_cast<int32_t*>(ws + L.off[W_LASTQ]);
  return tt;
}

const int32_t* pipe_status_word(const PipeSpec& s, const void* workspace) {
  Layout L;
  pipe_layout(s, L);
  return reinterpret_cast<const int32_t*>(static_cast<const char*>(workspace) + L.off[W_MISC]) + M_STATUS;
}

// One-time (per device) shared-memory opt-in of the two big-smem kernels.
static int ensure_attrs() {
  static std::mutex mu;
  static bool done[64] = {false};
  int dev = 0;
  int rc = report(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  std::lock_guard<std::mutex> g(mu);
  if (dev >= 0 && dev < 64 && done[dev]) return 0;
  if ((rc = report(cudaFuncSetAttribute(k_prepare<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemLimit - 1024),
                   "smem attr")))
    return rc;
  if ((rc = report(cudaFuncSetAttribute(k_prepare<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemLimit - 1024),
                   "smem attr")))
    return rc;
  if ((rc = report(cudaFuncSetAttribute(k_sweep<TileNarrow>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kSmemLimit - 1024), "smem attr")))
    return rc;
  if ((rc = report(cudaFuncSetAttribute(k_sweep<TileWide>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kSmemLimit - 1024), "smem attr")))
    return rc;
  if ((rc = report(cudaFuncSetAttribute(k_sweep<TileNarrow512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kSmemLimit - 1024), "smem attr")))
    return rc;
  if ((rc = report(cudaFuncSetAttribute(k_sweep<TileSpec512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kSmemLimit - 1024), "smem attr")))
    return rc;
  if ((rc = report(cudaFuncSetAttribute(k_sweep<TileWide512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kSmemLimit - 1024), "smem attr")))
    return rc;
  if ((rc = report((cudaError_t)esweep_attrs(), "smem attr"))) return rc;
  if (dev >= 0 && dev < 64) done[dev] = true;
  return 0;
}

int pipe_bind(const PipeSpec& s, void* workspace, cudaStream_t st) {
  int rc = ensure_attrs();
  if (rc || s.h_soff.empty()) return rc;
  Layout L;
  pipe_layout(s, L);
  char* ws = static_cast<char*>(workspace);
  auto put = [&](int slot, const void* src, size_t bytes) -> int {
    if (!bytes) return 0;
    return report(cudaMemcpyAsync(ws + L.off[slot], src, bytes, cudaMemcpyHostToDevice, st), "table upload");
  };
  const size_t T = (size_t)s.T;
  if ((rc = put(W_TSOFF, s.h_soff.data(), (T + 1) * 4))) return rc;
  if ((rc = put(W_TEOFF, s.h_eoff.data(), (T + 1) * 8))) return rc;
  if ((rc = put(W_TQOFF, s.h_qoff.data(), (T + 1) * 8))) return rc;
  if ((rc = put(W_TC, s.h_C.data(), T * 4))) return rc;
  if ((rc = put(W_TBOFF, s.h_boff.data(), (T + 1) * 4))) return rc;
  if ((rc = put(W_TBITS, s.h_bits.data(), T * 8))) return rc;
  if ((rc = put(W_TCARRY, s.h_carry.data(), T * 8))) return rc;
  if ((rc = put(W_TGSUM, s.h_gsum.data(), T * 8))) return rc;
  if ((rc = put(W_UNITS, s.h_units.data(), s.h_units.size() * sizeof(CarryUnit)))) return rc;
  if ((rc = put(W_ORDER, s.h_order.data(), s.h_order.size() * 4))) return rc;
  return report(cudaStreamSynchronize(st), "table upload sync");
}

int pipe_enqueue(const PipeSpec& s, void* workspace, const int32_t* parent, const BwEvent* events,
                 const BwQuery* queries, int64_t* answers, cudaStream_t st, EventSet* timing, int* kernels_out) {
  // both sweeps stage events with 16-byte copies (cp.async, cp.async.bulk)
  if (s.E > 0 && (reinterpret_cast<uintptr_t>(events) & 15u) != 0) {
    std::fprintf(stderr, "bw replay: events must be 16-byte aligned (got %p)\n", static_cast<const void*>(events));
    return BW_EINVAL;
  }
  int rc = ensure_attrs();
  if (rc) return rc;
  Layout L;
  pipe_layout(s, L);
  char* ws = static_cast<char*>(workspace);
  auto at = [&](int slot) { return ws + L.off[slot]; };
  const TreeTabs tt = tree_tabs(L, ws);
  int32_t* misc = reinterpret_cast<int32_t*>(at(W_MISC));
  int32_t* status = misc + M_STATUS;
  int64_t* eoff = reinterpret_cast<int64_t*>(at(W_EOFF));
  int64_t* qoff = reinterpret_cast<int64_t*>(at(W_QOFF));
  int32_t* gpar = s.T > 1 ? reinterpret_cast<int32_t*>(at(W_GPAR)) : nullptr;
  int32_t* fork_head = reinterpret_cast<int32_t*>(at(W_FORK));
  int32_t* next_sib = reinterpret_cast<int32_t*>(at(W_NEXT));
  int64_t* cnt = reinterpret_cast<int64_t*>(at(W_CNT));
  int32_t* ehead = reinterpret_cast<int32_t*>(at(W_EHEAD));
  int32_t* xhead = reinterpret_cast<int32_t*>(at(W_XHEAD));
  uint64_t* rank_a = reinterpret_cast<uint64_t*>(at(W_RANKA));
  int32_t* partner = reinterpret_cast<int32_t*>(at(W_STEPS));
  StepDesc* desc = reinterpret_cast<StepDesc*>(at(W_DESC));
  int64_t* work = reinterpret_cast<int64_t*>(at(W_WORK));
  int64_t* scan_tmp = reinterpret_cast<int64_t*>(at(W_SCAN));
  BlockTab* blocks = reinterpret_cast<BlockTab*>(at(W_BLOCKS));
  int32_t* bmode = reinterpret_cast<int32_t*>(at(W_BMODE));
  const bool forest = !s.h_soff.empty();
  const CarryUnit* units = forest ? reinterpret_cast<const CarryUnit*>(at(W_UNITS)) : nullptr;
  const int32_t* order = forest ? reinterpret_cast<const int32_t*>(at(W_ORDER)) : nullptr;

  const int32_t S = s.S, T = s.T, B = s.B;
  const int grid = s.sms * 8;
  int kernels = 0;
  auto chk = [&](const char* what) { ++kernels; return report(cudaGetLastError(), what); };
  auto mark = [&](int i) { return timing ? report(cudaEventRecord(timing->ev[i], st), "event record") : 0; };
  if (timing) timing->chain = 0;
  if ((rc = mark(0))) return rc;

  // ---- 0/1. init + ingest
  k_init<<<(std::max(T, 16) + 255) / 256, 256, 0, st>>>(misc, tt, T, forest ? 0 : 1, S, s.E, s.Q, s.Cmax, s.nb1);
  if ((rc = chk("k_init"))) return rc;
  if (s.E > 0) {
    k_offsets<true><<<grid, 256, 0, st>>>(events, s.E, tt, T, S, eoff, status);
    if ((rc = chk("k_offsets(events)"))) return rc;
  } else {
    k_fill_i64<<<grid, 256, 0, st>>>(eoff, (int64_t)S + 1, 0);
    if ((rc = chk("k_fill(eoff)"))) return rc;
  }
  if (s.Q > 0) {
    k_offsets<false><<<grid, 256, 0, st>>>(queries, s.Q, tt, T, S, qoff, status);
    if ((rc = chk("k_offsets(queries)"))) return rc;
  } else {
    k_fill_i64<<<grid, 256, 0, st>>>(qoff, (int64_t)S + 1, 0);
    if ((rc = chk("k_fill(qoff)"))) return rc;
  }

  if ((rc = mark(1))) return rc;
  // ---- 2. linearise
  if ((rc = report(cudaMemsetAsync(fork_head, 0xFF, (size_t)S * 4, st), "memset"))) return rc;
  k_lin_children<<<grid, 256, 0, st>>>(parent, S, tt, T, gpar, fork_head, next_sib, s.chain_hint ? 1 : 0, status);
  if ((rc = chk("k_lin_children"))) return rc;
  const int32_t* gp = gpar ? gpar : parent;   // one tree: global = local ids
  k_lin_flags<<<grid, 256, 0, st>>>(gp, fork_head, S, cnt, status);
  if ((rc = chk("k_lin_flags"))) return rc;
  if ((rc = device_inclusive_scan_i64(cnt, S, scan_tmp, st, kernels))) return report((cudaError_t)rc, "scan");
  k_lin_heads<<<grid, 256, 0, st>>>(cnt, S, ehead, xhead, status);
  if ((rc = chk("k_lin_heads"))) return rc;
  k_lin_rank_init<<<grid, 256, 0, st>>>(cnt, ehead, xhead, gp, fork_head, next_sib, S, rank_a, status);
  if ((rc = chk("k_lin_rank_init"))) return rc;
  int32_t round = 0;
  for (int64_t span = 1; span < 2 * (int64_t)s.Smax; span <<= 1, ++round) {
    k_lin_round<<<grid, 256, 0, st>>>(rank_a, cnt, S, misc + M_ROUNDS, round, status);
    if ((rc = chk("k_lin_round"))) return rc;
  }
  const uint64_t* src = rank_a;
  k_lin_steps<<<grid, 256, 0, st>>>(src, cnt, ehead, xhead, S, tt, T, eoff, qoff, partner, desc, work, status);
  if ((rc = chk("k_lin_steps"))) return rc;

  if ((rc = mark(2))) return rc;
  // ---- 3. blocks
  if ((rc = device_inclusive_scan_i64(work, 2 * (int64_t)S, scan_tmp, st, kernels)))
    return report((cudaError_t)rc, "scan");
  k_blocks<<<(B + 127) / 128, 128, 0, st>>>(work, tt, T, B, blocks, status);
  if ((rc = chk("k_blocks"))) return rc;

  if ((rc = mark(3))) return rc;
  // ---- 4. prepare
  const SweepLayout& SL = s.SL;
  const size_t asmem = (size_t)SL.ww * 8 + ((size_t)SL.ww + 4) * 4 + 16;
  const size_t psmem = asmem + std::max(((size_t)SL.cap32 + 1) * 4, ((size_t)SL.cap64 + 1) * 8);
  PrepParams pp;
  pp.ev = events; pp.desc = desc; pp.partner = partner; pp.blocks = blocks;
  pp.order = order; pp.B = B; pp.ww = SL.ww; pp.cap32 = SL.cap32; pp.cap64 = SL.cap64;
  pp.bits = reinterpret_cast<uint64_t*>(at(W_BITS)); pp.rlut = reinterpret_cast<uint32_t*>(at(W_RLUT));
  pp.slices = reinterpret_cast<Slice*>(at(W_SLICES)); pp.nslices = reinterpret_cast<int32_t*>(at(W_NSLICES));
  pp.carry = reinterpret_cast<int64_t*>(at(W_CARRY)); pp.status = status; pp.bmode = bmode;
  pp.ticket = misc + M_PREP_TICKET;
  int occ_a = 0;
  if ((rc = report(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_a, k_prepare<0>, kPrepThreads, asmem),
                   "occupancy")))
    return rc;
  k_prepare<0><<<std::min(B, std::max(occ_a, 1) * s.sms), kPrepThreads, asmem, st>>>(pp);
  if ((rc = chk("k_prepare<0>"))) return rc;
  if (s.carry_words > 0) {   // some block hands a carry on
    pp.ticket = misc + M_PREPB_TICKET;
    k_prepare<1><<<std::min(B, 2 * s.sms), kPrepThreads, psmem, st>>>(pp);
    if ((rc = chk("k_prepare<1>"))) return rc;
  }

  if ((rc = mark(4))) return rc;
  // ---- 5. carry
  if (s.n_units > 0) {
    CarryParams cp;
    cp.carry = pp.carry; cp.gsum = reinterpret_cast<int64_t*>(at(W_GSUM)); cp.units = units;
    cp.chunks1 = (int32_t)(((int64_t)s.Cmax + 1 + kCarryChunk - 1) / kCarryChunk); cp.tt = tt; cp.status = status;
    if (s.group_pass) {
      k_carry_groups<<<s.n_units, kCarryChunk, 0, st>>>(cp);
      if ((rc = chk("k_carry_groups"))) return rc;
    }
    k_carry_apply<<<s.n_units, kCarryChunk, 0, st>>>(cp);
    if ((rc = chk("k_carry_apply"))) return rc;
  }

  if ((rc = mark(5))) return rc;
  // ---- 6. sweep
  if (s.Q > 0) {
    SweepParams sp;
    sp.ev = events; sp.qs = queries; sp.desc = desc; sp.blocks = blocks; sp.order = order; sp.B = B;
    sp.bits = pp.bits; sp.rlut = pp.rlut; sp.slices = pp.slices; sp.nslices = pp.nslices; sp.carry = pp.carry;
    sp.answers = answers; sp.status = status; sp.bmode = bmode; sp.ticket = misc + M_SWEEP_TICKET;
    const int sgrid = std::min(B, s.ctas_per_sm * s.sms);
    if (s.tile == kTileEulerId) {
      EsParams ep;
      ep.ev = reinterpret_cast<const uint4*>(events); ep.qs = queries; ep.desc = desc; ep.blocks = blocks;
      ep.order = order; ep.B = B; ep.cap32 = SL.cap32; ep.cap64 = SL.cap64;
      ep.bits = pp.bits; ep.rlut = pp.rlut; ep.slices = pp.slices; ep.nslices = pp.nslices; ep.carry = pp.carry;
      ep.answers = answers; ep.status = status; ep.bmode = bmode; ep.ticket = misc + M_SWEEP_TICKET;
      if ((rc = report((cudaError_t)esweep_launch(ep, std::min(B, s.sms), st), "k_esweep"))) return rc;
      ++kernels;
      if ((rc = mark(6))) return rc;
      if (kernels_out) *kernels_out = kernels;
      return 0;
    }
    switch (s.tile) {
      case kTileWideId: k_sweep<TileWide><<<sgrid, TileWide::kThreads, SL.bytes, st>>>(sp, SL); break;
      case kTileNarrow512Id:
        k_sweep<TileNarrow512><<<sgrid, TileNarrow512::kThreads, SL.bytes, st>>>(sp, SL);
        break;
      case kTileWide512Id: k_sweep<TileWide512><<<sgrid, TileWide512::kThreads, SL.bytes, st>>>(sp, SL); break;
      case kTileSpec512Id: k_sweep<TileSpec512><<<sgrid, TileSpec512::kThreads, SL.bytes, st>>>(sp, SL); break;
      default: k_sweep<TileNarrow><<<sgrid, TileNarrow::kThreads, SL.bytes, st>>>(sp, SL); break;
    }
    if ((rc = chk("k_sweep"))) return rc;
  }
  if ((rc = mark(6))) return rc;
  if (kernels_out) *kernels_out = kernels;
  return 0;
}

}  // namespace bw
