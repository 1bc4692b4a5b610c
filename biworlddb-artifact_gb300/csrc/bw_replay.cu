// bw_replay.cu -- GB300 (sm_103a) event-model version-tree replay.
//
// Pipeline enqueued by bw_replay_launch (one stream, no host round trip):
//
//   1. ingest    k_offsets       per-state [begin,end) ranges of the state-grouped
//                                event and query arrays, with input validation
//   2. linearise k_children ..   Euler tour of the version tree by list ranking
//                k_rank_*        (enter(v) applies v's events, exit(v) removes
//                k_steps         them: the reference's preorder apply/undo,
//                                batch_engine_v7.hpp:1021-1059, laid out flat)
//   3. blocks    k_work/scan     equal-work cut of the step sequence into state
//                k_bounds        blocks (batch_engine_v7.hpp:707-722 cuts equal
//                                state counts; here the cut follows events+queries)
//   4. prepare   k_prepare       per block: key bitmap + popcount rank table
//                                (the CSR rank-LUT of sparse_engine.hpp:70-102),
//                                smem-sized key slices, and the block's net key
//                                deltas as a dense key-prefix row
//   5. carry     k_carry_groups  column scan over blocks: carry prefix at every
//                k_carry_apply
//                                block start (batch_engine_v7.hpp:936-945, on the
//                                device instead of the host)
//   6. sweep     k_sweep         one CTA per block replays its steps from a zero
//                                local Fenwick tree in shared memory over the
//                                block's rank-compressed keys and answers every
//                                query as carry(hi)-carry(lo)+local(hi)-local(lo)
//                                (batch_engine_v7.hpp:849-961 fused)
//
// All arithmetic is int64 with two's-complement wrap (done in uint64), so any
// summation order gives the reference's bits.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <vector>

#include "bw_gpu.h"
#include "bw_common.cuh"

namespace bw {

// ------------------------------------------------------------------ constants
constexpr int kPrepThreads = 512;             // CTA width of the prepare kernel (two per SM)
constexpr int kWinBits = 18;                  // rank window: 2^18 keys per smem bitmap
constexpr int kWinWords = 1 << (kWinBits - 6);
constexpr int kMaxSlices = 64;                // key slices per block
constexpr int kSmemLimit = 232448;            // 227 KiB dynamic smem per CTA on sm_100/103
constexpr int kSmemPerSM = 233472;            // 228 KiB shared memory per SM

struct StepDesc {        // one Euler step, 24 bytes
  int64_t e0;            // first event of the node
  int64_t q0;            // first query of the node (enter steps)
  int32_t ne;            // event count
  int32_t nq;            // query count on enter, -1 on exit
};

struct Slice {           // contiguous key range with <= cap distinct block keys
  int32_t word_lo, word_hi;  // bitmap words [word_lo, word_hi)
  uint32_t rank_lo;          // block-local rank of the first key of the slice
  uint32_t n;                // distinct keys in the slice
};

struct Plan {            // device pointers carved from the workspace
  int64_t* eoff;         // S+1
  int64_t* qoff;         // S+1
  int32_t* first_child;  // S
  int32_t* next_sib;     // S
  uint64_t* rank_a;      // 2S  (next:int32 | dist:int32)
  uint64_t* rank_b;      // 2S
  int32_t* steps;        // 2S  (v: enter v, ~v: exit v)
  int32_t* tin;          // S   step index of enter(v)
  int32_t* tout;         // S   step index of exit(v) (INT32_MAX when not swept)
  int32_t* bmode;        // B   1 = the block's applied |delta| sum is < 2^31
  int64_t* gsum;         // ceil(B/16) x (C+1) carry group sums
  StepDesc* desc;        // 2S
  int64_t* work;         // 2S  inclusive work prefix
  int64_t* scan_tmp;     // scan partials
  int32_t* bounds;       // B+1
  int32_t* misc;         // [0] status, [1] last query step + 1, [2] chain flag
  uint64_t* bits;        // B * nwords
  uint32_t* rlut;        // B * (nwords + 1)
  Slice* slices;         // B * kMaxSlices
  int32_t* nslices;      // B
  int64_t* carry;        // B * (C + 1)
};

__device__ __forceinline__ void set_status(int32_t* st, int32_t code) { atomicCAS(st, 0, code); }

// ------------------------------------------------------------------ 1. ingest
// Per-state [off[s], off[s+1]) ranges of a state-grouped array of records whose
// first field is the u32 state; checks grouping and key/interval ranges.
template <bool kEvents>
__global__ void k_offsets(const void* items, int64_t n, int32_t S, uint32_t C, int64_t* off,
                          int32_t* status) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    uint32_t s, prev;
    if (kEvents) {
      const BwEvent* ev = static_cast<const BwEvent*>(items);
      s = ev[i].state;
      prev = i ? ev[i - 1].state : 0u;
      if (ev[i].key >= C) set_status(status, BW_STATUS_EVENT_KEY_RANGE);
    } else {
      const BwQuery* qs = static_cast<const BwQuery*>(items);
      s = qs[i].state;
      prev = i ? qs[i - 1].state : 0u;
      if (qs[i].lo > C || qs[i].hi > C) set_status(status, BW_STATUS_QUERY_RANGE);
    }
    if (s >= (uint32_t)S) { set_status(status, BW_STATUS_STATE_RANGE); continue; }
    if (i && s < prev) {
      set_status(status, kEvents ? BW_STATUS_EVENTS_UNSORTED : BW_STATUS_QUERIES_UNSORTED);
      continue;
    }
    // off[x] = i for every state x in (prev, s] (x = 0..s for the first item)
    for (uint32_t x = i ? prev + 1 : 0u; x <= s; ++x) off[x] = i;
    if (i == n - 1)
      for (int64_t x = (int64_t)s + 1; x <= S; ++x) off[x] = n;
  }
}

__global__ void k_init_misc(int32_t* misc) {
  if (threadIdx.x < 4) misc[threadIdx.x] = threadIdx.x == 2 ? 1 : 0;
}

__global__ void k_fill_i64(int64_t* p, int64_t n, int64_t v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

// ------------------------------------------------------------------ 2. linearise
// Unordered child lists by atomic exchange: first_child[p] heads a singly linked
// sibling list.  Child order does not change any answer (a state's answer only
// depends on its root path), only the step order.
__global__ void k_children(const int32_t* parent, int32_t S, int32_t* first_child, int32_t* next_sib,
                           int32_t* status, int32_t* chain_flag) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < S; v += gridDim.x * blockDim.x) {
    const int32_t p = parent[v];
    if (v == 0) {
      if (p != -1) set_status(status, BW_STATUS_BAD_PARENT);
      next_sib[0] = -1;
      continue;
    }
    if (p < 0 || p >= v) { set_status(status, BW_STATUS_BAD_PARENT); next_sib[v] = -1; continue; }
    if (p != v - 1) atomicExch(chain_flag, 0);
    next_sib[v] = atomicExch(&first_child[p], v);
  }
}

// Euler circuit successor of arc x (enter(v) = 2v, exit(v) = 2v+1), packed with
// the distance-to-end counter used by list ranking.
__device__ __forceinline__ uint64_t pack_rank(int32_t next, uint32_t dist) {
  return ((uint64_t)(uint32_t)next << 32) | dist;
}
__global__ void k_rank_init(const int32_t* parent, const int32_t* first_child, const int32_t* next_sib,
                            int32_t S, uint64_t* r, const int32_t* status) {
  if (*status) return;  // a rejected parent array must not drive any index below
  const int64_t n = 2 * (int64_t)S;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = (int32_t)(x >> 1);
    int32_t nx;
    if ((x & 1) == 0) {
      const int32_t c = first_child[v];
      nx = c >= 0 ? 2 * c : 2 * v + 1;
    } else if (v == 0) {
      nx = -1;
    } else {
      const int32_t s = next_sib[v];
      nx = s >= 0 ? 2 * s : 2 * parent[v] + 1;
    }
    r[x] = pack_rank(nx, 1u);
  }
}
// One Wyllie pointer-jumping round: dist(x) += dist(next(x)), next(x) = next(next(x)).
__global__ void k_rank_round(const uint64_t* __restrict__ src, uint64_t* __restrict__ dst, int64_t n,
                             const int32_t* status) {
  if (*status) return;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t a = src[x];
    const int32_t nx = (int32_t)(a >> 32);
    if (nx < 0) { dst[x] = a; continue; }
    const uint64_t b = src[nx];
    dst[x] = (b & 0xFFFFFFFF00000000ull) | (uint32_t)((uint32_t)a + (uint32_t)b);
  }
}
// Step sequence and per-step descriptors; records the last step that answers
// queries (steps after it cannot change any answer and are trimmed).
__global__ void k_steps(const uint64_t* r, int32_t S, const int64_t* eoff, const int64_t* qoff,
                        int32_t* steps, StepDesc* desc, int32_t* last_q, int32_t* tin, int32_t* tout,
                        const int32_t* status) {
  if (*status) return;  // offsets or ranks may be incomplete after an input error
  const int64_t n = 2 * (int64_t)S;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pos = n - (int64_t)(uint32_t)r[x];
    const int32_t v = (int32_t)(x >> 1);
    const bool enter = (x & 1) == 0;
    steps[pos] = enter ? v : ~v;
    (enter ? tin : tout)[v] = (int32_t)pos;
    StepDesc d;
    d.e0 = eoff[v];
    d.ne = (int32_t)(eoff[v + 1] - eoff[v]);
    d.q0 = qoff[v];
    d.nq = enter ? (int32_t)(qoff[v + 1] - qoff[v]) : -1;
    desc[pos] = d;
    if (enter && d.nq > 0) atomicMax(last_q, (int32_t)pos + 1);
  }
}
// Parent check for callers that assert a chain.
__global__ void k_check_chain(const int32_t* parent, int32_t S, int32_t* status) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < S; v += gridDim.x * blockDim.x)
    if (parent[v] != v - 1) set_status(status, BW_STATUS_BAD_PARENT);
}
// Chain layout without list ranking: step v enters state v.
__global__ void k_steps_chain(int32_t S, const int64_t* eoff, const int64_t* qoff, int32_t* steps,
                              StepDesc* desc, int32_t* last_q, int32_t* tin, int32_t* tout,
                              const int32_t* status) {
  if (*status) return;
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < S; v += gridDim.x * blockDim.x) {
    steps[v] = v;
    tin[v] = v;
    tout[v] = 0x7FFFFFFF;  // a chain never leaves a state before the last query
    StepDesc d;
    d.e0 = eoff[v];
    d.ne = (int32_t)(eoff[v + 1] - eoff[v]);
    d.q0 = qoff[v];
    d.nq = (int32_t)(qoff[v + 1] - qoff[v]);
    desc[v] = d;
    if (d.nq > 0) atomicMax(last_q, v + 1);
  }
}

// ------------------------------------------------------------------ 3. blocks
constexpr int64_t kStepCost = 64;   // fixed cost of a step (two CTA barriers) in event units
constexpr int64_t kQueryCost = 2;   // a query is two prefix probes

// Work of each step (0 past the last query step, so the cut balances only the
// steps that are swept).
__global__ void k_work(const StepDesc* desc, int64_t n, const int32_t* last_q, int64_t* work) {
  const int64_t lim = last_q[-1] ? 0 : *last_q;  // last_q[-1] is the status word
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const StepDesc d = desc[t];
    work[t] = t < lim ? kStepCost + d.ne + (d.nq > 0 ? kQueryCost * d.nq : 0) : 0;
  }
}
// bounds[b] = number of steps whose inclusive work prefix is <= b*W/B.
__global__ void k_bounds(const int64_t* work, int64_t T, int32_t B, int32_t* bounds) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b > B) return;
  if (T == 0) { bounds[b] = 0; return; }
  const int64_t W = work[T - 1];
  if (b == B) { bounds[b] = (int32_t)T; return; }
  const int64_t lim = (int64_t)(((__int128)W * b) / B);
  int64_t lo = 0, hi = T;  // first index with work > lim
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (work[mid] <= lim) lo = mid + 1; else hi = mid;
  }
  bounds[b] = (int32_t)lo;
}

// ------------------------------------------------------------------ 4. prepare
struct PrepParams {
  const BwEvent* ev;
  const StepDesc* desc;
  const int32_t* steps;
  const int32_t* tin;
  const int32_t* tout;
  const int32_t* bounds;
  int32_t nwords;
  int32_t ww;              // rank-table window in bitmap words (<= kWinWords)
  uint32_t C;
  uint32_t cap32, cap64;   // slice rank capacity with int32 / int64 sweep nodes
  uint64_t* bits;
  uint32_t* rlut;
  Slice* slices;
  int32_t* nslices;
  int64_t* carry;
  int32_t* status;
  int32_t* bmode;
};

// Visit the (key, signed delta) of the block's steps that matter: mode 0 (key
// set) skips exits of nodes entered in the block (their keys come with the
// enter, flagged by `twice` since the sweep applies them twice); mode 1 (net
// deltas) also skips enters of nodes that exit in the block, since the two cancel.  Warps take steps round robin, lanes take events; loop
// bounds are warp-uniform and f is called by all 32 lanes (valid marks real
// events), so f may use warp-collective operations.
template <typename F>
__device__ __forceinline__ void for_block_events(const PrepParams& p, int32_t t0, int32_t t1, int mode, F&& f) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int32_t t = t0 + warp; t < t1; t += nw) {
    const StepDesc d = p.desc[t];
    const bool neg = d.nq < 0;
    const int32_t x = p.steps[t];
    const int32_t u = x >= 0 ? x : ~x;
    const bool exits_here = !neg && p.tout[u] < t1;
    if (neg) {
      if (p.tin[u] >= t0) continue;         // entered in this block: keys known, deltas cancel
    } else if (mode == 1 && exits_here) {
      continue;                             // leaves within this block: net zero
    }
    for (int32_t i0 = 0; i0 < d.ne; i0 += 32) {
      const int32_t i = i0 + lane;
      const bool valid = i < d.ne;
      uint32_t k = 0;
      uint64_t v = 0;
      if (valid) {
        const BwEvent e = p.ev[d.e0 + i];
        k = e.key;
        v = neg ? (uint64_t)0 - (uint64_t)e.delta : (uint64_t)e.delta;
      }
      f(k, v, valid, exits_here);
    }
  }
}

__global__ void __launch_bounds__(kPrepThreads, 2) k_prepare(PrepParams p) {
  if (*p.status) return;  // bounds/descriptors are not trustworthy after an input error
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* sbits = reinterpret_cast<uint64_t*>(smem);                    // ww words
  uint32_t* srl = reinterpret_cast<uint32_t*>(sbits + p.ww);              // ww + 2
  // histogram: int32 per rank when the block's nodes are int32 (exact, same
  // bound), int64 otherwise; both fit the same bytes (cap32 ~ 2 * cap64)
  unsigned char* hist_raw = reinterpret_cast<unsigned char*>(srl + p.ww + 2 + (p.ww & 1));  // 8-byte aligned
  __shared__ uint64_t s_wsum[kPrepThreads / 32];
  __shared__ int32_t s_nsl;
  __shared__ int32_t s_mode;

  const int b = blockIdx.x;
  const int32_t t0 = p.bounds[b], t1 = p.bounds[b + 1];
  uint64_t* gbits = p.bits + (size_t)b * p.nwords;
  uint32_t* grl = p.rlut + (size_t)b * (p.nwords + 1);
  Slice* gsl = p.slices + (size_t)b * kMaxSlices;
  if (threadIdx.x == 0) s_nsl = 0;
  uint32_t rank_base = 0;
  uint64_t mass = 0;  // per-thread partial of the block's applied |delta| sum

  // ---- pass A: per window, key bitmap -> rank table -> slices
  for (int32_t w0 = 0; w0 < p.nwords; w0 += p.ww) {
    const int32_t ww = min(p.ww, p.nwords - w0);
    for (int i = threadIdx.x; i < ww; i += blockDim.x) sbits[i] = 0;
    __syncthreads();
    const uint32_t klo = (uint32_t)w0 << 6;
    const uint32_t khi = (uint32_t)imin64((int64_t)(w0 + ww) << 6, (int64_t)p.C);
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
      int32_t ns = s_nsl;
      int32_t lo = 0;
      while (lo < ww) {
        int32_t hi = lo + 1;
        while (hi < ww && srl[hi + 1] - srl[lo] <= cap) ++hi;
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
    grl[p.nwords] = rank_base;
    if (s_nsl > kMaxSlices) set_status(p.status, BW_STATUS_TOO_MANY_SLICES);
    p.nslices[b] = min(s_nsl, kMaxSlices);
    p.bmode[b] = s_mode;
  }
  __syncthreads();
  const int32_t nsl = min(s_nsl, kMaxSlices);

  // ---- pass B: per slice, net key deltas of the block -> dense key-prefix row
  int64_t* row = p.carry + (size_t)b * ((size_t)p.C + 1);
  const bool h32 = s_mode != 0;
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
    const uint32_t khi = (uint32_t)imin64((int64_t)s.word_hi << 6, (int64_t)p.C);
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
  if (threadIdx.x == 0) row[p.C] = (int64_t)base;
}

// ------------------------------------------------------------------ 5. carry
// In place: row b becomes the exclusive sum over blocks < b of the per-block
// key-prefix rows, i.e. the key prefix of the state vector at block b's start.
// Two passes over groups of kCarryGroup rows, so that every (group, column) pair
// is its own thread and all rows of a group are loaded at once: group sums, then
// each group adds the sums of the groups before it and writes its rows.
constexpr int kCarryGroup = 16;

__global__ void k_carry_groups(const int64_t* carry, int32_t B, int64_t width, int64_t* gsum,
                               const int32_t* status) {
  if (*status) return;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t g = blockIdx.y, r0 = g * kCarryGroup;
  if (k >= width) return;
  const int64_t* p = carry + (size_t)r0 * width + k;
  const int32_t n = min(kCarryGroup, B - r0);
  uint64_t v[kCarryGroup];
#pragma unroll
  for (int i = 0; i < kCarryGroup; ++i) v[i] = i < n ? (uint64_t)p[(size_t)i * width] : 0;
  uint64_t sum = 0;
#pragma unroll
  for (int i = 0; i < kCarryGroup; ++i) sum += v[i];
  gsum[(size_t)g * width + k] = (int64_t)sum;
}

__global__ void k_carry_apply(int64_t* carry, int32_t B, int64_t width, const int64_t* gsum,
                              const int32_t* status) {
  if (*status) return;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t g = blockIdx.y, r0 = g * kCarryGroup;
  if (k >= width) return;
  int64_t* p = carry + (size_t)r0 * width + k;
  const int32_t n = min(kCarryGroup, B - r0);
  uint64_t v[kCarryGroup];
#pragma unroll
  for (int i = 0; i < kCarryGroup; ++i) v[i] = i < n ? (uint64_t)p[(size_t)i * width] : 0;
  uint64_t run = 0;
  for (int32_t j = 0; j < g; ++j) run += (uint64_t)gsum[(size_t)j * width + k];
#pragma unroll
  for (int i = 0; i < kCarryGroup; ++i) {
    if (i < n) p[(size_t)i * width] = (int64_t)run;
    run += v[i];
  }
}

// ------------------------------------------------------------------ 6. sweep
struct SweepParams {
  const BwEvent* ev;
  const BwQuery* qs;
  const StepDesc* desc;
  const int32_t* bounds;
  const uint64_t* bits;
  const uint32_t* rlut;
  const Slice* slices;
  const int32_t* nslices;
  const int64_t* carry;
  int64_t* answers;
  int32_t nwords;
  uint32_t C;
  const int32_t* status;
  const int32_t* bmode;   // per block: 1 = int32 Fenwick nodes are exact, 0 = int64
};

// The sweep keeps the block-local prefix structure in shared memory as chunks of
// kChunk ranks: a Fenwick tree inside every chunk (levels below the chunk top),
// the chunk totals T[h], and per-warp copies of the exclusive prefix of the chunk
// totals, rebuilt by each warp before every probe phase.  An update touches only
// its own chunk; a probe reads the prefix copy plus <= kChunkLevels nodes.
//
// Staging is per thread: thread i prefetches, with cp.async, event i and query i
// of the step kAhead ahead into its own slots and waits for them with its own
// wait_group, so staging needs no barrier.  Barriers only order the Fenwick: after
// the updates of a step that has queries (probes must see them) and after its
// probes (the next updates must not run under them).  Steps without queries (the
// exits of a tree walk, states without queries) run back to back with none.
// Step descriptors come from a shared ring refilled every kDescRefill steps.
constexpr int kSweepThreads = 256;
constexpr int kSweepWarps = kSweepThreads / 32;
constexpr int kChunk = 256;
constexpr int kChunkBits = 8;
constexpr int kChunkLevels = 8;            // Fenwick levels inside a chunk (below its top)
constexpr int kChunkStride = 257;          // words per chunk: odd stride spreads node x of
                                           // different chunks over different banks
constexpr int kMaxChunks = 128;
constexpr int kAhead = 3;                  // steps prefetched ahead of the one processed
constexpr int kSlots = kAhead + 1;         // per-thread prefetch slots
constexpr int kDescRing = 64;              // step descriptors held in shared memory
constexpr int kDescRefill = 32;            // ring refill period in steps
constexpr int kRebuildPer = 5;             // chunk totals per lane in a prefix rebuild

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

// Shared-memory layout of the sweep for a rank-table window of `ww` words.  The
// Fenwick nodes of a block are int32 when the block's applied |delta| sum is below
// 2^31 (every node value is a sum of a subset of those deltas, so it cannot
// overflow) and int64 otherwise; the same byte budget then holds twice as many
// int32 chunks.  Chunk totals and prefixes are always int64.
struct SweepLayout {
  int32_t ww;             // rank-table words reserved
  int32_t nch32, nch64;   // chunk capacity with int32 / int64 nodes
  uint32_t cap32, cap64;  // rank capacities
  size_t off_rl, off_fine, off_T, off_P, off_desc, off_ev, off_q, bytes;
};
__host__ __device__ inline SweepLayout sweep_layout(int32_t nwords, size_t budget) {
  SweepLayout L;
  L.ww = nwords < kWinWords ? nwords : kWinWords;
  auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
  const size_t fixed = al((size_t)L.ww * 8) + al(((size_t)L.ww + 2) * 4) + al(sizeof(StepDesc) * kDescRing) +
                       (size_t)kSlots * kSweepThreads * 16 + al((size_t)kSlots * kSweepThreads * 12) +
                       (size_t)kSweepWarps * (kMaxChunks + 1) * 8 + 128;
  const size_t per32 = (size_t)kChunkStride * 4 + 8;  // int32 nodes + chunk total
  int32_t n32 = budget > fixed ? (int32_t)((budget - fixed) / per32) : 0;
  if (n32 > kMaxChunks) n32 = kMaxChunks;
  L.nch32 = n32;
  L.nch64 = (int32_t)(((size_t)n32 * kChunkStride * 4) / ((size_t)kChunkStride * 8));
  L.cap32 = (uint32_t)L.nch32 * kChunk;
  L.cap64 = (uint32_t)L.nch64 * kChunk;
  size_t o = al((size_t)L.ww * 8);
  L.off_rl = o;   o = al(o + ((size_t)L.ww + 2) * 4);
  L.off_fine = o; o = al(o + (size_t)n32 * kChunkStride * 4);
  L.off_T = o;    o = al(o + (size_t)n32 * 8);
  L.off_P = o;    o = al(o + (size_t)kSweepWarps * (kMaxChunks + 1) * 8);
  L.off_desc = o; o = al(o + sizeof(StepDesc) * kDescRing);
  L.off_ev = o;   o = al(o + (size_t)kSlots * kSweepThreads * 16);
  L.off_q = o;    o = al(o + (size_t)kSlots * kSweepThreads * 12);
  L.bytes = o;
  return L;
}

// Point update of one chunk: the Fenwick nodes above local index l (l in
// 1..kChunk, stopping below the chunk top, at most kChunkLevels nodes) and the
// chunk total.  int64 nodes use exact 32-bit-pair atomics with all low-word
// atomics issued before any high-word one (one shared-atomic round trip);
// int32 nodes take plain 32-bit atomics with no return value.
template <typename Node>
__device__ __forceinline__ void chunk_add(Node* f, unsigned long long* tot, uint32_t l, uint64_t v) {
  const unsigned lo = (unsigned)v, hi = (unsigned)(v >> 32);
  unsigned* tw = reinterpret_cast<unsigned*>(tot);
  if constexpr (sizeof(Node) == 4) {
    uint32_t x = l;
#pragma unroll
    for (int lv = 0; lv < kChunkLevels; ++lv) {
      if (x < (uint32_t)kChunk) atomicAdd(reinterpret_cast<unsigned*>(f) + x, lo);
      x += x & (0u - x);
    }
    shared_add_u64(tot, v);
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

template <typename Node>
__device__ __forceinline__ void sweep_block(const SweepParams& p, const SweepLayout& L, unsigned char* smem) {
  uint64_t* sbits = reinterpret_cast<uint64_t*>(smem);
  uint32_t* srl = reinterpret_cast<uint32_t*>(smem + L.off_rl);
  Node* fine = reinterpret_cast<Node*>(smem + L.off_fine);
  unsigned long long* T = reinterpret_cast<unsigned long long*>(smem + L.off_T);
  StepDesc* ring = reinterpret_cast<StepDesc*>(smem + L.off_desc);
  unsigned char* evs = smem + L.off_ev;   // [slot][thread] 16 B
  unsigned char* qss = smem + L.off_q;    // [slot][thread] 12 B
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  unsigned long long* Pw = reinterpret_cast<unsigned long long*>(smem + L.off_P) + (size_t)warp * (kMaxChunks + 1);

  const int b = blockIdx.x;
  const int32_t t0 = p.bounds[b], t1 = p.bounds[b + 1];
  if (t0 >= t1) return;
  const int32_t nsl = p.nslices[b];
  const uint64_t* gbits = p.bits + (size_t)b * p.nwords;
  const uint32_t* grl = p.rlut + (size_t)b * (p.nwords + 1);
  const int64_t* crow = p.carry + (size_t)b * ((size_t)p.C + 1);
  unsigned char* my_ev = evs + 16 * tid;
  unsigned char* my_q = qss + 12 * tid;

  auto desc_at = [&](int32_t t) -> StepDesc {
    StepDesc d;
    if (t < t1) d = p.desc[t];
    else { d.e0 = 0; d.q0 = 0; d.ne = 0; d.nq = -1; }
    return d;
  };
  // Prefetch this thread's event and query of step t into slot t % kSlots.
  auto stage_own = [&](int32_t t) {
    const StepDesc d = ring[(t - t0) % kDescRing];
    const int sl = (t - t0) % kSlots;
    if (tid < d.ne) cp_async16(my_ev + (size_t)sl * kSweepThreads * 16, p.ev + d.e0 + tid);
    if (tid < d.nq) {
      const uint32_t* src = reinterpret_cast<const uint32_t*>(p.qs + d.q0 + tid);
      unsigned char* dq = my_q + (size_t)sl * kSweepThreads * 12;
      cp_async4(dq, src);
      cp_async4(dq + 4, src + 1);
      cp_async4(dq + 8, src + 2);
    }
    cp_async_commit();
  };

  for (int32_t si = 0; si < nsl; ++si) {
    const Slice s = p.slices[(size_t)b * kMaxSlices + si];
    const int32_t nwd = s.word_hi - s.word_lo;
    const uint32_t klo = (uint32_t)s.word_lo << 6;
    const uint32_t khi = (uint32_t)imin64((int64_t)s.word_hi << 6, (int64_t)p.C);
    const uint32_t nch = (s.n + kChunk - 1) / kChunk;
    const bool first = si == 0;
    for (int i = tid; i < nwd; i += kSweepThreads) {
      sbits[i] = gbits[s.word_lo + i];
      srl[i] = grl[s.word_lo + i] - s.rank_lo;
    }
    for (uint32_t i = tid; i < nch * kChunkStride; i += kSweepThreads) fine[i] = 0;
    for (uint32_t i = tid; i < nch; i += kSweepThreads) T[i] = 0;
    for (int i = tid; i < kDescRing; i += kSweepThreads) ring[i] = desc_at(t0 + i);
    __syncthreads();

    // prologue: own items of the first kAhead steps; step t0 landed before its carries
    for (int u = 0; u < kAhead; ++u) stage_own(t0 + u);
    cp_async_wait<kAhead - 1>();
    uint64_t ca_lo = 0, ca_hi = 0, cb_lo = 0, cb_hi = 0;
    if (first) {
      const StepDesc d = ring[0];
      const uint32_t* q = reinterpret_cast<const uint32_t*>(my_q);
      if (tid < d.nq && q[2] > q[1]) {
        ca_lo = (uint64_t)__ldg(crow + q[1]);
        ca_hi = (uint64_t)__ldg(crow + q[2]);
      }
    }
    bool dirty = true;

    // One step.  The carries of step t arrive in (c_lo, c_hi); those of step t + 1
    // are loaded into (n_lo, n_hi); the loop alternates the pairs statically.
    auto step = [&](int32_t t, uint64_t& c_lo, uint64_t& c_hi, uint64_t& n_lo, uint64_t& n_hi) {
      const int32_t rel = t - t0;
      if (rel >= kDescRefill && rel % kDescRefill == 0) {
        // ring entries of steps rel-32..rel-1 are done; refill them with rel+32..rel+63
        __syncthreads();
        for (int i = tid; i < kDescRefill; i += kSweepThreads)
          ring[(rel + kDescRefill + i) % kDescRing] = desc_at(t + kDescRefill + i);
        __syncthreads();
      }
      const StepDesc d = ring[rel % kDescRing];
      stage_own(t + kAhead);
      cp_async_wait<kAhead - 1>();   // own items of steps t and t + 1 have landed
      const int sl = rel % kSlots;
      if (first && t + 1 < t1) {
        const StepDesc d1 = ring[(rel + 1) % kDescRing];
        const uint32_t* q = reinterpret_cast<const uint32_t*>(my_q + (size_t)((rel + 1) % kSlots) * kSweepThreads * 12);
        if (tid < d1.nq && q[2] > q[1]) {
          n_lo = (uint64_t)__ldg(crow + q[1]);
          n_hi = (uint64_t)__ldg(crow + q[2]);
        }
      }
      // updates of step t (exit steps remove the node's events)
      if (s.n && d.ne > 0) {
        const bool neg = d.nq < 0;
        for (int i = tid; i < d.ne; i += kSweepThreads) {
          uint32_t k;
          uint64_t v;
          if (i < kSweepThreads) {
            const BwEvent* e = reinterpret_cast<const BwEvent*>(my_ev + (size_t)sl * kSweepThreads * 16);
            k = e->key;
            v = (uint64_t)e->delta;
          } else {
            const BwEvent e = p.ev[d.e0 + i];
            k = e.key;
            v = (uint64_t)e.delta;
          }
          if (k >= klo && k < khi) {
            if (neg) v = (uint64_t)0 - v;
            const uint32_t r = local_rank(sbits, srl, k - klo);
            chunk_add<Node>(fine + (size_t)(r >> kChunkBits) * kChunkStride, T + (r >> kChunkBits),
                            (r & (kChunk - 1u)) + 1u, v);
          }
        }
        dirty = true;
      }
      if (d.nq <= 0) return;  // no probes: the next step's updates may follow at once
      __syncthreads();         // every update of steps <= t is applied
      if (dirty) {
        // this warp's copy of the exclusive prefix of the chunk totals
        const uint32_t per = ((nch + 31) / 32) | 1u;  // odd: lanes hit different banks
        const uint32_t lo = lane * per;
        uint64_t tv[kRebuildPer];
        uint64_t sum = 0;
#pragma unroll
        for (int i = 0; i < kRebuildPer; ++i) {
          tv[i] = ((uint32_t)i < per && lo + i < nch) ? T[lo + i] : 0;
          sum += tv[i];
        }
        uint64_t x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
          if (lane >= o) x += y;
        }
        uint64_t run = x - sum;
#pragma unroll
        for (int i = 0; i < kRebuildPer; ++i) {
          if ((uint32_t)i < per && lo + i < nch) Pw[lo + i] = run;
          run += tv[i];
        }
        if (lane == 31) Pw[nch] = x;
        __syncwarp();
      }
      dirty = false;
      const uint32_t* q = reinterpret_cast<const uint32_t*>(my_q + (size_t)sl * kSweepThreads * 12);
      for (int j = tid; j < d.nq; j += kSweepThreads) {
        uint32_t lo, hi;
        uint64_t acc = 0;
        if (j < kSweepThreads) {
          lo = q[1];
          hi = q[2];
          if (first) acc = c_hi - c_lo;
        } else {
          const BwQuery qq = p.qs[d.q0 + j];
          lo = qq.lo;
          hi = qq.hi;
          if (first && hi > lo) acc = (uint64_t)__ldg(crow + hi) - (uint64_t)__ldg(crow + lo);
        }
        int64_t* out = p.answers + d.q0 + j;
        if (hi <= lo) {
          if (first) *out = 0;
          continue;
        }
        acc += slice_prefix2(fine, Pw, s.n, sbits, srl, klo, khi, hi);
        acc -= slice_prefix2(fine, Pw, s.n, sbits, srl, klo, khi, lo);
        *out = first ? (int64_t)acc : (int64_t)((uint64_t)*out + acc);
      }
      __syncthreads();  // probes done before the next step's updates
    };
    for (int32_t t = t0; t < t1; t += 2) {
      step(t, ca_lo, ca_hi, cb_lo, cb_hi);
      if (t + 1 < t1) step(t + 1, cb_lo, cb_hi, ca_lo, ca_hi);
    }
    cp_async_wait<0>();
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kSweepThreads, 2) k_sweep(SweepParams p, SweepLayout L) {
  extern __shared__ __align__(16) unsigned char smem[];
  if (*p.status) return;  // never index with descriptors of rejected input
  if (p.bmode[blockIdx.x]) sweep_block<unsigned>(p, L, smem);
  else sweep_block<unsigned long long>(p, L, smem);
}

// ------------------------------------------------------------------ host side
static inline size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

struct Layout {
  size_t off[24];
  size_t total;
};

static int32_t pick_blocks(const BwReplayArgs* a, int sms) {
  if (a->blocks > 0) return a->blocks;
  const int64_t work = a->n_events * 2 + a->n_queries * kQueryCost + (int64_t)a->n_states * 2 * kStepCost;
  int64_t B = 2 * (int64_t)sms;                    // two sweep CTAs per SM hide each other's latency
  const int64_t min_work = 65536;                  // below this a block is launch-dominated
  if (work / min_work < B) B = work / min_work;
  const double carry_budget = 4.0e9;               // bytes of dense carry rows
  const int64_t by_mem = (int64_t)(carry_budget / (8.0 * ((double)a->n_keys + 1.0)));
  if (by_mem < B) B = by_mem;
  if (B < 1) B = 1;
  return (int32_t)B;
}

static int32_t words_of(uint32_t C) { return (int32_t)(((uint64_t)C + 63) >> 6); }

static void layout(const BwReplayArgs* a, int32_t B, Layout& L) {
  const size_t S = (size_t)a->n_states, S2 = 2 * S;
  const size_t nw = (size_t)words_of(a->n_keys);
  size_t o = 0;
  auto take = [&](int i, size_t bytes) { L.off[i] = o; o = align_up(o + bytes); };
  take(0, (S + 1) * 8);            // eoff
  take(1, (S + 1) * 8);            // qoff
  take(2, S * 4);                  // first_child
  take(3, S * 4);                  // next_sib
  take(4, S2 * 8);                 // rank_a
  take(5, S2 * 8);                 // rank_b
  take(6, S2 * 4);                 // steps
  take(7, S2 * sizeof(StepDesc));  // desc
  take(8, S2 * 8);                 // work
  take(9, scan_tmp_bytes(S2));     // scan partials
  take(10, ((size_t)B + 1) * 4);   // bounds
  take(11, 64);                    // misc
  take(12, (size_t)B * nw * 8);    // bits
  take(13, (size_t)B * (nw + 1) * 4);  // rlut
  take(14, (size_t)B * kMaxSlices * sizeof(Slice));
  take(15, (size_t)B * 4);         // nslices
  take(16, (size_t)B * ((size_t)a->n_keys + 1) * 8);  // carry rows
  take(17, S * 4);                 // tin
  take(18, S * 4);                 // tout
  take(19, (size_t)B * 4);         // bmode
  take(20, (size_t)((B + kCarryGroup - 1) / kCarryGroup) * ((size_t)a->n_keys + 1) * 8);  // carry group sums
  L.total = o;
}

// Prepare smem: window bitmap + rank table + histogram (int32 x cap32+1 or
// int64 x cap64+1, whichever is larger).
static size_t prepare_smem(int32_t ww, uint32_t cap32, uint32_t cap64) {
  const size_t h32 = ((size_t)cap32 + 1) * 4, h64 = ((size_t)cap64 + 1) * 8;
  return (size_t)ww * 8 + ((size_t)ww + 4) * 4 + (h32 > h64 ? h32 : h64) + 16;
}

struct LastInfo { int32_t kernels = 0, blocks = 0; };
static std::mutex g_info_mu;
static LastInfo g_last;

// Stage timing (BW_REPLAY_TIMING): one set of BW_STAGE_COUNT+1 events per timed
// launch since the last reset; sets are kept for reuse across runs.
struct EventSet { cudaEvent_t ev[BW_STAGE_COUNT + 1]; };
static std::vector<EventSet> g_sets;
static size_t g_sets_used = 0;

static int report(cudaError_t e, const char* what) {
  if (e != cudaSuccess) std::fprintf(stderr, "bw_replay: %s failed: %s\n", what, cudaGetErrorString(e));
  return (int)e;
}

static int validate_args(const BwReplayArgs* a) {
  if (!a || a->n_states < 1 || a->n_events < 0 || a->n_queries < 0 || a->n_keys < 1) return BW_EINVAL;
  if ((int64_t)a->n_states >= ((int64_t)1 << 30)) return BW_EINVAL;
  return 0;
}

}  // namespace bw

using namespace bw;

extern "C" int bw_replay_workspace_size(const BwReplayArgs* a, size_t* bytes) {
  if (validate_args(a) || !bytes) return BW_EINVAL;
  int sms = 0, dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return report(e, "device query");
  Layout L;
  layout(a, pick_blocks(a, sms), L);
  *bytes = L.total;
  return 0;
}

extern "C" int bw_replay_launch(const BwReplayArgs* a) {
  if (validate_args(a) || !a->workspace || !a->parent || (a->n_events && !a->events) ||
      (a->n_queries && (!a->queries || !a->answers)))
    return BW_EINVAL;
  if ((reinterpret_cast<uintptr_t>(a->workspace) & 255) != 0) return BW_EINVAL;
  cudaStream_t st = static_cast<cudaStream_t>(a->stream);
  int sms = 0, dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return report(e, "device query");
  const int32_t B = pick_blocks(a, sms);
  Layout L;
  layout(a, B, L);
  if (a->workspace_bytes < L.total) {
    std::fprintf(stderr, "bw_replay: workspace %zu < required %zu bytes\n", a->workspace_bytes, L.total);
    return BW_EINVAL;
  }
  char* ws = static_cast<char*>(a->workspace);
  Plan P;
  P.eoff = reinterpret_cast<int64_t*>(ws + L.off[0]);
  P.qoff = reinterpret_cast<int64_t*>(ws + L.off[1]);
  P.first_child = reinterpret_cast<int32_t*>(ws + L.off[2]);
  P.next_sib = reinterpret_cast<int32_t*>(ws + L.off[3]);
  P.rank_a = reinterpret_cast<uint64_t*>(ws + L.off[4]);
  P.rank_b = reinterpret_cast<uint64_t*>(ws + L.off[5]);
  P.steps = reinterpret_cast<int32_t*>(ws + L.off[6]);
  P.desc = reinterpret_cast<StepDesc*>(ws + L.off[7]);
  P.work = reinterpret_cast<int64_t*>(ws + L.off[8]);
  P.scan_tmp = reinterpret_cast<int64_t*>(ws + L.off[9]);
  P.bounds = reinterpret_cast<int32_t*>(ws + L.off[10]);
  P.misc = reinterpret_cast<int32_t*>(ws + L.off[11]);
  P.bits = reinterpret_cast<uint64_t*>(ws + L.off[12]);
  P.rlut = reinterpret_cast<uint32_t*>(ws + L.off[13]);
  P.slices = reinterpret_cast<Slice*>(ws + L.off[14]);
  P.nslices = reinterpret_cast<int32_t*>(ws + L.off[15]);
  P.carry = reinterpret_cast<int64_t*>(ws + L.off[16]);
  P.tin = reinterpret_cast<int32_t*>(ws + L.off[17]);
  P.tout = reinterpret_cast<int32_t*>(ws + L.off[18]);
  P.bmode = reinterpret_cast<int32_t*>(ws + L.off[19]);
  P.gsum = reinterpret_cast<int64_t*>(ws + L.off[20]);

  const int32_t S = a->n_states;
  const int64_t S2 = 2 * (int64_t)S;
  const uint32_t C = a->n_keys;
  const int32_t nwords = words_of(C);
  int kernels = 0;
  const int grid = sms * 8;
  auto chk = [&](const char* what) { ++kernels; return report(cudaGetLastError(), what); };
  int rc;
  const bool timing = (a->flags & BW_REPLAY_TIMING) != 0;
  EventSet* evs = nullptr;
  if (timing) {
    if (g_sets_used == g_sets.size()) {
      EventSet es;
      for (auto& ev : es.ev)
        if ((rc = report(cudaEventCreate(&ev), "event create"))) return rc;
      g_sets.push_back(es);
    }
    evs = &g_sets[g_sets_used++];
  }
  auto mark = [&](int i) { return timing ? report(cudaEventRecord(evs->ev[i], st), "event record") : 0; };
  if ((rc = mark(0))) return rc;

  // misc: status = 0, last query step = 0, chain flag = 1 (a kernel, so the whole
  // pipeline stays capturable in a CUDA graph)
  k_init_misc<<<1, 32, 0, st>>>(P.misc);
  if ((rc = chk("k_init_misc"))) return rc;

  // ---- 1. ingest
  if (a->n_events > 0) {
    k_offsets<true><<<grid, 256, 0, st>>>(a->events, a->n_events, S, C, P.eoff, P.misc);
    if ((rc = chk("k_offsets(events)"))) return rc;
  } else {
    k_fill_i64<<<grid, 256, 0, st>>>(P.eoff, (int64_t)S + 1, 0);
    if ((rc = chk("k_fill(eoff)"))) return rc;
  }
  if (a->n_queries > 0) {
    k_offsets<false><<<grid, 256, 0, st>>>(a->queries, a->n_queries, S, C, P.qoff, P.misc);
    if ((rc = chk("k_offsets(queries)"))) return rc;
  } else {
    k_fill_i64<<<grid, 256, 0, st>>>(P.qoff, (int64_t)S + 1, 0);
    if ((rc = chk("k_fill(qoff)"))) return rc;
  }

  if ((rc = mark(1))) return rc;
  // ---- 2. linearise
  int64_t T;  // steps before trimming
  if (a->flags & BW_REPLAY_CHAIN_HINT) {
    k_check_chain<<<grid, 256, 0, st>>>(a->parent, S, P.misc);
    if ((rc = chk("k_check_chain"))) return rc;
    k_steps_chain<<<grid, 256, 0, st>>>(S, P.eoff, P.qoff, P.steps, P.desc, P.misc + 1, P.tin, P.tout, P.misc);
    if ((rc = chk("k_steps_chain"))) return rc;
    T = S;
  } else {
    if ((rc = report(cudaMemsetAsync(P.first_child, 0xFF, (size_t)S * 4, st), "memset"))) return rc;
    k_children<<<grid, 256, 0, st>>>(a->parent, S, P.first_child, P.next_sib, P.misc, P.misc + 2);
    if ((rc = chk("k_children"))) return rc;
    k_rank_init<<<grid, 256, 0, st>>>(a->parent, P.first_child, P.next_sib, S, P.rank_a, P.misc);
    if ((rc = chk("k_rank_init"))) return rc;
    uint64_t* src = P.rank_a;
    uint64_t* dst = P.rank_b;
    for (int64_t span = 1; span < S2; span <<= 1) {
      k_rank_round<<<grid, 256, 0, st>>>(src, dst, S2, P.misc);
      if ((rc = chk("k_rank_round"))) return rc;
      uint64_t* t = src; src = dst; dst = t;
    }
    k_steps<<<grid, 256, 0, st>>>(src, S, P.eoff, P.qoff, P.steps, P.desc, P.misc + 1, P.tin, P.tout, P.misc);
    if ((rc = chk("k_steps"))) return rc;
    T = S2;
  }

  if ((rc = mark(2))) return rc;
  // ---- 3. blocks (over all T steps; steps past the last query step are given
  // no work by clamping the bound to the trimmed length on the device)
  k_work<<<grid, 256, 0, st>>>(P.desc, T, P.misc + 1, P.work);
  if ((rc = chk("k_work"))) return rc;
  if ((rc = device_inclusive_scan_i64(P.work, T, P.scan_tmp, st, kernels))) return rc;
  k_bounds<<<(B + 1 + 127) / 128, 128, 0, st>>>(P.work, T, B, P.bounds);
  if ((rc = chk("k_bounds"))) return rc;
  k_trim_bounds<<<(B + 1 + 127) / 128, 128, 0, st>>>(P.bounds, B, P.misc + 1);
  if ((rc = chk("k_trim_bounds"))) return rc;

  if ((rc = mark(3))) return rc;
  // ---- 4. prepare (slices are sized for the sweep's shared-memory chunk capacity;
  // two sweep CTAs share an SM when there are at least two blocks per SM)
  const int ctas_per_sm = B >= 2 * sms ? 2 : 1;
  const size_t sweep_budget = (size_t)(kSmemPerSM / ctas_per_sm) - 3072;
  const SweepLayout SL = sweep_layout(nwords, sweep_budget);
  const uint32_t cap32 = SL.cap32, cap64 = SL.cap64;
  const size_t smem = prepare_smem(SL.ww, cap32, cap64);
  static bool attr_done = false;
  if (!attr_done) {
    if ((rc = report(cudaFuncSetAttribute(k_prepare, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemLimit - 1024), "smem attr"))) return rc;
    if ((rc = report(cudaFuncSetAttribute(k_sweep, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemLimit - 1024), "smem attr"))) return rc;
    attr_done = true;
  }
  PrepParams pp;
  pp.ev = a->events; pp.desc = P.desc; pp.steps = P.steps; pp.tin = P.tin; pp.tout = P.tout; pp.bounds = P.bounds; pp.nwords = nwords; pp.ww = SL.ww; pp.C = C; pp.cap32 = cap32; pp.cap64 = cap64;
  pp.bits = P.bits; pp.rlut = P.rlut; pp.slices = P.slices; pp.nslices = P.nslices; pp.carry = P.carry;
  pp.status = P.misc; pp.bmode = P.bmode;
  k_prepare<<<B, kPrepThreads, smem, st>>>(pp);
  if ((rc = chk("k_prepare"))) return rc;

  if ((rc = mark(4))) return rc;
  // ---- 5. carry
  {
    const int64_t width = (int64_t)C + 1;
    const dim3 cg((unsigned)((width + 255) / 256), (unsigned)((B + kCarryGroup - 1) / kCarryGroup));
    if (cg.y > 1) {
      k_carry_groups<<<cg, 256, 0, st>>>(P.carry, B, width, P.gsum, P.misc);
      if ((rc = chk("k_carry_groups"))) return rc;
    }
    k_carry_apply<<<cg, 256, 0, st>>>(P.carry, B, width, P.gsum, P.misc);
    if ((rc = chk("k_carry_apply"))) return rc;
  }

  if ((rc = mark(5))) return rc;
  // ---- 6. sweep
  if (a->n_queries > 0) {
    SweepParams sp;
    sp.ev = a->events; sp.qs = a->queries; sp.desc = P.desc; sp.bounds = P.bounds; sp.bits = P.bits;
    sp.rlut = P.rlut; sp.slices = P.slices; sp.nslices = P.nslices; sp.carry = P.carry;
    sp.answers = a->answers; sp.nwords = nwords; sp.C = C; sp.status = P.misc; sp.bmode = P.bmode;
    k_sweep<<<B, kSweepThreads, SL.bytes, st>>>(sp, SL);
    if ((rc = chk("k_sweep"))) return rc;
  }
  if ((rc = mark(6))) return rc;
  {
    std::lock_guard<std::mutex> g(g_info_mu);
    g_last.kernels = kernels;
    g_last.blocks = B;
  }
  return 0;
}

extern "C" int bw_replay_timing_reset(void) {
  g_sets_used = 0;
  return 0;
}

extern "C" int bw_replay_stage_times(float* ms, int32_t* launches) {
  if (!ms) return BW_EINVAL;
  for (int i = 0; i < BW_STAGE_COUNT; ++i) ms[i] = 0.f;
  if (launches) *launches = (int32_t)g_sets_used;
  if (g_sets_used == 0) return 0;
  int rc = report(cudaEventSynchronize(g_sets[g_sets_used - 1].ev[BW_STAGE_COUNT]), "event sync");
  if (rc) return rc;
  for (size_t k = 0; k < g_sets_used; ++k)
    for (int i = 0; i < BW_STAGE_COUNT; ++i) {
      float t = 0.f;
      if ((rc = report(cudaEventElapsedTime(&t, g_sets[k].ev[i], g_sets[k].ev[i + 1]), "event elapsed"))) return rc;
      ms[i] += t;
    }
  return 0;
}

extern "C" int bw_replay_status(const BwReplayArgs* a, int32_t* status) {
  if (!a || !a->workspace || !status) return BW_EINVAL;
  int sms = 0, dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return report(e, "device query");
  Layout L;
  layout(a, pick_blocks(a, sms), L);
  cudaStream_t st = static_cast<cudaStream_t>(a->stream);
  int32_t v = 0;
  e = cudaMemcpyAsync(&v, static_cast<char*>(a->workspace) + L.off[11], 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return report(e, "status read");
  *status = v;
  return 0;
}

extern "C" int bw_replay_last_info(const BwReplayArgs*, int32_t* kernels, int32_t* blocks) {
  std::lock_guard<std::mutex> g(g_info_mu);
  if (kernels) *kernels = g_last.kernels;
  if (blocks) *blocks = g_last.blocks;
  return 0;
}

extern "C" int bw_device_info(int32_t* sm_count, int32_t* arch_tag) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return report(e, "device query");
  if (sm_count) *sm_count = sms;
  if (arch_tag) *arch_tag = BW_ARCH_TAG;
  return 0;
}
