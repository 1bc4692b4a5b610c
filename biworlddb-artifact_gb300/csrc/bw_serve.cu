// bw_serve.cu -- served form of the version-tree replay: a device-resident version
// store and a persistent request loop.
//
// Store.  Every version v keeps its own events sorted by key with their inclusive
// delta prefix ("overlay", in an arena), a parent pointer, and either a dense
// key-prefix row (a "checkpoint": row[k] = sum of the deltas with key < k over
// v's whole root path) or a short list of overlay members: the versions between
// its nearest checkpoint ancestor (exclusive) and itself (inclusive).  A child
// reads its parent's row and the members' overlays; nothing is copied.  The
// initial tree gets checkpoints densely enough that every member list is short,
// with the checkpoint spacing picked so that the store fits the HBM admission cap.
// A range-sum query on v is row[hi] - row[lo] of v's checkpoint plus, for each
// member (one per lane), pre(hi) - pre(lo) found by binary search in its overlay.
//
// Loop.  One persistent kernel, one request per warp: a warp claims the next
// request index, waits until the host has published it (acquire load of the tail
// in host-mapped memory), waits until the version it reads is ready, executes it,
// writes the answer into host-mapped memory and releases its completion flag.  A
// commit or fork creates the next version id: its overlay is sorted in the warp, its
// member list is the parent's plus itself (a link to the parent once the list is
// full) and its ready flag is released when its tables are written.  Requests are
// claimed in log order and only wait on earlier ones, and every CTA of the grid is
// resident, so no wait can cycle; every wait is also bounded (an iteration limit and
// a host abort flag), after which the kernel records an error and returns.
//
// Host.  bw_serve_run publishes requests at their arrival times (open loop) while
// keeping at most max_inflight unfinished requests admitted (the slots of the
// continuous batch), records completion times on the same host clock, and admits
// the run only if its commit events fit the store's event arena (the memory cap).
#include <cuda_runtime.h>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "bw_gpu.h"

namespace {

constexpr int kD = 32;                       // overlay members per version list (one per lane)
constexpr int kServeThreads = 256;
constexpr int kServeWarps = kServeThreads / 32;
constexpr int kMaxCommit = 128;              // events per commit
constexpr uint64_t kSpinLimit = 1ull << 25;  // default bound of every device wait, in polls (each with a nanosleep backoff)
constexpr int kRowThreads = 256;

int report(cudaError_t e, const char* what) {
  if (e != cudaSuccess) std::fprintf(stderr, "bw_serve: %s failed: %s\n", what, cudaGetErrorString(e));
  return (int)e;
}

struct StoreDev {
  uint32_t C;
  int32_t* parent;
  int32_t* anc;      // nearest checkpoint ancestor-or-self (-1: none)
  int32_t* rowid;    // row of a checkpoint version, -1 otherwise
  int32_t* clen;     // overlay members in the list
  int32_t* link;     // version whose list continues this one (-1: none)
  int32_t* members;  // kD per version
  int64_t* ev_off;   // overlay of the version in the arena
  int32_t* ev_cnt;
  uint32_t* akey;    // arena: keys sorted per version
  int64_t* apre;     // arena: inclusive delta prefix in key order
  int64_t* rows;     // checkpoint rows, (C + 1) each
  int32_t* ready;
  unsigned long long* arena_top;
};

struct RunDev {
  const BwServeRequest* req;   // host-mapped
  const BwEvent* cev;          // host-mapped commit events
  const uint32_t* tail;        // host-mapped: requests published
  const uint32_t* abort;       // host-mapped: stop waiting
  int64_t* ans;                // host-mapped answers
  uint32_t* done;              // host-mapped completion flags
  unsigned int* head;          // device: next request to claim
  uint32_t* dtail;             // device: copy of the published count (written by the dispatcher)
  uint32_t n;
  int32_t* err;                // host-mapped: first error (1 = wait limit or abort)
  uint64_t spin_limit;         // polls before a wait gives up
};

__device__ __forceinline__ uint32_t ld_acquire_sys(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_sys(uint32_t* p, uint32_t v) {
  asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int32_t ld_acquire_gpu(const int32_t* p) {
  int32_t v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu(int32_t* p, int32_t v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) { return *(const volatile uint32_t*)p; }

// Sum of the deltas of version m's own events with key < x.
__device__ __forceinline__ uint64_t overlay_prefix(const StoreDev& d, int32_t m, uint32_t x) {
  const int64_t off = d.ev_off[m];
  int32_t lo = 0, hi = d.ev_cnt[m];
  while (lo < hi) {
    const int32_t mid = (lo + hi) >> 1;
    if (d.akey[off + mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo ? (uint64_t)d.apre[off + lo - 1] : 0ull;
}

// Lane 0 waits (bounded) until ready[v] is set; returns false on abort/limit.
__device__ bool wait_ready(const StoreDev& d, const RunDev& r, int32_t v) {
  const int lane = threadIdx.x & 31;
  int ok = 1;
  if (lane == 0) {
    uint64_t it = 0;
    unsigned ns = 32;
    while (ld_acquire_gpu(d.ready + v) == 0) {
      if (++it > r.spin_limit || ((it & 255) == 0 && ld_volatile(r.abort))) {
        atomicCAS(r.err, 0, 1);
        ok = 0;
        break;
      }
      __nanosleep(ns);
      if (ns < 2048) ns <<= 1;
    }
  }
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

__global__ void __launch_bounds__(kServeThreads) k_serve(StoreDev d, RunDev r) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // Dispatcher: one warp polls the host's published count and republishes it in
  // device memory, so the serving warps poll L2 instead of host memory.  (Request
  // records and commit events are written before the launch.)
  if (blockIdx.x == 0 && warp == 0) {
    if (lane == 0) {
      uint32_t seen = 0;
      uint64_t idle = 0;
      while (seen < r.n) {
        const uint32_t t = ld_acquire_sys(r.tail);
        if (t != seen) {
          seen = t;
          idle = 0;
          asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(r.dtail), "r"(t) : "memory");
        } else {
          if (ld_volatile(r.abort) || ++idle > r.spin_limit) {
            atomicCAS(r.err, 0, 1);
            break;
          }
          __nanosleep(64);
        }
      }
    }
    return;
  }
  __shared__ uint32_t s_key[kServeWarps][kMaxCommit];
  __shared__ int64_t s_del[kServeWarps][kMaxCommit];
  __shared__ uint32_t s_skey[kServeWarps][kMaxCommit];
  __shared__ int64_t s_sdel[kServeWarps][kMaxCommit];
  const uint32_t W = d.C + 1;
  for (;;) {
    uint32_t idx = 0;
    if (lane == 0) idx = atomicAdd(r.head, 1u);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= r.n) return;
    int ok = 1;
    uint32_t f[8];
    if (lane == 0) {
      uint64_t it = 0;
      unsigned ns = 32;
      while (true) {
        uint32_t t;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(t) : "l"(r.dtail) : "memory");
        if (t > idx) break;
        // the host-mapped abort/error words are read only every 256 polls (C2C traffic)
        if (++it > r.spin_limit ||
            ((it & 255) == 0 && (ld_volatile(r.abort) || ld_volatile(reinterpret_cast<const uint32_t*>(r.err))))) {
          atomicCAS(r.err, 0, 1);
          ok = 0;
          break;
        }
        __nanosleep(ns);
        if (ns < 1024) ns <<= 1;
      }
      if (ok) {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(r.req + idx);
#pragma unroll
        for (int i = 0; i < 8; ++i) f[i] = src[i];
      }
    }
    if (!__shfl_sync(0xffffffffu, ok, 0)) return;
#pragma unroll
    for (int i = 0; i < 8; ++i) f[i] = __shfl_sync(0xffffffffu, f[i], 0);
    const uint32_t kind = f[0], ver = f[1], lo = f[2], hi = f[3], nv = f[4], ne = f[5];
    const uint64_t eoff = (uint64_t)f[6] | ((uint64_t)f[7] << 32);
    if (!wait_ready(d, r, (int32_t)ver)) return;
    int64_t answer = 0;
    if (kind == BW_REQ_QUERY) {
      uint64_t sum = 0;
      if (hi > lo) {
        int32_t cur = (int32_t)ver;
        while (cur >= 0) {
          const int32_t len = d.clen[cur];
          for (int32_t i = lane; i < len; i += 32) {
            const int32_t m = d.members[(int64_t)cur * kD + i];
            sum += overlay_prefix(d, m, hi) - overlay_prefix(d, m, lo);
          }
          cur = d.link[cur];
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        const int32_t a = d.anc[ver];
        if (a >= 0) {
          const int64_t* row = d.rows + (int64_t)d.rowid[a] * W;
          sum += (uint64_t)row[hi] - (uint64_t)row[lo];
        }
      }
      answer = (int64_t)sum;
    } else {
      // commit (events) or fork (none): version nv, child of ver
      const int32_t p = (int32_t)ver, w = (int32_t)nv;
      const int32_t n = kind == BW_REQ_COMMIT ? (int32_t)min(ne, (uint32_t)kMaxCommit) : 0;
      for (int32_t i = lane; i < n; i += 32) {
        const BwEvent e = r.cev[eoff + i];
        s_key[warp][i] = e.key;
        s_del[warp][i] = e.delta;
      }
      __syncwarp();
      // rank sort by (key, position), then the delta prefix in key order
      for (int32_t i = lane; i < n; i += 32) {
        const uint32_t k = s_key[warp][i];
        int32_t rank = 0;
        for (int32_t j = 0; j < n; ++j) {
          const uint32_t kj = s_key[warp][j];
          rank += (kj < k || (kj == k && j < i)) ? 1 : 0;
        }
        s_skey[warp][rank] = k;
        s_sdel[warp][rank] = s_del[warp][i];
      }
      __syncwarp();
      int64_t off = 0;
      if (lane == 0 && n > 0) off = (int64_t)atomicAdd(d.arena_top, (unsigned long long)n);
      off = __shfl_sync(0xffffffffu, off, 0);
      const int32_t per = (n + 31) / 32, a0 = min(n, lane * per), a1 = min(n, a0 + per);
      uint64_t part = 0;
      for (int32_t i = a0; i < a1; ++i) part += (uint64_t)s_sdel[warp][i];
      uint64_t incl = part;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      uint64_t run = incl - part;
      for (int32_t i = a0; i < a1; ++i) {
        run += (uint64_t)s_sdel[warp][i];
        d.akey[off + i] = s_skey[warp][i];
        d.apre[off + i] = (int64_t)run;
      }
      const bool pck = d.rowid[p] >= 0;
      const int32_t plen = d.clen[p], plink = d.link[p];
      int32_t len, lnk;
      if (pck) {               // parent is a checkpoint: the list is the new version
        len = 1;
        lnk = -1;
        if (lane == 0) d.members[(int64_t)w * kD] = w;
      } else if (plen < kD && plink < 0) {   // parent's list plus the new version
        len = plen + 1;
        lnk = -1;
        for (int32_t i = lane; i < plen; i += 32) d.members[(int64_t)w * kD + i] = d.members[(int64_t)p * kD + i];
        if (lane == 0) d.members[(int64_t)w * kD + plen] = w;
      } else {                 // full list: the new version, then the parent's lists
        len = 1;
        lnk = p;
        if (lane == 0) d.members[(int64_t)w * kD] = w;
      }
      if (lane == 0) {
        d.parent[w] = p;
        d.anc[w] = pck ? p : d.anc[p];
        d.rowid[w] = -1;
        d.clen[w] = len;
        d.link[w] = lnk;
        d.ev_off[w] = off;
        d.ev_cnt[w] = n;
      }
      __syncwarp();
      __threadfence();
      if (lane == 0) st_release_gpu(d.ready + w, 1);
    }
    if (lane == 0) {
      r.ans[idx] = answer;
      st_release_sys(r.done + idx, 1u);
    }
  }
}

// Checkpoint rows of one level: row = base row (the nearest checkpoint strictly
// above, or zero) + the prefix of every member overlay, column by column.
__global__ void __launch_bounds__(kRowThreads) k_build_rows(StoreDev d, const int32_t* ck, const int32_t* base,
                                                            const int64_t* moff, const int32_t* mlist, int32_t n) {
  const int32_t i = blockIdx.x;
  if (i >= n) return;
  const uint32_t W = d.C + 1;
  const int32_t c = ck[i];
  int64_t* out = d.rows + (int64_t)d.rowid[c] * W;
  const int64_t* in = base[i] >= 0 ? d.rows + (int64_t)d.rowid[base[i]] * W : nullptr;
  const int64_t m0 = moff[i], m1 = moff[i + 1];
  for (uint32_t j = threadIdx.x; j < W; j += blockDim.x) {
    uint64_t v = in ? (uint64_t)in[j] : 0ull;
    for (int64_t k = m0; k < m1; ++k) v += overlay_prefix(d, mlist[k], j);
    out[j] = (int64_t)v;
  }
}

}  // namespace

struct BwServe {
  int dev = 0;
  uint32_t C = 0;
  int32_t S0 = 0;            // initial versions
  int64_t next = 0;          // next version id (versions created by earlier runs persist)
  int32_t max_versions = 0;
  int64_t arena_cap = 0, arena_used0 = 0;
  int32_t checkpoints = 0, spacing = 0;
  size_t store_bytes = 0;
  StoreDev d{};
  void* mem = nullptr;       // one device allocation for the store
  unsigned int* head = nullptr;
  int32_t warps = 0;
  int32_t grid = 0;
  uint64_t spin_limit = 0;   // polls before a device wait gives up
};

namespace {

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

void free_store(BwServe* s) {
  if (s->mem) cudaFree(s->mem);
  s->mem = nullptr;
}

}  // namespace

extern "C" int bw_serve_create(const BwServeConfig* cfg, BwServe** out) {
  if (!cfg || !out || cfg->n_states < 1 || !cfg->parent || cfg->n_keys < 1 || cfg->n_events < 0 ||
      (cfg->n_events && !cfg->events) || cfg->max_versions < cfg->n_states || cfg->max_events < cfg->n_events ||
      cfg->max_versions >= (1 << 30))
    return BW_EINVAL;
  *out = nullptr;
  const int32_t S = cfg->n_states;
  const uint32_t C = cfg->n_keys;
  const int32_t V = cfg->max_versions;
  const int64_t E = cfg->n_events, Ecap = cfg->max_events;
  const int32_t* par = cfg->parent;
  for (int32_t v = 0; v < S; ++v)
    if ((v == 0 && par[v] != -1) || (v > 0 && (par[v] < 0 || par[v] >= v))) return BW_EINVAL;
  const BwEvent* ev = cfg->events;
  for (int64_t i = 0; i < E; ++i)
    if (ev[i].state >= (uint32_t)S || ev[i].key >= C || (i && ev[i].state < ev[i - 1].state)) return BW_EINVAL;

  // ---- overlays: each state's events sorted by key, inclusive delta prefix
  std::vector<int64_t> eoff(S + 1, 0);
  for (int64_t i = 0; i < E; ++i) eoff[ev[i].state + 1]++;
  for (int32_t v = 0; v < S; ++v) eoff[v + 1] += eoff[v];
  std::vector<uint32_t> akey(E);
  std::vector<int64_t> apre(E);
  {
    const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
      th.emplace_back([&, t]() {
        std::vector<std::pair<uint32_t, int64_t>> tmp;
        for (int32_t v = (int32_t)t; v < S; v += (int32_t)nt) {
          tmp.clear();
          for (int64_t i = eoff[v]; i < eoff[v + 1]; ++i) tmp.emplace_back(ev[i].key, ev[i].delta);
          std::stable_sort(tmp.begin(), tmp.end(),
                           [](const std::pair<uint32_t, int64_t>& a, const std::pair<uint32_t, int64_t>& b) {
                             return a.first < b.first;
                           });
          uint64_t run = 0;
          for (size_t k = 0; k < tmp.size(); ++k) {
            run += (uint64_t)tmp[k].second;
            akey[eoff[v] + k] = tmp[k].first;
            apre[eoff[v] + k] = (int64_t)run;
          }
        }
      });
    for (auto& x : th) x.join();
  }

  // ---- checkpoint spacing: the densest that fits the cap (a version is a
  // checkpoint when its member list would exceed `spacing`)
  const size_t row_bytes = ((size_t)C + 1) * 8;
  const size_t fixed = align256((size_t)V * 4) * 6 + align256((size_t)V * kD * 4) + align256((size_t)V * 8) +
                       align256((size_t)Ecap * 4) + align256((size_t)Ecap * 8) + 4096;
  const int32_t limit = cfg->chain_limit > 0 ? std::min(cfg->chain_limit, kD) : kD;
  std::vector<int32_t> clen(S), isck(S);
  int32_t spacing = 0, nck = 0;
  for (int32_t sp : {1, 2, 3, 4, 6, 8, 12, 16, 24, 32}) {
    if (sp > limit) break;
    nck = 0;
    for (int32_t v = 0; v < S; ++v) {
      const int32_t p = par[v];
      int32_t l = p < 0 ? 0 : (isck[p] ? 1 : clen[p] + 1);
      isck[v] = p < 0 || l > sp;
      if (isck[v]) { l = 0; ++nck; }
      clen[v] = l;
    }
    spacing = sp;
    if (fixed + (size_t)nck * row_bytes <= cfg->hbm_cap_bytes) break;
  }
  const size_t total = fixed + (size_t)nck * row_bytes;
  if (total > cfg->hbm_cap_bytes) {
    std::fprintf(stderr, "bw_serve: the store needs %zu bytes, more than the %zu-byte cap\n", total,
                 cfg->hbm_cap_bytes);
    return BW_EINVAL;
  }

  // ---- host tables
  std::vector<int32_t> anc(V, -1), rowid(V, -1), link(V, -1), ready(V, 0), cl(V, 0), cnt(V, 0);
  std::vector<int32_t> members((size_t)V * kD, -1);
  std::vector<int64_t> off(V, 0);
  std::vector<int32_t> level(S, 0);
  int32_t r = 0, maxlevel = 0;
  for (int32_t v = 0; v < S; ++v) {
    const int32_t p = par[v];
    off[v] = eoff[v];
    cnt[v] = (int32_t)(eoff[v + 1] - eoff[v]);
    ready[v] = 1;
    if (isck[v]) {
      rowid[v] = r++;
      anc[v] = v;
      cl[v] = 0;
      level[v] = p < 0 ? 0 : level[anc[p]] + 1;
      maxlevel = std::max(maxlevel, level[v]);
    } else {
      anc[v] = anc[p];
      if (isck[p]) {
        cl[v] = 1;
        members[(size_t)v * kD] = v;
      } else {
        cl[v] = cl[p] + 1;
        for (int32_t i = 0; i < cl[p]; ++i) members[(size_t)v * kD + i] = members[(size_t)p * kD + i];
        members[(size_t)v * kD + cl[p]] = v;
      }
    }
  }
  // row build lists, by level: base = the checkpoint strictly above, members = the
  // parent's list plus the checkpoint itself
  std::vector<std::vector<int32_t>> lv_ck(maxlevel + 1), lv_base(maxlevel + 1), lv_m(maxlevel + 1);
  std::vector<std::vector<int64_t>> lv_off(maxlevel + 1, std::vector<int64_t>(1, 0));
  for (int32_t v = 0; v < S; ++v) {
    if (!isck[v]) continue;
    const int32_t p = par[v], L = level[v];
    lv_ck[L].push_back(v);
    lv_base[L].push_back(p < 0 ? -1 : anc[p]);
    if (p >= 0 && !isck[p])
      for (int32_t i = 0; i < cl[p]; ++i) lv_m[L].push_back(members[(size_t)p * kD + i]);
    lv_m[L].push_back(v);
    lv_off[L].push_back((int64_t)lv_m[L].size());
  }

  // ---- device store
  BwServe* s = new BwServe();
  int rc = report(cudaGetDevice(&s->dev), "cudaGetDevice");
  if (rc) { delete s; return rc; }
  s->C = C; s->S0 = S; s->next = S; s->max_versions = V; s->arena_cap = Ecap; s->arena_used0 = E;
  s->spin_limit = cfg->spin_limit ? cfg->spin_limit : kSpinLimit;
  s->checkpoints = nck; s->spacing = spacing; s->store_bytes = total;
  size_t o = 0;
  auto take = [&](size_t bytes) { const size_t at = o; o += align256(bytes); return at; };
  const size_t o_parent = take((size_t)V * 4), o_anc = take((size_t)V * 4), o_row = take((size_t)V * 4),
               o_clen = take((size_t)V * 4), o_link = take((size_t)V * 4), o_ready = take((size_t)V * 4),
               o_mem = take((size_t)V * kD * 4), o_off = take((size_t)V * 8), o_cnt = take((size_t)V * 4),
               o_akey = take((size_t)Ecap * 4), o_apre = take((size_t)Ecap * 8), o_top = take(8),
               o_head = take(8), o_rows = take((size_t)nck * row_bytes);
  if ((rc = report(cudaMalloc(&s->mem, o), "cudaMalloc(store)"))) { delete s; return rc; }
  char* m = static_cast<char*>(s->mem);
  StoreDev& d = s->d;
  d.C = C;
  d.parent = reinterpret_cast<int32_t*>(m + o_parent);
  d.anc = reinterpret_cast<int32_t*>(m + o_anc);
  d.rowid = reinterpret_cast<int32_t*>(m + o_row);
  d.clen = reinterpret_cast<int32_t*>(m + o_clen);
  d.link = reinterpret_cast<int32_t*>(m + o_link);
  d.ready = reinterpret_cast<int32_t*>(m + o_ready);
  d.members = reinterpret_cast<int32_t*>(m + o_mem);
  d.ev_off = reinterpret_cast<int64_t*>(m + o_off);
  d.ev_cnt = reinterpret_cast<int32_t*>(m + o_cnt);
  d.akey = reinterpret_cast<uint32_t*>(m + o_akey);
  d.apre = reinterpret_cast<int64_t*>(m + o_apre);
  d.arena_top = reinterpret_cast<unsigned long long*>(m + o_top);
  d.rows = reinterpret_cast<int64_t*>(m + o_rows);
  s->head = reinterpret_cast<unsigned int*>(m + o_head);
  std::vector<int32_t> parv(V, -1);
  std::copy(par, par + S, parv.begin());
  const unsigned long long top = (unsigned long long)E;
  auto up = [&](void* dst, const void* src, size_t bytes) -> int {
    return bytes ? report(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), "store upload") : 0;
  };
  if ((rc = up(d.parent, parv.data(), (size_t)V * 4)) || (rc = up(d.anc, anc.data(), (size_t)V * 4)) ||
      (rc = up(d.rowid, rowid.data(), (size_t)V * 4)) || (rc = up(d.clen, cl.data(), (size_t)V * 4)) ||
      (rc = up(d.link, link.data(), (size_t)V * 4)) || (rc = up(d.ready, ready.data(), (size_t)V * 4)) ||
      (rc = up(d.members, members.data(), (size_t)V * kD * 4)) || (rc = up(d.ev_off, off.data(), (size_t)V * 8)) ||
      (rc = up(d.ev_cnt, cnt.data(), (size_t)V * 4)) || (rc = up(d.akey, akey.data(), (size_t)E * 4)) ||
      (rc = up(d.apre, apre.data(), (size_t)E * 8)) || (rc = up(d.arena_top, &top, 8))) {
    free_store(s);
    delete s;
    return rc;
  }
  // checkpoint rows, level by level (a level reads only rows of earlier levels)
  for (int32_t L = 0; L <= maxlevel && !rc; ++L) {
    const int32_t n = (int32_t)lv_ck[L].size();
    if (!n) continue;
    int32_t *dck = nullptr, *dbase = nullptr, *dm = nullptr;
    int64_t* doff = nullptr;
    const size_t nm = lv_m[L].size();
    if ((rc = report(cudaMalloc(&dck, (size_t)n * 4), "cudaMalloc")) ||
        (rc = report(cudaMalloc(&dbase, (size_t)n * 4), "cudaMalloc")) ||
        (rc = report(cudaMalloc(&dm, nm * 4), "cudaMalloc")) ||
        (rc = report(cudaMalloc(&doff, ((size_t)n + 1) * 8), "cudaMalloc")) ||
        (rc = up(dck, lv_ck[L].data(), (size_t)n * 4)) || (rc = up(dbase, lv_base[L].data(), (size_t)n * 4)) ||
        (rc = up(dm, lv_m[L].data(), nm * 4)) || (rc = up(doff, lv_off[L].data(), ((size_t)n + 1) * 8))) {
    } else {
      k_build_rows<<<n, kRowThreads>>>(d, dck, dbase, doff, dm, n);
      rc = report(cudaGetLastError(), "k_build_rows");
      if (!rc) rc = report(cudaDeviceSynchronize(), "k_build_rows sync");
    }
    cudaFree(dck); cudaFree(dbase); cudaFree(dm); cudaFree(doff);
  }
  if (rc) {
    free_store(s);
    delete s;
    return rc;
  }
  int per_sm = 0, sms = 0;
  rc = report(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_serve, kServeThreads, 0), "occupancy");
  if (!rc) rc = report(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->dev), "device query");
  if (rc || per_sm < 1) {
    free_store(s);
    delete s;
    return rc ? rc : BW_EINVAL;
  }
  s->grid = per_sm * sms;
  s->warps = s->grid * kServeWarps;
  *out = s;
  return 0;
}

extern "C" int bw_serve_reset(BwServe* s) {
  if (!s) return BW_EINVAL;
  const size_t extra = (size_t)(s->max_versions - s->S0);
  int rc = 0;
  if (extra) rc = report(cudaMemset(s->d.ready + s->S0, 0, extra * 4), "reset");
  const unsigned long long top = (unsigned long long)s->arena_used0;
  if (!rc) rc = report(cudaMemcpy(s->d.arena_top, &top, 8, cudaMemcpyHostToDevice), "reset");
  if (!rc) s->next = s->S0;
  return rc;
}

extern "C" int bw_serve_info(const BwServe* s, BwServeStats* st) {
  if (!s || !st) return BW_EINVAL;
  std::memset(st, 0, sizeof(*st));
  st->checkpoints = s->checkpoints;
  st->spacing = s->spacing;
  st->store_bytes = s->store_bytes;
  st->warps = s->warps;
  return 0;
}

extern "C" int bw_serve_destroy(BwServe* s) {
  if (!s) return 0;
  free_store(s);
  delete s;
  return 0;
}

extern "C" int bw_serve_run(BwServe* s, const BwServeRequest* reqs, int64_t n, const BwEvent* commit_events,
                            int64_t n_commit_events, const double* arrival_s, int32_t max_inflight,
                            double timeout_s, int64_t* answers, float* latency_us, BwServeStats* stats) {
  if (!s || n < 0 || n >= ((int64_t)1 << 31) || (n && (!reqs || !answers || !latency_us)) || max_inflight < 1 ||
      n_commit_events < 0 || (n_commit_events && !commit_events))
    return BW_EINVAL;
  // validate the log: versions exist when read, new ids are consecutive, commits fit
  int64_t next = s->next, new_events = 0, q = 0, c = 0, f = 0;
  for (int64_t i = 0; i < n; ++i) {
    const BwServeRequest& r = reqs[i];
    if (r.version >= (uint64_t)next) return BW_EINVAL;
    if (r.kind == BW_REQ_QUERY) {
      if (r.lo > s->C || r.hi > s->C) return BW_EINVAL;
      ++q;
    } else if (r.kind == BW_REQ_COMMIT || r.kind == BW_REQ_FORK) {
      if (r.new_version != (uint64_t)next || next >= s->max_versions) return BW_EINVAL;
      if (r.kind == BW_REQ_COMMIT) {
        if (r.n_events > (uint32_t)kMaxCommit || r.events_off + r.n_events > (uint64_t)n_commit_events) return BW_EINVAL;
        for (uint32_t k = 0; k < r.n_events; ++k)
          if (commit_events[r.events_off + k].key >= s->C) return BW_EINVAL;
        new_events += r.n_events;
        ++c;
      } else {
        ++f;
      }
      ++next;
    } else {
      return BW_EINVAL;
    }
  }
  // admission by memory footprint: the run's commits must fit the event arena
  unsigned long long top = 0;
  int rc = report(cudaMemcpy(&top, s->d.arena_top, 8, cudaMemcpyDeviceToHost), "arena read");
  if (rc) return rc;
  if ((int64_t)top + new_events > s->arena_cap) {
    std::fprintf(stderr, "bw_serve: the run's %lld commit events exceed the arena (%lld free of %lld)\n",
                 (long long)new_events, (long long)(s->arena_cap - (int64_t)top), (long long)s->arena_cap);
    return BW_EINVAL;
  }
  if (n == 0) return 0;
  // host-mapped buffers for the run
  BwServeRequest* h_req = nullptr;
  BwEvent* h_cev = nullptr;
  uint32_t* h_ctl = nullptr;   // [0] tail, [1] abort, [2] device error
  int64_t* h_ans = nullptr;
  uint32_t* h_done = nullptr;
  auto cleanup = [&]() {
    if (h_req) cudaFreeHost(h_req);
    if (h_cev) cudaFreeHost(h_cev);
    if (h_ctl) cudaFreeHost(h_ctl);
    if (h_ans) cudaFreeHost(h_ans);
    if (h_done) cudaFreeHost(h_done);
  };
  const size_t ncev = (size_t)std::max<int64_t>(1, n_commit_events);
  if ((rc = report(cudaHostAlloc((void**)&h_req, (size_t)n * sizeof(BwServeRequest), cudaHostAllocMapped), "host alloc")) ||
      (rc = report(cudaHostAlloc((void**)&h_cev, ncev * sizeof(BwEvent), cudaHostAllocMapped), "host alloc")) ||
      (rc = report(cudaHostAlloc((void**)&h_ctl, 64, cudaHostAllocMapped), "host alloc")) ||
      (rc = report(cudaHostAlloc((void**)&h_ans, (size_t)n * 8, cudaHostAllocMapped), "host alloc")) ||
      (rc = report(cudaHostAlloc((void**)&h_done, (size_t)n * 4, cudaHostAllocMapped), "host alloc"))) {
    cleanup();
    return rc;
  }
  std::memcpy(h_req, reqs, (size_t)n * sizeof(BwServeRequest));
  if (n_commit_events) std::memcpy(h_cev, commit_events, (size_t)n_commit_events * sizeof(BwEvent));
  std::memset(h_ctl, 0, 64);
  std::memset(h_done, 0, (size_t)n * 4);
  RunDev r{};
  void* p = nullptr;
  if ((rc = report(cudaHostGetDevicePointer(&p, h_req, 0), "mapped pointer"))) { cleanup(); return rc; }
  r.req = static_cast<const BwServeRequest*>(p);
  if ((rc = report(cudaHostGetDevicePointer(&p, h_cev, 0), "mapped pointer"))) { cleanup(); return rc; }
  r.cev = static_cast<const BwEvent*>(p);
  if ((rc = report(cudaHostGetDevicePointer(&p, h_ctl, 0), "mapped pointer"))) { cleanup(); return rc; }
  r.tail = static_cast<const uint32_t*>(p);
  r.abort = static_cast<const uint32_t*>(p) + 1;
  if ((rc = report(cudaHostGetDevicePointer(&p, h_ans, 0), "mapped pointer"))) { cleanup(); return rc; }
  r.ans = static_cast<int64_t*>(p);
  if ((rc = report(cudaHostGetDevicePointer(&p, h_done, 0), "mapped pointer"))) { cleanup(); return rc; }
  r.done = static_cast<uint32_t*>(p);
  r.head = s->head;
  r.dtail = reinterpret_cast<uint32_t*>(s->head) + 1;
  r.n = (uint32_t)n;
  r.spin_limit = s->spin_limit;
  r.err = reinterpret_cast<int32_t*>(const_cast<uint32_t*>(r.tail) + 2);
  cudaStream_t st = nullptr;
  if ((rc = report(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream"))) { cleanup(); return rc; }
  if ((rc = report(cudaMemsetAsync(s->head, 0, 8, st), "memset"))) {
    cudaStreamDestroy(st);
    cleanup();
    return rc;
  }
  k_serve<<<s->grid, kServeThreads, 0, st>>>(s->d, r);
  if ((rc = report(cudaGetLastError(), "k_serve"))) {
    cudaStreamDestroy(st);
    cleanup();
    return rc;
  }
  // producer (open-loop arrivals, bounded in-flight slots) and consumer on the host clock
  using clk = std::chrono::steady_clock;
  std::vector<clk::time_point> t_done(n);
  std::atomic<int64_t> completed{0};
  std::atomic<bool> stop{false};
  const clk::time_point t0 = clk::now() + std::chrono::microseconds(200);
  auto sched = [&](int64_t i) {
    const double a = arrival_s ? arrival_s[i] : 0.0;
    return t0 + std::chrono::nanoseconds((int64_t)(a * 1e9));
  };
  std::thread producer([&]() {
    int64_t i = 0;
    while (i < n && !stop.load(std::memory_order_relaxed)) {
      const clk::time_point now = clk::now();
      int64_t j = i;
      const int64_t lim = completed.load(std::memory_order_acquire) + max_inflight;
      while (j < n && j < lim && sched(j) <= now) ++j;
      if (j > i) {
        __atomic_store_n(h_ctl, (uint32_t)j, __ATOMIC_RELEASE);
        i = j;
      }
    }
  });
  std::vector<uint8_t> seen(n, 0);
  const clk::time_point deadline = clk::now() + std::chrono::duration_cast<clk::duration>(std::chrono::duration<double>(timeout_s));
  int64_t done_n = 0;
  bool timed_out = false;
  while (done_n < n) {
    const int64_t pub = (int64_t)__atomic_load_n(h_ctl, __ATOMIC_ACQUIRE);
    const int64_t hi = std::min<int64_t>(pub, done_n + 65536);
    const clk::time_point now = clk::now();
    for (int64_t k = done_n; k < hi; ++k)
      if (!seen[k] && __atomic_load_n(h_done + k, __ATOMIC_ACQUIRE)) {
        seen[k] = 1;
        t_done[k] = now;
      }
    while (done_n < n && seen[done_n]) ++done_n;
    completed.store(done_n, std::memory_order_release);
    if (__atomic_load_n(h_ctl + 2, __ATOMIC_ACQUIRE)) break;   // the device gave up waiting
    if (now > deadline) {
      timed_out = true;
      break;
    }
  }
  if (timed_out) __atomic_store_n(h_ctl + 1, 1u, __ATOMIC_RELEASE);
  stop.store(true);
  producer.join();
  const clk::time_point t_end = clk::now();
  rc = report(cudaStreamSynchronize(st), "k_serve sync");
  const uint32_t err = __atomic_load_n(h_ctl + 2, __ATOMIC_ACQUIRE);
  cudaStreamDestroy(st);
  if (!rc && (err || timed_out)) {
    std::fprintf(stderr, "bw_serve: the loop stopped early (%s)\n", timed_out ? "host timeout" : "device wait limit");
    rc = BW_EINVAL;
  }
  if (!rc) {
    s->next = next;
    for (int64_t k = 0; k < n; ++k) {
      answers[k] = h_ans[k];
      const clk::time_point a = std::max(sched(k), t0);
      latency_us[k] = (float)(std::chrono::duration<double, std::micro>(t_done[k] - a).count());
    }
    if (stats) {
      std::memset(stats, 0, sizeof(*stats));
      stats->requests = n;
      stats->queries = q;
      stats->commits = c;
      stats->forks = f;
      stats->wall_s = std::chrono::duration<double>(t_end - t0).count();
      stats->checkpoints = s->checkpoints;
      stats->spacing = s->spacing;
      stats->store_bytes = s->store_bytes;
      stats->warps = s->warps;
    }
  }
  cleanup();
  return rc;
}
