// bw_csr.cu -- sparse-key CSR rank-LUT: device build and lookups.
//
// The reference's CsrBase (sparse_engine.hpp:70-102) ranks a class by a per-64-class
// bitmap word and a cumulative popcount table, and build_csr_base
// (sparse_engine.hpp:287-360) fills it with two row scans over a dense class domain.
// Over a sparse 2^40-key universe a bitmap is not affordable, so here the same rank
// (number of index keys below k) and the same range sum (pre[rank(hi)-1] -
// pre[rank(lo)-1]) come from:
//   build    LSD radix sort of the (key, amount) pairs, 8 bits per pass, stable
//            tile scatter (per-warp digit counts, __match_any_sync ranks);
//            run-length merge of equal keys with the amounts summed; inclusive scan
//            of the amounts (the cumulative prefix `pre`); a bucket LUT
//            lut[b] = #keys below b << shift sized to the caller's byte budget,
//            filled by warps that each cover the bucket gaps of 32 keys with
//            coalesced stores; the low `shift` bits of every key as u16 when
//            shift <= 16, so a probe reads 2 LUT words + a few 2-byte entries.
//   lookup   one thread per 2 point keys / per range, 128-bit loads and stores;
//            a bucket's keys are searched by bisection over the low bits.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "bw_gpu.h"
#include "bw_common.cuh"

namespace bw {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;                          // per thread
constexpr int kSortTile = kSortThreads * kSortItems;    // 4096 pairs per CTA
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kDigits = 256;

inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

// Per-tile digit counts, digit-major: hist[d * ntiles + tile].
// The first pass (check_bits > 0) also flags keys outside [0, 2^check_bits).
__global__ void __launch_bounds__(kSortThreads) k_sort_hist(const uint64_t* __restrict__ keys, int64_t n,
                                                            int shift, int64_t ntiles, int64_t* __restrict__ hist,
                                                            int check_bits, int32_t* __restrict__ status) {
  __shared__ unsigned cnt[kDigits];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kSortTile;
  bool bad = false;
#pragma unroll 4
  for (int j = 0; j < kSortItems; ++j) {
    const int64_t i = base + (int64_t)j * kSortThreads + threadIdx.x;
    if (i < n) {
      const uint64_t k = keys[i];
      atomicAdd(&cnt[(unsigned)(k >> shift) & 255u], 1u);
      if (check_bits > 0 && (k >> check_bits) != 0) bad = true;
    }
  }
  if (bad) atomicExch(status, 1);
  __syncthreads();
  hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

// Stable scatter of one tile by digit.  Warp w owns items [w*32*kSortItems, ...) of
// the tile in groups of 32; ranks inside a group come from __match_any_sync, and
// groups, warps and tiles are taken in input order, so equal digits keep their order.
__global__ void __launch_bounds__(kSortThreads) k_sort_scatter(
    const uint64_t* __restrict__ kin, const int64_t* __restrict__ vin, uint64_t* __restrict__ kout,
    int64_t* __restrict__ vout, int64_t n, int shift, int64_t ntiles, const int64_t* __restrict__ hist_incl) {
  __shared__ unsigned wcnt[kSortWarps][kDigits];
  __shared__ int64_t dbase[kDigits];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int w = 0; w < kSortWarps; ++w) wcnt[w][threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kSortTile + (int64_t)warp * (32 * kSortItems);
  uint64_t k[kSortItems];
  int64_t v[kSortItems];
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const int64_t i = base + j * 32 + lane;
    k[j] = i < n ? kin[i] : 0;
    v[j] = i < n ? vin[i] : 0;
  }
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const bool valid = base + j * 32 + lane < n;
    const unsigned d = valid ? ((unsigned)(k[j] >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    if (valid && (peers & lt) == 0) wcnt[warp][d] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  {
    const int d = threadIdx.x;
    unsigned run = 0;
    for (int w = 0; w < kSortWarps; ++w) {
      const unsigned c = wcnt[w][d];
      wcnt[w][d] = run;
      run += c;
    }
    dbase[d] = hist_incl[(int64_t)d * ntiles + blockIdx.x] - (int64_t)run;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const bool valid = base + j * 32 + lane < n;
    const unsigned d = valid ? ((unsigned)(k[j] >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    if (valid) {
      const int64_t pos = dbase[d] + wcnt[warp][d] + __popc(peers & lt);
      kout[pos] = k[j];
      vout[pos] = v[j];
    }
    __syncwarp();
    if (valid && (peers & lt) == 0) wcnt[warp][d] += __popc(peers);
    __syncwarp();
  }
}

// flag[i] = 1 where i is the last item of a run of equal keys.
__global__ void k_run_flags(const uint64_t* __restrict__ k, int64_t n, int64_t* __restrict__ flag) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    flag[i] = (i + 1 == n || k[i + 1] != k[i]) ? 1 : 0;
}

// The last item of every run writes its key, the cumulative amount and the low bits
// at its run index (pos[i] - 1); the last item overall writes the count.
__global__ void k_run_compact(const uint64_t* __restrict__ k, const int64_t* __restrict__ vscan,
                              const int64_t* __restrict__ pos, int64_t n, int shift, uint64_t* __restrict__ ukeys,
                              int64_t* __restrict__ pre, uint16_t* __restrict__ low, int64_t* __restrict__ count) {
  const uint64_t mask = shift >= 64 ? ~0ull : ((1ull << shift) - 1ull);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (i + 1 == n || k[i + 1] != k[i]) {
      const int64_t u = pos[i] - 1;
      ukeys[u] = k[i];
      pre[u] = vscan[i];
      if (low) low[u] = (uint16_t)(k[i] & mask);
      if (i + 1 == n) *count = pos[i];
    }
  }
}

// lut[b] = number of keys whose bucket is below b, for b up to the last key's bucket.
// Warp w handles keys [32w, 32w+32): the buckets (bucket(key[32w-1]), bucket(key[32w+31])]
// get the warp's base index plus the count of its lanes with a lower bucket, found by
// bisection over the lanes' buckets with shuffles.
// Buckets are clamped to [0, nb) so that keys outside the universe (a flagged input
// error) cannot write past the table.
__global__ void k_lut_fill(const uint64_t* __restrict__ ukeys, const int64_t* __restrict__ count, int shift,
                           int64_t nb, uint32_t* __restrict__ lut) {
  const int64_t m = *count;
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = gw; w * 32 < m; w += nw) {
    const int64_t u0 = w * 32;
    const int64_t u = u0 + lane;
    const int64_t bu = u < m ? (int64_t)(ukeys[u] >> shift) : INT64_MAX;
    const int64_t bstart = u0 ? imin64((int64_t)(ukeys[u0 - 1] >> shift), nb - 1) + 1 : 0;
    const int64_t ulast = (u0 + 32 < m ? u0 + 32 : m) - 1;
    const int64_t bend = imin64((int64_t)(ukeys[ulast] >> shift), nb - 1);
    for (int64_t b0 = bstart; b0 <= bend; b0 += 32) {
      const int64_t b = b0 + lane;
      int lo = 0;
#pragma unroll
      for (int step = 16; step; step >>= 1) {
        const int64_t x = __shfl_sync(0xffffffffu, bu, lo + step - 1);
        if (x < b) lo += step;
      }
      const int64_t x = __shfl_sync(0xffffffffu, bu, lo);
      if (x < b) ++lo;
      if (b <= bend) lut[b] = (uint32_t)(u0 + lo);
    }
  }
}

// Buckets past the last key's bucket (all of them when there are no keys) hold m.
__global__ void k_lut_tail(const uint64_t* __restrict__ ukeys, const int64_t* __restrict__ count, int shift,
                           int64_t nb, uint32_t* __restrict__ lut) {
  const int64_t m = *count;
  const int64_t first = m ? imin64((int64_t)(ukeys[m - 1] >> shift), nb - 1) + 1 : 0;
  for (int64_t b = first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += (int64_t)gridDim.x * blockDim.x)
    lut[b] = (uint32_t)m;
}

// rank(k) = number of index keys below k; *present when k is one of them.
__device__ __forceinline__ int64_t csr_rank(const BwCsr& x, int64_t m, uint64_t k, bool& present) {
  present = false;
  if (x.key_bits < 64 && (k >> x.key_bits) != 0) return m;
  const int64_t b = (int64_t)(k >> x.shift);
  // clamped to [0, m]: an index built from flagged input stays memory-safe
  int64_t lo = imin64(__ldg(x.lut + b), m);
  int64_t hi = b + 1 < x.n_buckets ? imin64(__ldg(x.lut + b + 1), m) : m;
  const int64_t end = hi;   // the bucket's keys are [lo, end)
  if (x.low) {
    // keys of one bucket share their high bits: compare the low `shift` bits
    const uint16_t t = (uint16_t)(k & ((1ull << x.shift) - 1ull));
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (__ldg(x.low + mid) < t) lo = mid + 1; else hi = mid;
    }
    present = lo < end && __ldg(x.low + lo) == t;
  } else {
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (__ldg(x.keys + mid) < k) lo = mid + 1; else hi = mid;
    }
    present = lo < end && __ldg(x.keys + lo) == k;
  }
  return lo;
}

__global__ void k_csr_point(BwCsr x, const uint64_t* __restrict__ keys, int64_t n, int64_t* __restrict__ out) {
  const int64_t m = *x.count;
  const int64_t npairs = n >> 1;
  const ulonglong2* kv = reinterpret_cast<const ulonglong2*>(keys);
  longlong2* ov = reinterpret_cast<longlong2*>(out);
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npairs; p += (int64_t)gridDim.x * blockDim.x) {
    const ulonglong2 k = kv[p];
    bool pa, pb;
    const int64_t ra = csr_rank(x, m, k.x, pa);
    const int64_t rb = csr_rank(x, m, k.y, pb);
    ov[p] = make_longlong2(pa ? ra : -ra - 1, pb ? rb : -rb - 1);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    bool pr;
    const int64_t r = csr_rank(x, m, keys[n - 1], pr);
    out[n - 1] = pr ? r : -r - 1;
  }
}

__global__ void k_csr_range(BwCsr x, const uint64_t* __restrict__ bounds, int64_t n, int64_t* __restrict__ out) {
  const int64_t m = *x.count;
  const ulonglong2* bv = reinterpret_cast<const ulonglong2*>(bounds);
  longlong2* ov = reinterpret_cast<longlong2*>(out);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const ulonglong2 q = bv[i];
    bool pr;
    const int64_t a = csr_rank(x, m, q.x, pr);
    const int64_t b = csr_rank(x, m, q.y, pr);
    uint64_t sum = 0;
    if (a != b) {
      const uint64_t shi = b ? (uint64_t)__ldg(x.pre + b - 1) : 0;
      const uint64_t slo = a ? (uint64_t)__ldg(x.pre + a - 1) : 0;
      sum = shi - slo;
    }
    ov[i] = make_longlong2(b - a, (int64_t)sum);
  }
}

// Versioned sparse keys (the event model over the index's ranks): event records
// keyed by the rank of their u64 key (a key missing from the index gets rank m, which
// the replay reports as out of range), and query records over rank intervals -- a
// point lookup of a present key is [rank, rank + 1), of an absent one empty; a range
// lookup [lo, hi) over keys is [rank(lo), rank(hi)) over ranks.
__global__ void k_csr_events(BwCsr x, const uint32_t* __restrict__ states, const uint64_t* __restrict__ keys,
                             const int64_t* __restrict__ deltas, int64_t n, BwEvent* __restrict__ out) {
  const int64_t m = *x.count;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    bool pr;
    const int64_t r = csr_rank(x, m, keys[i], pr);
    BwEvent e;
    e.state = states[i];
    e.key = (uint32_t)(pr ? r : m);
    e.delta = deltas[i];
    out[i] = e;
  }
}
__global__ void k_csr_queries(BwCsr x, const uint32_t* __restrict__ states, const uint64_t* __restrict__ lo,
                              const uint64_t* __restrict__ hi, int64_t n, BwQuery* __restrict__ out) {
  const int64_t m = *x.count;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    bool pr;
    const int64_t a = csr_rank(x, m, lo[i], pr);
    BwQuery q;
    q.state = states[i];
    if (!hi) {
      q.lo = pr ? (uint32_t)a : 0u;
      q.hi = pr ? (uint32_t)a + 1u : 0u;
    } else {
      bool pb;
      q.lo = (uint32_t)a;
      q.hi = (uint32_t)csr_rank(x, m, hi[i], pb);
    }
    out[i] = q;
  }
}

struct CsrLayout {
  int32_t shift = 0, passes = 0;
  int64_t nb = 0, ntiles = 0;
  size_t off_count, off_status, off_keys, off_pre, off_low, off_lut;     // persistent index
  size_t off_ka, off_va, off_kb, off_vb, off_hist, off_tmp;  // build scratch
  size_t total;
};

int csr_layout(int64_t n, int32_t key_bits, size_t budget, CsrLayout& L) {
  if (n < 0 || n >= ((int64_t)1 << 31) || key_bits < 1 || key_bits > 63 || budget < 4) return BW_EINVAL;
  int lb = 0;  // log2 of the bucket count
  while (lb < key_bits && ((size_t)1 << (lb + 1)) * 4 <= budget) ++lb;
  L.nb = (int64_t)1 << lb;
  L.shift = key_bits - lb;
  L.passes = (key_bits + 7) / 8;
  L.ntiles = (n + kSortTile - 1) / kSortTile;
  const size_t un = (size_t)(n > 0 ? n : 1);
  size_t o = 0;
  auto take = [&](size_t bytes) { const size_t at = o; o = al256(o + bytes); return at; };
  L.off_count = take(8);
  L.off_status = take(4);
  L.off_keys = take(un * 8);
  L.off_pre = take(un * 8);
  L.off_low = take(L.shift <= 16 ? un * 2 : 0);
  L.off_lut = take((size_t)L.nb * 4);
  L.off_ka = take(un * 8);
  L.off_va = take(un * 8);
  L.off_kb = take(un * 8);
  L.off_vb = take(un * 8);
  const size_t nh = (size_t)kDigits * (size_t)(L.ntiles > 0 ? L.ntiles : 1);
  L.off_hist = take(nh * 8);
  const size_t scan_n = nh > un ? nh : un;
  L.off_tmp = take(scan_tmp_bytes(scan_n));
  L.total = o;
  return 0;
}

int report(cudaError_t e, const char* what) {
  if (e != cudaSuccess) std::fprintf(stderr, "bw_csr: %s failed: %s\n", what, cudaGetErrorString(e));
  return (int)e;
}

int grid_for(int64_t items, int threads) {
  int sms = 0, dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    sms = 148;
  const int64_t want = (items + threads - 1) / threads;
  const int64_t cap = (int64_t)sms * 16;
  return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

}  // namespace
}  // namespace bw

using namespace bw;

extern "C" int bw_csr_workspace_size(int64_t n_items, int32_t key_bits, size_t lut_budget_bytes, size_t* bytes) {
  if (!bytes) return BW_EINVAL;
  CsrLayout L;
  if (csr_layout(n_items, key_bits, lut_budget_bytes, L)) return BW_EINVAL;
  *bytes = L.total;
  return 0;
}

extern "C" int bw_csr_build(const uint64_t* keys, const int64_t* amounts, int64_t n_items, int32_t key_bits,
                            size_t lut_budget_bytes, void* workspace, size_t workspace_bytes, void* stream,
                            BwCsr* out) {
  CsrLayout L;
  if (!out || !workspace || csr_layout(n_items, key_bits, lut_budget_bytes, L)) return BW_EINVAL;
  if (n_items > 0 && (!keys || !amounts)) return BW_EINVAL;
  if ((reinterpret_cast<uintptr_t>(workspace) & 255) != 0) return BW_EINVAL;
  if (workspace_bytes < L.total) {
    std::fprintf(stderr, "bw_csr_build: workspace %zu < required %zu bytes\n", workspace_bytes, L.total);
    return BW_EINVAL;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* ws = static_cast<char*>(workspace);
  int64_t* count = reinterpret_cast<int64_t*>(ws + L.off_count);
  int32_t* status = reinterpret_cast<int32_t*>(ws + L.off_status);
  uint64_t* ukeys = reinterpret_cast<uint64_t*>(ws + L.off_keys);
  int64_t* pre = reinterpret_cast<int64_t*>(ws + L.off_pre);
  uint16_t* low = L.shift <= 16 ? reinterpret_cast<uint16_t*>(ws + L.off_low) : nullptr;
  uint32_t* lut = reinterpret_cast<uint32_t*>(ws + L.off_lut);
  uint64_t* ka = reinterpret_cast<uint64_t*>(ws + L.off_ka);
  int64_t* va = reinterpret_cast<int64_t*>(ws + L.off_va);
  uint64_t* kb = reinterpret_cast<uint64_t*>(ws + L.off_kb);
  int64_t* vb = reinterpret_cast<int64_t*>(ws + L.off_vb);
  int64_t* hist = reinterpret_cast<int64_t*>(ws + L.off_hist);
  int64_t* tmp = reinterpret_cast<int64_t*>(ws + L.off_tmp);
  int rc;
  int kernels = 0;
  if ((rc = report(cudaMemsetAsync(count, 0, 8, st), "memset"))) return rc;
  if ((rc = report(cudaMemsetAsync(status, 0, 4, st), "memset"))) return rc;
  const int64_t n = n_items;
  uint64_t* ksorted = ka;
  int64_t* vsorted = va;
  if (n > 0) {
    // ---- LSD radix sort, 8 bits per pass; pass p reads (src) and writes (dst)
    const uint64_t* ksrc = keys;
    const int64_t* vsrc = amounts;
    uint64_t* kdst = ka;
    int64_t* vdst = va;
    for (int p = 0; p < L.passes; ++p) {
      const int shift = 8 * p;
      k_sort_hist<<<(unsigned)L.ntiles, kSortThreads, 0, st>>>(ksrc, n, shift, L.ntiles, hist,
                                                                p == 0 ? key_bits : 0, status);
      if ((rc = report(cudaGetLastError(), "k_sort_hist"))) return rc;
      if ((rc = device_inclusive_scan_i64(hist, (int64_t)kDigits * L.ntiles, tmp, st, kernels))) return rc;
      k_sort_scatter<<<(unsigned)L.ntiles, kSortThreads, 0, st>>>(ksrc, vsrc, kdst, vdst, n, shift, L.ntiles, hist);
      if ((rc = report(cudaGetLastError(), "k_sort_scatter"))) return rc;
      ksorted = kdst;
      vsorted = vdst;
      ksrc = kdst;
      vsrc = vdst;
      kdst = (kdst == ka) ? kb : ka;
      vdst = (vdst == va) ? vb : va;
    }
    // ---- run-length merge: cumulative amounts (inclusive scan of the sorted
    // amounts, read at the last item of each run) and run indices
    int64_t* pos = reinterpret_cast<int64_t*>(ksorted == ka ? kb : ka);   // free buffer
    const int g = grid_for(n, 256);
    k_run_flags<<<g, 256, 0, st>>>(ksorted, n, pos);
    if ((rc = report(cudaGetLastError(), "k_run_flags"))) return rc;
    if ((rc = device_inclusive_scan_i64(pos, n, tmp, st, kernels))) return rc;
    if ((rc = device_inclusive_scan_i64(vsorted, n, tmp, st, kernels))) return rc;
    k_run_compact<<<g, 256, 0, st>>>(ksorted, vsorted, pos, n, L.shift, ukeys, pre, low, count);
    if ((rc = report(cudaGetLastError(), "k_run_compact"))) return rc;
    k_lut_fill<<<grid_for(n, 256), 256, 0, st>>>(ukeys, count, L.shift, L.nb, lut);
    if ((rc = report(cudaGetLastError(), "k_lut_fill"))) return rc;
  }
  k_lut_tail<<<grid_for(L.nb, 256), 256, 0, st>>>(ukeys, count, L.shift, L.nb, lut);
  if ((rc = report(cudaGetLastError(), "k_lut_tail"))) return rc;
  out->key_bits = key_bits;
  out->shift = L.shift;
  out->n_buckets = L.nb;
  out->count = count;
  out->status = status;
  out->keys = ukeys;
  out->pre = pre;
  out->lut = lut;
  out->low = low;
  return 0;
}

static int check_index(const BwCsr* x) {
  if (!x || !x->count || !x->status || !x->lut || !x->keys || !x->pre || x->key_bits < 1 || x->key_bits > 63 || x->shift < 0 ||
      x->shift > x->key_bits || x->n_buckets != ((int64_t)1 << (x->key_bits - x->shift)) || (x->low && x->shift > 16))
    return BW_EINVAL;
  return 0;
}

extern "C" int bw_csr_point(const BwCsr* idx, const uint64_t* keys, int64_t n, int64_t* out, void* stream) {
  if (check_index(idx) || n < 0 || (n > 0 && (!keys || !out))) return BW_EINVAL;
  if (n == 0) return 0;
  if ((reinterpret_cast<uintptr_t>(keys) & 15) || (reinterpret_cast<uintptr_t>(out) & 15)) return BW_EINVAL;
  k_csr_point<<<grid_for((n + 1) / 2, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(*idx, keys, n, out);
  return report(cudaGetLastError(), "k_csr_point");
}

extern "C" int bw_csr_range(const BwCsr* idx, const uint64_t* bounds, int64_t n, int64_t* out, void* stream) {
  if (check_index(idx) || n < 0 || (n > 0 && (!bounds || !out))) return BW_EINVAL;
  if (n == 0) return 0;
  if ((reinterpret_cast<uintptr_t>(bounds) & 15) || (reinterpret_cast<uintptr_t>(out) & 15)) return BW_EINVAL;
  k_csr_range<<<grid_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(*idx, bounds, n, out);
  return report(cudaGetLastError(), "k_csr_range");
}

extern "C" int bw_csr_status(const BwCsr* idx, int32_t* status) {
  if (check_index(idx) || !status) return BW_EINVAL;
  int rc = report(cudaDeviceSynchronize(), "synchronise");
  if (rc) return rc;
  return report(cudaMemcpy(status, idx->status, 4, cudaMemcpyDeviceToHost), "status read");
}

extern "C" int bw_csr_events(const BwCsr* idx, const uint32_t* states, const uint64_t* keys, const int64_t* deltas,
                             int64_t n, BwEvent* out, void* stream) {
  if (check_index(idx) || n < 0 || (n > 0 && (!states || !keys || !deltas || !out))) return BW_EINVAL;
  if (n == 0) return 0;
  k_csr_events<<<grid_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(*idx, states, keys, deltas, n, out);
  return report(cudaGetLastError(), "k_csr_events");
}

extern "C" int bw_csr_queries(const BwCsr* idx, const uint32_t* states, const uint64_t* lo, const uint64_t* hi,
                              int64_t n, BwQuery* out, void* stream) {
  if (check_index(idx) || n < 0 || (n > 0 && (!states || !lo || !out))) return BW_EINVAL;
  if (n == 0) return 0;
  k_csr_queries<<<grid_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(*idx, states, lo, hi, n, out);
  return report(cudaGetLastError(), "k_csr_queries");
}
