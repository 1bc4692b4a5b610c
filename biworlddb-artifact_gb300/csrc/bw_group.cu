// bw_group.cu -- grouping ungrouped event and query arrays by state on the device
// (bw_group_events, bw_group_queries; include/bw_gpu.h).
//
// The replay takes events and queries grouped by state.  A caller whose records
// arrive in another order (an event stream, a log merged from several writers)
// groups them here: a stable LSD radix sort of 16-byte records by their u32 state,
// 8 bits per pass over the bits the state count needs (three passes up to 16.7M
// states).  Per pass, k_grp_hist counts the digits of every 2,048-record tile
// (digit-major, so one inclusive scan gives every tile's output base per digit) and
// k_grp_scatter writes each tile stably: warps take their 32-record groups in input
// order, ranks inside a group from __match_any_sync.  Queries travel as 16-byte
// records (state, lo, hi, input index) so the caller gets, beside the grouped
// queries, the input position of each one (bw_scatter_answers puts the answers back
// in input order).  The first pass also checks every state against the state count
// (BW_STATUS_STATE_RANGE in the status word).
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "bw_gpu.h"
#include "bw_common.cuh"

namespace bw {
namespace {

constexpr int kGrpThreads = 256;
constexpr int kGrpItems = 8;                           // records per thread
constexpr int kGrpTile = kGrpThreads * kGrpItems;      // 2,048 records per CTA
constexpr int kGrpWarps = kGrpThreads / 32;
constexpr int kGrpDigits = 256;

inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

__global__ void __launch_bounds__(kGrpThreads) k_grp_hist(const uint4* __restrict__ rec, int64_t n, int shift,
                                                          int64_t ntiles, int64_t* __restrict__ hist,
                                                          uint32_t n_states, int32_t* __restrict__ status) {
  __shared__ unsigned cnt[kGrpDigits];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kGrpTile;
  bool bad = false;
#pragma unroll 4
  for (int j = 0; j < kGrpItems; ++j) {
    const int64_t i = base + (int64_t)j * kGrpThreads + threadIdx.x;
    if (i < n) {
      const uint32_t s = rec[i].x;
      atomicAdd(&cnt[(s >> shift) & 255u], 1u);
      bad |= s >= n_states;
    }
  }
  if (bad && status) atomicCAS(status, 0, BW_STATUS_STATE_RANGE);
  __syncthreads();
  hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(kGrpThreads) k_grp_scatter(const uint4* __restrict__ in, uint4* __restrict__ out,
                                                             int64_t n, int shift, int64_t ntiles,
                                                             const int64_t* __restrict__ hist_incl) {
  __shared__ unsigned wcnt[kGrpWarps][kGrpDigits];
  __shared__ int64_t dbase[kGrpDigits];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int w = 0; w < kGrpWarps; ++w) wcnt[w][threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kGrpTile + (int64_t)warp * (32 * kGrpItems);
  uint4 r[kGrpItems];
#pragma unroll
  for (int j = 0; j < kGrpItems; ++j) {
    const int64_t i = base + j * 32 + lane;
    r[j] = i < n ? in[i] : make_uint4(0, 0, 0, 0);
  }
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int j = 0; j < kGrpItems; ++j) {
    const bool valid = base + j * 32 + lane < n;
    const unsigned d = valid ? ((r[j].x >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    if (valid && (peers & lt) == 0) wcnt[warp][d] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  {
    const int d = threadIdx.x;
    unsigned run = 0;
    for (int w = 0; w < kGrpWarps; ++w) {
      const unsigned c = wcnt[w][d];
      wcnt[w][d] = run;
      run += c;
    }
    dbase[d] = hist_incl[(int64_t)d * ntiles + blockIdx.x] - (int64_t)run;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kGrpItems; ++j) {
    const bool valid = base + j * 32 + lane < n;
    const unsigned d = valid ? ((r[j].x >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    if (valid) out[dbase[d] + wcnt[warp][d] + __popc(peers & lt)] = r[j];
    __syncwarp();
    if (valid && (peers & lt) == 0) wcnt[warp][d] += __popc(peers);
    __syncwarp();
  }
}

// 12-byte queries <-> 16-byte (state, lo, hi, input index) records
__global__ void k_grp_qin(const BwQuery* __restrict__ q, int64_t n, uint4* __restrict__ rec) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const BwQuery x = q[i];
    rec[i] = make_uint4(x.state, x.lo, x.hi, (uint32_t)i);
  }
}
__global__ void k_grp_qout(const uint4* __restrict__ rec, int64_t n, BwQuery* __restrict__ q,
                           int64_t* __restrict__ order) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint4 r = rec[i];
    q[i] = BwQuery{r.x, r.y, r.z};
    if (order) order[i] = (int64_t)r.w;
  }
}

int grp_passes(int32_t n_states) {
  int bits = 0;
  while (bits < 32 && ((uint64_t)1 << bits) < (uint64_t)(n_states > 1 ? n_states : 1)) ++bits;
  return bits == 0 ? 1 : (bits + 7) / 8;
}

struct GrpLayout {
  size_t status, hist, tmp, rec_a, rec_b, total;
  int64_t ntiles;
};
GrpLayout grp_layout(int64_t n, bool queries) {
  GrpLayout L;
  L.ntiles = (n + kGrpTile - 1) / kGrpTile;
  if (L.ntiles < 1) L.ntiles = 1;
  const size_t nh = (size_t)kGrpDigits * (size_t)L.ntiles;
  size_t o = 0;
  L.status = o;  o = al256(o + 4);
  L.hist = o;    o = al256(o + nh * 8);
  L.tmp = o;     o = al256(o + scan_tmp_bytes(nh));
  L.rec_a = o;   o = al256(o + (size_t)n * 16);
  L.rec_b = o;   o = al256(o + (queries ? (size_t)n * 16 : 0));
  L.total = o;
  return L;
}

int grp_report(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return 0;
  std::fprintf(stderr, "bw_group: %s: %s\n", what, cudaGetErrorString(e));
  return (int)e;
}

// Sorts n records from `src` (read-only) ending in `dst`; `a` is scratch of n records.
int grp_sort(const uint4* src, uint4* dst, uint4* a, int64_t n, int32_t n_states, const GrpLayout& L, char* ws,
             cudaStream_t st) {
  const int passes = grp_passes(n_states);
  int64_t* hist = reinterpret_cast<int64_t*>(ws + L.hist);
  int64_t* tmp = reinterpret_cast<int64_t*>(ws + L.tmp);
  int32_t* status = reinterpret_cast<int32_t*>(ws + L.status);
  int rc = grp_report(cudaMemsetAsync(status, 0, 4, st), "status reset");
  int kernels = 0;
  const uint4* in = src;
  for (int p = 0; p < passes && !rc; ++p) {
    uint4* out = ((passes - p) % 2 == 1) ? dst : a;   // the last pass lands in dst
    k_grp_hist<<<(unsigned)L.ntiles, kGrpThreads, 0, st>>>(in, n, 8 * p, L.ntiles, hist, (uint32_t)n_states,
                                                          p == 0 ? status : nullptr);
    if ((rc = grp_report(cudaGetLastError(), "histogram launch"))) break;
    if ((rc = device_inclusive_scan_i64(hist, (int64_t)kGrpDigits * L.ntiles, tmp, st, kernels))) {
      rc = grp_report((cudaError_t)rc, "scan");
      break;
    }
    k_grp_scatter<<<(unsigned)L.ntiles, kGrpThreads, 0, st>>>(in, out, n, 8 * p, L.ntiles, hist);
    if ((rc = grp_report(cudaGetLastError(), "scatter launch"))) break;
    in = out;
  }
  return rc;
}

}  // namespace
}  // namespace bw

using namespace bw;

extern "C" int bw_group_workspace_size(int64_t n, int32_t queries, size_t* bytes) {
  if (n < 0 || !bytes) return BW_EINVAL;
  *bytes = grp_layout(n, queries != 0).total;
  return 0;
}

extern "C" int bw_group_events(const BwEvent* in, int64_t n, int32_t n_states, BwEvent* out, void* workspace,
                               size_t workspace_bytes, void* stream) {
  if (n < 0 || n_states < 1 || (n && (!in || !out || (const void*)in == (const void*)out))) return BW_EINVAL;
  const GrpLayout L = grp_layout(n, false);
  if (!workspace || workspace_bytes < L.total) return BW_EINVAL;
  if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) return BW_EINVAL;
  if (n == 0) return 0;
  char* ws = static_cast<char*>(workspace);
  return grp_sort(reinterpret_cast<const uint4*>(in), reinterpret_cast<uint4*>(out),
                  reinterpret_cast<uint4*>(ws + L.rec_a), n, n_states, L, ws, static_cast<cudaStream_t>(stream));
}

extern "C" int bw_group_queries(const BwQuery* in, int64_t n, int32_t n_states, BwQuery* out, int64_t* order,
                                void* workspace, size_t workspace_bytes, void* stream) {
  if (n < 0 || n_states < 1 || n >= ((int64_t)1 << 32) || (n && (!in || !out))) return BW_EINVAL;
  const GrpLayout L = grp_layout(n, true);
  if (!workspace || workspace_bytes < L.total) return BW_EINVAL;
  if (n == 0) return 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* ws = static_cast<char*>(workspace);
  // passes alternate between the final buffer F and the other one; the packed
  // records start in whichever buffer the first pass does not write
  uint4* F = reinterpret_cast<uint4*>(ws + L.rec_a);
  uint4* Y = reinterpret_cast<uint4*>(ws + L.rec_b);
  uint4* X = (grp_passes(n_states) % 2) ? Y : F;
  const int64_t blocks = (n + 255) / 256;
  const unsigned g = (unsigned)(blocks < 4096 ? blocks : 4096);
  k_grp_qin<<<g, 256, 0, st>>>(in, n, X);
  int rc = grp_report(cudaGetLastError(), "query pack launch");
  if (!rc) rc = grp_sort(X, F, Y, n, n_states, L, ws, st);
  if (rc) return rc;
  k_grp_qout<<<g, 256, 0, st>>>(F, n, out, order);
  return grp_report(cudaGetLastError(), "query unpack launch");
}

extern "C" int bw_group_status(const void* workspace, int32_t* status) {
  if (!workspace || !status) return BW_EINVAL;
  return grp_report(cudaMemcpy(status, workspace, 4, cudaMemcpyDeviceToHost), "status read");
}
