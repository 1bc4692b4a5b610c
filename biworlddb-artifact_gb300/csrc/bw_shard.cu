// bw_shard.cu -- device side of a chain split across ranks (one process per GPU).
//
// A chain's events grouped by state are its replay order, so rank r can take the
// contiguous state range [s_r, s_{r+1}) and replay it alone as a chain of its own;
// what the ranks above it miss is the carry, the dense key histogram of every event
// below s_r: an exclusive scan over ranks of each rank's own histogram (the
// reference's serial carry pass, batch_engine_v7.hpp:936-945, lifted from state
// blocks to ranks).  These entries give a rank its histogram, the key prefix of a
// carry vector, and the carry added to its answers inside [lo, hi) (the combine,
// batch_engine_v7.hpp:948-961).  The scan itself is the caller's exchange.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "bw_gpu.h"
#include "bw_common.cuh"

namespace bw {
namespace {

constexpr int kHistThreads = 512;
constexpr uint32_t kHistSmemKeys = 16384;   // keys held per CTA in shared memory

int shard_report(cudaError_t e, const char* what) {
  if (e != cudaSuccess) std::fprintf(stderr, "bw_shard: %s failed: %s\n", what, cudaGetErrorString(e));
  return (int)e;
}

// Per-CTA histogram in shared memory (exact 32-bit-pair atomics), merged into the
// global histogram with one 64-bit atomic per nonzero key.
__global__ void __launch_bounds__(kHistThreads) k_hist_smem(const BwEvent* ev, int64_t n, uint32_t C,
                                                            unsigned long long* hist) {
  extern __shared__ unsigned long long h[];
  for (uint32_t k = threadIdx.x; k < C; k += blockDim.x) h[k] = 0;
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const BwEvent e = ev[i];
    if (e.key < C) shared_add_u64(h + e.key, (uint64_t)e.delta);
  }
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < C; k += blockDim.x)
    if (h[k]) atomicAdd(hist + k, h[k]);
}

__global__ void k_hist_global(const BwEvent* ev, int64_t n, uint32_t C, unsigned long long* hist) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const BwEvent e = ev[i];
    if (e.key < C) atomicAdd(hist + e.key, (unsigned long long)e.delta);
  }
}

// prefix[k] = sum of vec[j] for j < k, k = 0..n (one CTA, chunked block scans).
__global__ void __launch_bounds__(1024) k_key_prefix(const int64_t* vec, uint32_t n, int64_t* prefix) {
  uint64_t carry = 0;
  for (uint32_t c0 = 0; c0 <= n; c0 += blockDim.x) {
    const uint32_t k = c0 + threadIdx.x;
    const uint64_t v = k < n ? (uint64_t)vec[k] : 0;
    uint64_t total = 0;
    const uint64_t ex = block_exclusive_scan<uint64_t>(v, &total);
    if (k <= n) prefix[k] = (int64_t)(carry + ex);
    carry += total;
  }
}

__global__ void k_add_carry(const BwQuery* qs, int64_t n, uint32_t C, const int64_t* prefix, int64_t* ans) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const BwQuery q = qs[i];
    const uint32_t lo = min(q.lo, C), hi = min(q.hi, C);
    if (lo < hi) ans[i] = (int64_t)((uint64_t)ans[i] + (uint64_t)prefix[hi] - (uint64_t)prefix[lo]);
  }
}

// dst[slot[i]] = src[i] where 0 <= slot[i] < n_dst: answers of a stream workload's
// chain queries (stream order) into the reference's answer order.
__global__ void k_scatter(const int64_t* src, const int64_t* slot, int64_t n, int64_t* dst, int64_t n_dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = slot[i];
    if (s >= 0 && s < n_dst) dst[s] = src[i];
  }
}

int grid_for(int64_t n, int threads) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t need = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)(sms > 0 ? sms : 1) * 4;
  return (int)(need < 1 ? 1 : (need < cap ? need : cap));
}

}  // namespace
}  // namespace bw

using namespace bw;

extern "C" int bw_key_histogram(const BwEvent* events, int64_t n, uint32_t n_keys, int64_t* hist, void* stream) {
  if (n < 0 || n_keys < 1 || !hist || (n && !events)) return BW_EINVAL;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = shard_report(cudaMemsetAsync(hist, 0, (size_t)n_keys * 8, st), "histogram reset");
  if (rc || n == 0) return rc;
  unsigned long long* h = reinterpret_cast<unsigned long long*>(hist);
  if (n_keys <= kHistSmemKeys) {
    static bool attr = false;   // one-time, as gpu_v7_launch's
    if (!attr) {
      if ((rc = shard_report(cudaFuncSetAttribute(k_hist_smem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)(kHistSmemKeys * 8)), "histogram attribute")))
        return rc;
      attr = true;
    }
    k_hist_smem<<<grid_for(n, kHistThreads), kHistThreads, (size_t)n_keys * 8, st>>>(events, n, n_keys, h);
  } else {
    k_hist_global<<<grid_for(n, 256), 256, 0, st>>>(events, n, n_keys, h);
  }
  return shard_report(cudaGetLastError(), "histogram launch");
}

extern "C" int bw_key_prefix(const int64_t* vec, uint32_t n, int64_t* prefix, void* stream) {
  if (!vec || !prefix || n < 1) return BW_EINVAL;
  k_key_prefix<<<1, 1024, 0, static_cast<cudaStream_t>(stream)>>>(vec, n, prefix);
  return shard_report(cudaGetLastError(), "key prefix launch");
}

extern "C" int bw_add_range_carry(const BwQuery* queries, int64_t n, uint32_t n_keys, const int64_t* prefix,
                                  int64_t* answers, void* stream) {
  if (n < 0 || n_keys < 1 || !prefix || (n && (!queries || !answers))) return BW_EINVAL;
  if (n == 0) return 0;
  k_add_carry<<<grid_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(queries, n, n_keys, prefix, answers);
  return shard_report(cudaGetLastError(), "carry launch");
}

extern "C" int bw_scatter_answers(const int64_t* src, const int64_t* slot, int64_t n, int64_t* dst, int64_t n_dst,
                                  void* stream) {
  if (n < 0 || n_dst < 0 || (n && (!src || !slot || !dst))) return BW_EINVAL;
  if (n == 0) return 0;
  k_scatter<<<grid_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(src, slot, n, dst, n_dst);
  return shard_report(cudaGetLastError(), "scatter launch");
}
