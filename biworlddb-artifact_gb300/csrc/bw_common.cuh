// bw_common.cuh -- device helpers shared by the GB300 kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#if defined(__CUDA_ARCH__)
#define BW_ARCH_TAG (__CUDA_ARCH__)
#else
#define BW_ARCH_TAG 1030
#endif

namespace bw {

__host__ __device__ __forceinline__ int64_t imin64(int64_t a, int64_t b) { return a < b ? a : b; }

// ------------------------------------------------------------------ rank LUT
// Rank of key offset x inside a slice: popcount rank table + bitmap word, the
// CSR rank-LUT probe of sparse_engine.hpp:77-86 (rlut + popcount(word & mask)).
__device__ __forceinline__ uint32_t local_rank(const uint64_t* bits, const uint32_t* rl, uint32_t x) {
  const uint32_t wi = x >> 6;
  const uint64_t m = (1ull << (x & 63)) - 1ull;
  return rl[wi] + (uint32_t)__popcll(bits[wi] & m);
}

// Exact 64-bit add into a shared-memory word with two 32-bit atomics.  The low
// word's atomic returns its old value; its unsigned overflow is the carry into the
// high word.  Any interleaving of such adds leaves (hi:lo) equal to the sum modulo
// 2^64 once all of them have completed (readers wait at a barrier).  On sm_103 a
// contended 64-bit shared atomicAdd is one to two orders of magnitude slower than
// this pair (measured: 22.6 ms vs 0.53 ms for 512k adds per SM on one address).
__device__ __forceinline__ void shared_add_u64(unsigned long long* addr, uint64_t v) {
  unsigned* w = reinterpret_cast<unsigned*>(addr);
  const unsigned lo = (unsigned)v;
  const unsigned old = atomicAdd(w, lo);
  const unsigned hi = (unsigned)(v >> 32) + ((old + lo) < old ? 1u : 0u);
  if (hi) atomicAdd(w + 1, hi);
}

// Set bit b of a shared-memory bitmap of 64-bit words with a 32-bit atomic.
__device__ __forceinline__ void shared_set_bit(uint64_t* words, uint32_t b) {
  atomicOr(reinterpret_cast<unsigned*>(words) + (b >> 5), 1u << (b & 31));
}

// Fenwick point update at 1-based index i over n nodes (one thread).
__device__ __forceinline__ void fenwick_add(unsigned long long* fen, uint32_t n, uint32_t i, uint64_t d) {
  for (; i <= n; i += i & (0u - i)) shared_add_u64(fen + i, d);
}

__device__ __forceinline__ uint64_t fenwick_prefix(const unsigned long long* fen, uint32_t r) {
  uint64_t s = 0;
  for (uint32_t i = r; i; i &= i - 1) s += fen[i];
  return s;
}

// Prefix (keys < k) of the current slice's contribution: 0 below the slice, the
// slice total above it, the Fenwick prefix at the key's rank inside it.
__device__ __forceinline__ uint64_t slice_prefix(const unsigned long long* fen, uint32_t n, const uint64_t* bits,
                                                 const uint32_t* rl, uint32_t klo, uint32_t khi, uint32_t k) {
  if (k <= klo) return 0;
  if (k >= khi) return fenwick_prefix(fen, n);
  return fenwick_prefix(fen, local_rank(bits, rl, k - klo));
}

// ------------------------------------------------------------------ block scans
// Block-wide exclusive scan of a per-thread value; returns the block total.
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* total_out = nullptr) {
  __shared__ T s_warp[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = lane < nw ? s_warp[lane] : (T)0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    s_warp[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  const T before = (warp ? s_warp[warp - 1] : (T)0) + x - v;
  const T total = s_warp[nw - 1];
  __syncthreads();
  if (total_out) *total_out = total;
  return before;
}

// out[i] = sum_{j<i} popcount(bits[j]) for i in [0, n]; returns the total.
__device__ __forceinline__ uint32_t block_exclusive_scan_popc(const uint64_t* bits, uint32_t* out, int n) {
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int lo = threadIdx.x * per, hi = min(n, lo + per);
  uint32_t local = 0;
  for (int i = lo; i < hi; ++i) local += (uint32_t)__popcll(bits[i]);
  uint32_t total = 0;
  uint32_t run = block_exclusive_scan<uint32_t>(local, &total);
  for (int i = lo; i < hi; ++i) {
    out[i] = run;
    run += (uint32_t)__popcll(bits[i]);
  }
  if (threadIdx.x == 0) out[n] = total;
  __syncthreads();
  return total;
}

// In-place exclusive scan of a[0..n) (uint64, wrapping).
__device__ __forceinline__ void block_exclusive_scan_u64(unsigned long long* a, uint32_t n) {
  const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
  const uint32_t lo = threadIdx.x * per, hi = min(n, lo + per);
  uint64_t local = 0;
  for (uint32_t i = lo; i < hi; ++i) local += a[i];
  uint64_t run = block_exclusive_scan<uint64_t>(local);
  for (uint32_t i = lo; i < hi; ++i) {
    const uint64_t v = a[i];
    a[i] = run;
    run += v;
  }
  __syncthreads();
}

// ------------------------------------------------------------------ device scan
// Kernels below have internal linkage: every translation unit that includes this
// header gets its own copy.
namespace {
constexpr int kScanThreads = 512;
constexpr int kScanPer = 8;
constexpr int64_t kScanTile = (int64_t)kScanThreads * kScanPer;

inline size_t scan_tmp_bytes(size_t n) { return ((n + kScanTile - 1) / kScanTile + 1) * 8; }

__global__ void k_scan_reduce(const int64_t* __restrict__ x, int64_t n, int64_t* __restrict__ part) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  uint64_t s = 0;
  for (int j = 0; j < kScanPer; ++j) {
    const int64_t i = base + (int64_t)j * kScanThreads + threadIdx.x;
    if (i < n) s += (uint64_t)x[i];
  }
  uint64_t total = 0;
  block_exclusive_scan<uint64_t>(s, &total);
  if (threadIdx.x == 0) part[blockIdx.x] = (int64_t)total;
}
__global__ void k_scan_parts(int64_t* part, int64_t np) {
  // single CTA: exclusive scan of the tile totals in place
  uint64_t carry = 0;
  for (int64_t c0 = 0; c0 < np; c0 += blockDim.x) {
    const int64_t i = c0 + threadIdx.x;
    const uint64_t v = i < np ? (uint64_t)part[i] : 0;
    uint64_t total = 0;
    const uint64_t ex = block_exclusive_scan<uint64_t>(v, &total);
    if (i < np) part[i] = (int64_t)(carry + ex);
    carry += total;
  }
}
__global__ void k_scan_apply(int64_t* __restrict__ x, int64_t n, const int64_t* __restrict__ part) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
  uint64_t v[kScanPer];
  uint64_t s = 0;
#pragma unroll
  for (int j = 0; j < kScanPer; ++j) {
    const int64_t i = base + j;
    v[j] = i < n ? (uint64_t)x[i] : 0;
    s += v[j];
  }
  uint64_t run = block_exclusive_scan<uint64_t>(s) + (uint64_t)part[blockIdx.x];
#pragma unroll
  for (int j = 0; j < kScanPer; ++j) {
    const int64_t i = base + j;
    run += v[j];
    if (i < n) x[i] = (int64_t)run;
  }
}

// Inclusive scan of x[0..n) in place (three launches, counted into `kernels`).
inline int device_inclusive_scan_i64(int64_t* x, int64_t n, int64_t* tmp, cudaStream_t st, int& kernels) {
  if (n <= 0) return 0;
  const int64_t np = (n + kScanTile - 1) / kScanTile;
  k_scan_reduce<<<(unsigned)np, kScanThreads, 0, st>>>(x, n, tmp);
  k_scan_parts<<<1, 1024, 0, st>>>(tmp, np);
  k_scan_apply<<<(unsigned)np, kScanThreads, 0, st>>>(x, n, tmp);
  kernels += 3;
  return (int)cudaGetLastError();
}

}  // namespace
}  // namespace bw
