// bw_v7.cu -- drop-in GB300 implementation of the reference's GPU v7 C ABI
// (gpu_v7.h:49-50): the same plan arrays in, the same lvals / dV / answers out.
//
// Kernel design (not the reference's): one CTA of 512 threads per state block.
//  * Row edits touch at most two classes; one warp applies them.
//  * A factor edit's merged support (batch_engine_v7.hpp:1578-1629) is spread over
//    all threads; each support class gets one Fenwick point update (32-bit-pair
//    shared atomics, bw_common.cuh), instead of writing the dense leaf and
//    rebuilding the whole Fenwick tree in O(C) as gpu_v7.cu:41-71 does.
//  * The dense block leaf delta lives directly in the caller's dV row (global
//    memory), so shared memory holds only the Fenwick tree and the factor vector
//    and the class domain can reach ~28k classes instead of ~6k.
//  * The next node is prefetched into registers while the current one is applied.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "bw_gpu.h"
#include "bw_common.cuh"

namespace bw {

constexpr int kV7Threads = 512;
constexpr int kV7SmemLimit = 232448 - 1024;

__global__ void __launch_bounds__(kV7Threads) k_v7_block(GpuV7Args a) {
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned long long* fen = reinterpret_cast<unsigned long long*>(smem);   // Cpfx
  int64_t* fac = reinterpret_cast<int64_t*>(fen + a.Cpfx);                  // G
  const int b = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const int Cpfx = a.Cpfx, ncls = a.ncls, G = a.G, q = a.q;
  int64_t* leaf = a.dV + (size_t)b * Cpfx;
  for (int i = tid; i < Cpfx; i += nt) { fen[i] = 0; leaf[i] = 0; }
  for (int i = tid; i < G; i += nt) fac[i] = a.fac_start[(size_t)b * G + i];
  __syncthreads();
  const int v0 = a.block_v0[b], v1 = a.block_v1[b];
  const int64_t* need = a.need_off + (size_t)b * G;
  GpuV7Node nxt;
  if (v0 < v1) nxt = a.nodes[v0];
  for (int v = v0; v < v1; ++v) {
    const GpuV7Node p = nxt;
    if (v + 1 < v1) nxt = a.nodes[v + 1];
    if (p.kind == 1) {
      // lane 0 removes the old row image, lane 1 adds the new one (distinct
      // leaf/devbuf cells unless old == new, which the atomics tolerate)
      if (tid < 32) {
        const bool is_old = tid == 0, is_new = tid == 1;
        bool act = false;
        uint32_t c1 = 0;
        uint64_t w = 0;
        if (is_old && p.ex_old && p.amt_old != 0) {
          act = true;
          c1 = (uint32_t)p.c_old + 1u;
          w = (uint64_t)0 - (uint64_t)fac[p.g_old] * (uint64_t)p.amt_old;
          atomicAdd(reinterpret_cast<unsigned long long*>(leaf + c1), (unsigned long long)w);
          const int64_t off = need[p.g_old];
          if (off >= 0) atomicAdd(reinterpret_cast<unsigned long long*>(a.devbuf + off + p.ti_old),
                                  (unsigned long long)((uint64_t)0 - (uint64_t)p.amt_old));
        } else if (is_new && p.ex_new && p.amt_new != 0) {
          act = true;
          c1 = (uint32_t)p.c_new + 1u;
          w = (uint64_t)fac[p.g_new] * (uint64_t)p.amt_new;
          atomicAdd(reinterpret_cast<unsigned long long*>(leaf + c1), (unsigned long long)w);
          const int64_t off = need[p.g_new];
          if (off >= 0) atomicAdd(reinterpret_cast<unsigned long long*>(a.devbuf + off + p.ti_new),
                                  (unsigned long long)p.amt_new);
        }
        if (act) fenwick_add(fen, (uint32_t)ncls, c1, w);
      }
      __syncthreads();
    } else if (p.kind == 2) {
      const int g = p.g_old;
      const int row = a.g2row[g];
      const int64_t off = need[g];
      const uint64_t ds = (uint64_t)p.fac_val - (uint64_t)p.fac_prev;
      if (row >= 0 && off >= 0 && ds != 0) {
        const int kb = a.ms_off[row], ke = a.ms_off[row + 1];
        for (int k0 = kb; k0 < ke; k0 += nt) {
          const int k = k0 + tid;
          bool act = false;
          uint32_t c1 = 0;
          uint64_t d = 0;
          if (k < ke) {
            const int di = a.ms_dev[k];
            const uint64_t dev = di >= 0 ? (uint64_t)a.devbuf[off + di] : 0;
            d = ds * ((uint64_t)a.ms_base[k] + dev);
            if (d != 0) {
              act = true;
              c1 = (uint32_t)a.ms_cls[k] + 1u;
              leaf[c1] = (int64_t)((uint64_t)leaf[c1] + d);  // support classes are distinct
            }
          }
          if (act) fenwick_add(fen, (uint32_t)ncls, c1, d);
        }
      }
      __syncthreads();
      if (tid == 0) fac[g] = p.fac_val;
      __syncthreads();
    }
    for (int e = tid; e < 2 * q; e += nt) {
      const int kk = e >> 1;
      const int idx = (e & 1) ? a.qhb[(size_t)v * q + kk] : a.qlb[(size_t)v * q + kk];
      a.lvals[(size_t)(v - 1) * (size_t)(2 * q) + e] = (int64_t)fenwick_prefix(fen, (uint32_t)idx);
    }
    __syncthreads();
  }
}

__global__ void k_v7_combine(GpuV7CombineArgs a) {
  const int64_t total = (int64_t)a.nstates * a.q;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int v = (int)(i / a.q) + 1, k = (int)(i % a.q);
    const int64_t* cp = a.carrypref + (size_t)a.bidx[v] * a.Cpfx;
    const int lo = a.qlb[(size_t)v * a.q + k], hi = a.qhb[(size_t)v * a.q + k];
    const uint64_t base = (uint64_t)cp[hi] - (uint64_t)cp[lo];
    a.answers[i] = (int64_t)(base + ((uint64_t)a.lvals[2 * i + 1] - (uint64_t)a.lvals[2 * i]));
  }
}

// Column pass of the carry: vstart_b[k] for every block, written into carrypref.
__global__ void k_v7_vstart(int B, int Cpfx, const int64_t* vbase, const int64_t* dV, int64_t* cp) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < Cpfx; k += gridDim.x * blockDim.x) {
    uint64_t run = k ? (uint64_t)vbase[k] : 0;
    for (int b = 0; b < B; ++b) {
      cp[(size_t)b * Cpfx + k] = (int64_t)run;
      if (k) run += (uint64_t)dV[(size_t)b * Cpfx + k];
    }
  }
}
// Row pass: carrypref[b][k] = sum_{j=1..k} vstart_b[j], carrypref[b][0] = 0.
__global__ void k_v7_rowscan(int Cpfx, int64_t* cp) {
  int64_t* row = cp + (size_t)blockIdx.x * Cpfx;
  uint64_t carry = 0;
  for (int c0 = 0; c0 < Cpfx; c0 += blockDim.x) {
    const int k = c0 + threadIdx.x;
    const uint64_t v = (k < Cpfx && k > 0) ? (uint64_t)row[k] : 0;
    uint64_t total = 0;
    const uint64_t ex = block_exclusive_scan<uint64_t>(v, &total);
    if (k < Cpfx) row[k] = (int64_t)(carry + ex + v);
    carry += total;
  }
}

static int v7_report(cudaError_t e, const char* what) {
  if (e != cudaSuccess) std::fprintf(stderr, "gpu: %s failed: %s\n", what, cudaGetErrorString(e));
  return (int)e;
}

}  // namespace bw

using namespace bw;

extern "C" int gpu_v7_launch(const GpuV7Args* a) {
  if (!a || a->B < 1 || a->Cpfx < 1 || a->ncls < 0 || a->ncls + 1 > a->Cpfx || a->G < 1 || a->q < 1)
    return BW_EINVAL;
  const size_t smem = ((size_t)a->Cpfx + (size_t)a->G) * 8;
  if (smem > (size_t)kV7SmemLimit) {
    std::fprintf(stderr, "gpu: Cpfx=%d G=%d exceed the shared-memory budget (%zu > %d bytes)\n", a->Cpfx,
                 a->G, smem, kV7SmemLimit);
    return BW_EINVAL;
  }
  static bool attr_done = false;
  if (!attr_done) {
    int rc = v7_report(cudaFuncSetAttribute(k_v7_block, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            kV7SmemLimit), "func attr");
    if (rc) return rc;
    attr_done = true;
  }
  k_v7_block<<<a->B, kV7Threads, smem>>>(*a);
  return v7_report(cudaGetLastError(), "gpu_v7_launch");
}

extern "C" int gpu_combine_launch(const GpuV7CombineArgs* a) {
  if (!a || a->nstates < 0 || a->q < 1) return BW_EINVAL;
  const int64_t total = (int64_t)a->nstates * a->q;
  if (total == 0) return 0;
  const int blocks = (int)((total + 255) / 256 < 65535 ? (total + 255) / 256 : 65535);
  k_v7_combine<<<blocks, 256>>>(*a);
  return v7_report(cudaGetLastError(), "gpu_combine_launch");
}

extern "C" int bw_v7_carry_launch(int B, int Cpfx, const int64_t* vbase, const int64_t* dV,
                                  int64_t* carrypref, void* stream) {
  if (B < 1 || Cpfx < 1 || !vbase || !dV || !carrypref) return BW_EINVAL;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_v7_vstart<<<(Cpfx + 255) / 256, 256, 0, st>>>(B, Cpfx, vbase, dV, carrypref);
  int rc = v7_report(cudaGetLastError(), "carry column pass");
  if (rc) return rc;
  k_v7_rowscan<<<B, 1024, 0, st>>>(Cpfx, carrypref);
  return v7_report(cudaGetLastError(), "carry row pass");
}
