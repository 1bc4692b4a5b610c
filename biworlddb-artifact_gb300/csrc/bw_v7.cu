// bw_v7.cu -- drop-in GB300 implementation of the reference's GPU v7 C ABIs
// (gpu_v7.h:49-50, gpu_v7b.h:50-52, gpu_session.h:21-24): the same plan arrays in,
// the same lvals / dV / devbuf / answers out.
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
//  * Runs of up to 32 nodes without a factor edit are applied as one batch (warp 0,
//    one lane per node), and each of their queries subtracts the batch's later
//    updates below its bound: two barriers per batch instead of two per node.
//  * One kernel body serves the 56-byte node (gpu_v7.h), the 40-byte compact node
//    (gpu_v7b.h, gpu_session.h) and the session form, whose Fenwick tree and leaf
//    live in caller-owned global memory (any class domain).
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "bw_gpu.h"
#include "bw_common.cuh"

namespace bw {

constexpr int kV7Threads = 512;
constexpr int kV7Batch = 32;                  // nodes per batch (one warp's lanes)
constexpr int kV7SmemLimit = 232448 - 2048;   // dynamic shared memory; the batch arrays are static

// One plan for the three node encodings of the drop-in ABIs (gpu_v7.h, gpu_v7b.h,
// gpu_session.h): the kernel argument.
struct V7Run {
  int B, G, Cpfx, ncls, q;
  const void* nodes;
  const int32_t *v0, *v1;
  const int64_t* fac_start;
  const int32_t* g2row;
  const int32_t* ms_off;
  const int64_t *ms_cls, *ms_base;
  const int32_t* ms_dev;
  int64_t* devbuf;
  const int64_t* need_off;
  const int32_t *qlb, *qhb;
  int64_t *lvals, *dV;
  int64_t *gfen, *gleaf;   // session form: per-block Fenwick tree and leaf in global memory
};

struct NodeView {
  int kind;
  bool ex_old, ex_new;
  int g_old, c_old, ti_old, g_new, c_new, ti_new;
  int64_t amt_old, amt_new, fac_val, fac_prev;
};
__device__ __forceinline__ NodeView view_node(const GpuV7Node& n) {
  return NodeView{n.kind, n.ex_old != 0, n.ex_new != 0, n.g_old, n.c_old, n.ti_old, n.g_new, n.c_new, n.ti_new,
                  n.amt_old, n.amt_new, n.fac_val, n.fac_prev};
}
// compact node (gpu_v7b.h:6-12): kind bits 1 row / 2 factor, bit 2 ex_old, bit 3 ex_new;
// (a, b) = (amt_old, amt_new) for a row edit, (fac_val, fac_prev) for a factor edit
__device__ __forceinline__ NodeView view_node(const GpuV7bNode& n) {
  const int k = n.kind & 3;
  return NodeView{k, (n.kind & 4) != 0, (n.kind & 8) != 0, n.g_old, n.c_old, n.ti_old, n.g_new, n.c_new, n.ti_new,
                  k == 1 ? n.a : 0, k == 1 ? n.b : 0, k == 2 ? n.a : 0, k == 2 ? n.b : 0};
}

// Fenwick point update / prefix in shared memory (exact 32-bit-pair atomics) or in
// global memory (64-bit atomics; reads bypass L1, which the atomics do not update).
template <bool GLOBAL>
__device__ __forceinline__ void fen_add(unsigned long long* fen, uint32_t n, uint32_t i, uint64_t d) {
  if (GLOBAL) {
    for (; i <= n; i += i & (0u - i)) atomicAdd(fen + i, (unsigned long long)d);
  } else {
    fenwick_add(fen, n, i, d);
  }
}
template <bool GLOBAL>
__device__ __forceinline__ uint64_t fen_prefix(const unsigned long long* fen, uint32_t r) {
  uint64_t s = 0;
  for (uint32_t i = r; i; i &= i - 1) s += GLOBAL ? (uint64_t)__ldcg(fen + i) : (uint64_t)fen[i];
  return s;
}

template <typename Node, bool GLOBAL>
__global__ void __launch_bounds__(kV7Threads) k_v7_block(V7Run a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int b = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const int Cpfx = a.Cpfx, ncls = a.ncls, G = a.G, q = a.q;
  unsigned long long* fen = GLOBAL ? reinterpret_cast<unsigned long long*>(a.gfen + (size_t)b * Cpfx)
                                   : reinterpret_cast<unsigned long long*>(smem);
  int64_t* fac = reinterpret_cast<int64_t*>(smem + (GLOBAL ? 0 : (size_t)Cpfx * 8));   // G
  int64_t* leaf = (GLOBAL ? a.gleaf : a.dV) + (size_t)b * Cpfx;
  for (int i = tid; i < Cpfx; i += nt) { fen[i] = 0; leaf[i] = 0; }
  for (int i = tid; i < G; i += nt) fac[i] = a.fac_start[(size_t)b * G + i];
  __syncthreads();
  const Node* nodes = static_cast<const Node*>(a.nodes);
  const int v0 = a.v0[b], v1 = a.v1[b];
  const int64_t* need = a.need_off + (size_t)b * G;
  // A run of up to 32 consecutive nodes without a factor edit is one batch: warp 0
  // applies all of their row updates at once (the Fenwick sums commute), then every
  // query of node j reads the Fenwick prefix and takes back the updates of the
  // batch's later nodes that fall below its bound.  Two barriers per batch instead of
  // two per node; a factor edit is a batch of its own.
  __shared__ uint32_t upd_c1[2 * kV7Batch];   // 1-based class of each update, or ~0u for none
  __shared__ unsigned long long upd_w[2 * kV7Batch];
  __shared__ int batch_len;
  for (int v = v0; v < v1;) {
    if (tid < 32) {
      const int i = v + tid;
      const bool in = tid < kV7Batch && i < v1;
      NodeView p{};
      if (in) p = view_node(nodes[i]);
      const unsigned fac_mask = __ballot_sync(0xffffffffu, in && p.kind == 2);
      const unsigned in_mask = __ballot_sync(0xffffffffu, in);
      // a leading factor edit forms a batch of one; else the run before the first one
      const int k = (fac_mask & 1u) ? 1 : (fac_mask ? __ffs(fac_mask) - 1 : __popc(in_mask));
      if (tid == 0) batch_len = k;
      if (!(fac_mask & 1u) && tid < k) {
        uint32_t c_old = ~0u, c_new = ~0u;
        uint64_t w_old = 0, w_new = 0;
        if (p.kind == 1) {
          if (p.ex_old && p.amt_old != 0) {
            c_old = (uint32_t)p.c_old + 1u;
            w_old = (uint64_t)0 - (uint64_t)fac[p.g_old] * (uint64_t)p.amt_old;
            atomicAdd(reinterpret_cast<unsigned long long*>(leaf + c_old), (unsigned long long)w_old);
            const int64_t off = need[p.g_old];
            if (off >= 0) atomicAdd(reinterpret_cast<unsigned long long*>(a.devbuf + off + p.ti_old),
                                    (unsigned long long)((uint64_t)0 - (uint64_t)p.amt_old));
            fen_add<GLOBAL>(fen, (uint32_t)ncls, c_old, w_old);
          }
          if (p.ex_new && p.amt_new != 0) {
            c_new = (uint32_t)p.c_new + 1u;
            w_new = (uint64_t)fac[p.g_new] * (uint64_t)p.amt_new;
            atomicAdd(reinterpret_cast<unsigned long long*>(leaf + c_new), (unsigned long long)w_new);
            const int64_t off = need[p.g_new];
            if (off >= 0) atomicAdd(reinterpret_cast<unsigned long long*>(a.devbuf + off + p.ti_new),
                                    (unsigned long long)p.amt_new);
            fen_add<GLOBAL>(fen, (uint32_t)ncls, c_new, w_new);
          }
        }
        upd_c1[2 * tid] = c_old;
        upd_w[2 * tid] = w_old;
        upd_c1[2 * tid + 1] = c_new;
        upd_w[2 * tid + 1] = w_new;
      }
    }
    __syncthreads();
    const int k = batch_len;
    const NodeView f = view_node(nodes[v]);
    if (k == 1 && f.kind == 2) {
      const int g = f.g_old;
      const int row = a.g2row[g];
      const int64_t off = need[g];
      const uint64_t ds = (uint64_t)f.fac_val - (uint64_t)f.fac_prev;
      if (row >= 0 && off >= 0 && ds != 0) {
        const int kb = a.ms_off[row], ke = a.ms_off[row + 1];
        for (int k0 = kb; k0 < ke; k0 += nt) {
          const int kk = k0 + tid;
          bool act = false;
          uint32_t c1 = 0;
          uint64_t d = 0;
          if (kk < ke) {
            const int di = a.ms_dev[kk];
            // devbuf and leaf cells are also updated by global atomics (row edits),
            // which do not update L1: read them from L2
            const uint64_t dev = di >= 0 ? (uint64_t)__ldcg(a.devbuf + off + di) : 0;
            d = ds * ((uint64_t)a.ms_base[kk] + dev);
            if (d != 0) {
              act = true;
              c1 = (uint32_t)a.ms_cls[kk] + 1u;
              leaf[c1] = (int64_t)((uint64_t)__ldcg(leaf + c1) + d);  // support classes are distinct
            }
          }
          if (act) fen_add<GLOBAL>(fen, (uint32_t)ncls, c1, d);
        }
      }
      __syncthreads();
      if (tid == 0) fac[g] = f.fac_val;
      for (int e = tid; e < 2 * q; e += nt) {
        const int idx = (e & 1) ? a.qhb[(size_t)v * q + (e >> 1)] : a.qlb[(size_t)v * q + (e >> 1)];
        a.lvals[(size_t)(v - 1) * (size_t)(2 * q) + e] = (int64_t)fen_prefix<GLOBAL>(fen, (uint32_t)idx);
      }
    } else {
      // queries of the batch's nodes: the prefix after the whole batch, less the later
      // nodes' updates at or below the bound
      for (int e = tid; e < k * 2 * q; e += nt) {
        const int j = e / (2 * q), r = e - j * (2 * q);
        const int vv = v + j;
        const int idx = (r & 1) ? a.qhb[(size_t)vv * q + (r >> 1)] : a.qlb[(size_t)vv * q + (r >> 1)];
        uint64_t val = fen_prefix<GLOBAL>(fen, (uint32_t)idx);
        for (int u = 2 * (j + 1); u < 2 * k; ++u)
          if (upd_c1[u] <= (uint32_t)idx) val -= upd_w[u];
        a.lvals[(size_t)(vv - 1) * (size_t)(2 * q) + r] = (int64_t)val;
      }
    }
    __syncthreads();
    v += k;
  }
  if (GLOBAL && a.dV)   // the session form also reports the block's leaf delta in dV
    for (int i = tid; i < Cpfx; i += nt) a.dV[(size_t)b * Cpfx + i] = __ldcg(leaf + i);
}

// Block-start deviation snapshots on the device (the v7b/session snapshot entries):
// every row edit adds its deviation delta into the region of each later block that
// needs the edited group.
__global__ void k_v7_snap(int nstates, const GpuV7bNode* nodes, const int32_t* bidx, const int32_t* gb_off,
                          const int32_t* gb_block, const int64_t* gb_reg, int64_t* devbuf) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x + 1; v < nstates; v += gridDim.x * blockDim.x) {
    const GpuV7bNode n = nodes[v];
    if ((n.kind & 3) != 1) continue;
    const int b0 = bidx[v];
    auto scatter = [&](int g, int ti, uint64_t d) {
      // a group's occurrences are in ascending block order: skip to the first later block
      int lo = gb_off[g], hi = gb_off[g + 1];
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (gb_block[mid] > b0) hi = mid; else lo = mid + 1;
      }
      for (int at = lo; at < gb_off[g + 1]; ++at)
        atomicAdd(reinterpret_cast<unsigned long long*>(devbuf + gb_reg[at] + ti), (unsigned long long)d);
    };
    if (n.kind & 4) scatter(n.g_old, n.ti_old, (uint64_t)0 - (uint64_t)n.a);
    if (n.kind & 8) scatter(n.g_new, n.ti_new, (uint64_t)n.b);
  }
}

__global__ void k_zero2(int64_t* x, int64_t* y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = 0;
    y[i] = 0;
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

namespace bw {
namespace {

template <typename Args>
V7Run v7_run(const Args& a, const void* nodes, const int32_t* v0, const int32_t* v1) {
  V7Run r{};
  r.B = a.B; r.G = a.G; r.Cpfx = a.Cpfx; r.ncls = a.ncls; r.q = a.q;
  r.nodes = nodes; r.v0 = v0; r.v1 = v1; r.fac_start = a.fac_start; r.g2row = a.g2row;
  r.ms_off = a.ms_off; r.ms_cls = a.ms_cls; r.ms_base = a.ms_base; r.ms_dev = a.ms_dev;
  r.devbuf = a.devbuf; r.need_off = a.need_off; r.qlb = a.qlb; r.qhb = a.qhb; r.lvals = a.lvals; r.dV = a.dV;
  return r;
}

bool v7_dims_ok(int B, int G, int Cpfx, int ncls, int q) {
  return B >= 1 && Cpfx >= 1 && ncls >= 0 && ncls + 1 <= Cpfx && G >= 1 && q >= 1;
}

template <typename Node, bool GLOBAL>
int v7_block_launch(const V7Run& r, const char* what) {
  const size_t smem = ((GLOBAL ? 0 : (size_t)r.Cpfx) + (size_t)r.G) * 8;
  if (smem > (size_t)kV7SmemLimit) {
    std::fprintf(stderr, "gpu: Cpfx=%d G=%d exceed the shared-memory budget (%zu > %d bytes)%s\n", r.Cpfx, r.G,
                 smem, kV7SmemLimit, GLOBAL ? "" : "; the session entries keep the prefix in global memory");
    return BW_EINVAL;
  }
  static bool attr_done = false;   // one-time, not thread-safe (as the reference's, gpu_v7.cu:100-106)
  if (!attr_done) {
    int rc = v7_report(cudaFuncSetAttribute(k_v7_block<Node, GLOBAL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            kV7SmemLimit), "func attr");
    if (rc) return rc;
    attr_done = true;
  }
  k_v7_block<Node, GLOBAL><<<r.B, kV7Threads, smem>>>(r);
  return v7_report(cudaGetLastError(), what);
}

int snap_launch(int nstates, const GpuV7bNode* nodes, const int32_t* bidx, const int32_t* gb_off,
                const int32_t* gb_block, const int64_t* gb_reg, int64_t* devbuf, const char* what) {
  if (nstates < 1 || !nodes || !bidx || !gb_off || !devbuf) return BW_EINVAL;
  if (nstates < 2) return 0;
  const int threads = 256, blocks = (nstates - 1 + threads - 1) / threads;
  k_v7_snap<<<blocks < 65535 ? blocks : 65535, threads>>>(nstates, nodes, bidx, gb_off, gb_block, gb_reg, devbuf);
  return v7_report(cudaGetLastError(), what);
}

}  // namespace
}  // namespace bw

extern "C" int gpu_v7_launch(const GpuV7Args* a) {
  if (!a || !v7_dims_ok(a->B, a->G, a->Cpfx, a->ncls, a->q)) return BW_EINVAL;
  return v7_block_launch<GpuV7Node, false>(v7_run(*a, a->nodes, a->block_v0, a->block_v1), "gpu_v7_launch");
}

extern "C" int gpu_v7b_launch(const GpuV7bArgs* a) {
  if (!a || !v7_dims_ok(a->B, a->G, a->Cpfx, a->ncls, a->q)) return BW_EINVAL;
  return v7_block_launch<GpuV7bNode, false>(v7_run(*a, a->nodes, a->bv0, a->bv1), "gpu_v7b_launch");
}

extern "C" int gpu_v7b_snap_launch(const GpuV7bSnapArgs* a) {
  if (!a) return BW_EINVAL;
  return snap_launch(a->nstates, a->nodes, a->bidx, a->gb_off, a->gb_block, a->gb_reg, a->devbuf,
                     "gpu_v7b_snap_launch");
}

extern "C" int gpu_v7b_combine_launch(const GpuV7bCombineArgs* a) {
  static_assert(sizeof(GpuV7bCombineArgs) == sizeof(GpuV7CombineArgs), "combine layouts");
  return gpu_combine_launch(reinterpret_cast<const GpuV7CombineArgs*>(a));
}

extern "C" int gpu_sess_reset_launch(const GpuSessResetArgs* a) {
  if (!a || a->B < 1 || a->Cpfx < 1 || !a->fen || !a->leaf) return BW_EINVAL;
  const int64_t n = (int64_t)a->B * a->Cpfx;
  const int64_t blocks = (n + 255) / 256;
  k_zero2<<<(unsigned)(blocks < 65535 ? blocks : 65535), 256>>>(a->fen, a->leaf, n);
  return v7_report(cudaGetLastError(), "gpu_sess_reset_launch");
}

extern "C" int gpu_sess_run_launch(const GpuSessRunArgs* a) {
  static_assert(sizeof(GpuSessNode) == sizeof(GpuV7bNode), "session node layout");
  if (!a || !v7_dims_ok(a->B, a->G, a->Cpfx, a->ncls, a->q) || !a->fen || !a->leaf) return BW_EINVAL;
  V7Run r = v7_run(*a, a->nodes, a->bv0, a->bv1);
  r.gfen = a->fen;
  r.gleaf = a->leaf;
  return v7_block_launch<GpuV7bNode, true>(r, "gpu_sess_run_launch");
}

extern "C" int gpu_sess_snap_launch(const GpuSessSnapArgs* a) {
  if (!a) return BW_EINVAL;
  return snap_launch(a->nstates, reinterpret_cast<const GpuV7bNode*>(a->nodes), a->bidx, a->gb_off, a->gb_block,
                     a->gb_reg, a->devbuf, "gpu_sess_snap_launch");
}

extern "C" int gpu_sess_combine_launch(const GpuSessCombineArgs* a) {
  static_assert(sizeof(GpuSessCombineArgs) == sizeof(GpuV7CombineArgs), "combine layouts");
  return gpu_combine_launch(reinterpret_cast<const GpuV7CombineArgs*>(a));
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
