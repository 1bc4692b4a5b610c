// bw_expand.cu -- the factor expansion of a reference-native chain on the device
// (bw_native_expand, include/bw_gpu.h).
//
// A factor edit of group g at state v sets g's multiplier from m to m + ds; in the
// event model it becomes one event (v, c, ds * mass_g(v)[c]) for every class c of
// g's support, where mass_g(v) is the group's live amount per class just before v
// (the reference's per-group Fenwick rebuild, batch_engine_v7.hpp:1311-1340, and its
// base scan, :1350-1415, become this one pass).  For a chain, mass_g(v) is the
// base mass plus every row-edit update of g at states below v, so each group is an
// independent sequential timeline: k_expand runs one CTA per group, keeps the
// group's mass row in shared memory (global memory for supports past 20,480
// classes), applies the updates between two expansions in parallel (sums commute)
// and writes each expansion as coalesced 16-byte stores at its precomputed output
// range.  k_fixed copies the verbatim events (base rows, row edits) to their
// positions.  All arithmetic is uint64 with wrap, as the host builder's.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "bw_gpu.h"
#include "bw_common.cuh"

namespace bw {
namespace {

constexpr int kExpThreads = 256;
constexpr size_t kExpSmemMass = 160 * 1024;   // shared-memory mass row up to 20,480 classes

struct ExpandParams {
  int32_t G;
  int64_t n_fixed;
  const BwEvent* fixed;
  const int64_t* fixed_pos;
  const int64_t* sup_off;
  const uint32_t* sup_cls;
  const int64_t* base_mass;
  const int64_t* tl_off;
  const BwTimeline* tl;
  unsigned long long* gmass;   // global mass rows, parallel to sup_cls
  BwEvent* out;
  uint32_t smem_classes;       // groups up to this many classes use shared memory
};

__global__ void k_fixed(ExpandParams p) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n_fixed; i += (int64_t)gridDim.x * blockDim.x)
    p.out[p.fixed_pos[i]] = p.fixed[i];
}

__global__ void __launch_bounds__(kExpThreads) k_expand(ExpandParams p) {
  extern __shared__ unsigned long long smass[];
  __shared__ int first_exp;
  const int g = blockIdx.x, tid = threadIdx.x;
  const int64_t s0 = p.sup_off[g], n = p.sup_off[g + 1] - s0;
  const bool in_smem = n <= (int64_t)p.smem_classes;
  unsigned long long* mass = in_smem ? smass : p.gmass + s0;
  for (int64_t i = tid; i < n; i += kExpThreads) mass[i] = (unsigned long long)p.base_mass[s0 + i];
  const int64_t t1 = p.tl_off[g + 1];
  int64_t j = p.tl_off[g];
  __syncthreads();
  while (j < t1) {
    // a chunk of up to kExpThreads records: the updates before its first expansion
    // are applied together, then that expansion is written
    if (tid == 0) first_exp = kExpThreads;
    __syncthreads();
    BwTimeline r;
    const bool have = j + tid < t1;
    if (have) {
      r = p.tl[j + tid];
      if (r.idx < 0) atomicMin(&first_exp, tid);
    }
    __syncthreads();
    const int e = first_exp;
    if (have && tid < e) {
      if (in_smem) shared_add_u64(&mass[r.idx], (uint64_t)r.value);
      else atomicAdd(&mass[r.idx], (unsigned long long)r.value);
    }
    __syncthreads();
    if (e < kExpThreads) {
      const BwTimeline x = p.tl[j + e];
      BwEvent* o = p.out + x.out;
      const uint64_t ds = (uint64_t)x.value;
      for (int64_t i = tid; i < n; i += kExpThreads) {
        const uint64_t m = in_smem ? mass[i] : __ldcg(&mass[i]);
        BwEvent ev;
        ev.state = (uint32_t)x.state;
        ev.key = p.sup_cls[s0 + i];
        ev.delta = (int64_t)(ds * m);
        o[i] = ev;
      }
      __syncthreads();   // every read of this expansion precedes the next updates
      j += e + 1;
    } else {
      j += kExpThreads;
    }
  }
}

size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

struct ExpandLayout {
  size_t fixed, fixed_pos, sup_off, sup_cls, base_mass, tl_off, tl, gmass, total;
};

ExpandLayout expand_layout(const BwNativeCompact* c) {
  const size_t nsup = (size_t)c->sup_off[c->n_groups], ntl = (size_t)c->tl_off[c->n_groups];
  ExpandLayout L;
  size_t o = 0;
  L.fixed = o;      o = al256(o + (size_t)c->n_fixed * sizeof(BwEvent));
  L.fixed_pos = o;  o = al256(o + (size_t)c->n_fixed * 8);
  L.sup_off = o;    o = al256(o + ((size_t)c->n_groups + 1) * 8);
  L.sup_cls = o;    o = al256(o + nsup * 4);
  L.base_mass = o;  o = al256(o + nsup * 8);
  L.tl_off = o;     o = al256(o + ((size_t)c->n_groups + 1) * 8);
  L.tl = o;         o = al256(o + ntl * sizeof(BwTimeline));
  L.gmass = o;      o = al256(o + nsup * 8);
  L.total = o;
  return L;
}

int expand_report(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return 0;
  std::fprintf(stderr, "bw_native_expand: %s: %s\n", what, cudaGetErrorString(e));
  return (int)e;   // the failing call's cudaError_t, as every entry of this library
}

bool compact_ok(const BwNativeCompact* c) {
  return c && c->n_groups >= 1 && c->n_events >= 0 && c->n_fixed >= 0 && c->sup_off && c->tl_off &&
         (c->n_fixed == 0 || (c->fixed && c->fixed_pos)) && c->sup_off[0] == 0 && c->tl_off[0] == 0 &&
         (c->sup_off[c->n_groups] == 0 || (c->sup_cls && c->base_mass)) && (c->tl_off[c->n_groups] == 0 || c->tl);
}

}  // namespace
}  // namespace bw

using namespace bw;

extern "C" int bw_native_expand_workspace(const BwNativeCompact* c, size_t* bytes) {
  if (!compact_ok(c) || !bytes) return BW_EINVAL;
  *bytes = expand_layout(c).total;
  return 0;
}

extern "C" int bw_native_expand(const BwNativeCompact* c, BwEvent* events, void* workspace, size_t workspace_bytes,
                                void* stream) {
  if (!compact_ok(c) || (c->n_events && !events)) return BW_EINVAL;
  const ExpandLayout L = expand_layout(c);
  if (!workspace || workspace_bytes < L.total) return BW_EINVAL;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* ws = static_cast<char*>(workspace);
  const size_t G = (size_t)c->n_groups, nsup = (size_t)c->sup_off[G], ntl = (size_t)c->tl_off[G];
  struct Copy {
    size_t off;
    const void* src;
    size_t bytes;
  } copies[] = {{L.fixed, c->fixed, (size_t)c->n_fixed * sizeof(BwEvent)},
                {L.fixed_pos, c->fixed_pos, (size_t)c->n_fixed * 8},
                {L.sup_off, c->sup_off, (G + 1) * 8},
                {L.sup_cls, c->sup_cls, nsup * 4},
                {L.base_mass, c->base_mass, nsup * 8},
                {L.tl_off, c->tl_off, (G + 1) * 8},
                {L.tl, c->tl, ntl * sizeof(BwTimeline)}};
  int rc = 0;
  for (const Copy& x : copies)
    if (x.bytes && (rc = expand_report(cudaMemcpyAsync(ws + x.off, x.src, x.bytes, cudaMemcpyHostToDevice, st),
                                       "upload")))
      return rc;
  int64_t max_n = 0;
  for (size_t g = 0; g < G; ++g) max_n = max_n > c->sup_off[g + 1] - c->sup_off[g] ? max_n : c->sup_off[g + 1] - c->sup_off[g];
  const size_t smem_classes = kExpSmemMass / 8;
  const size_t smem = (size_t)(max_n < (int64_t)smem_classes ? max_n : (int64_t)smem_classes) * 8;
  static bool attr = false;   // one-time, as the other launches' attributes
  if (!attr) {
    if ((rc = expand_report(cudaFuncSetAttribute(k_expand, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)kExpSmemMass), "attribute")))
      return rc;
    attr = true;
  }
  ExpandParams p;
  p.G = c->n_groups;
  p.n_fixed = c->n_fixed;
  p.fixed = reinterpret_cast<const BwEvent*>(ws + L.fixed);
  p.fixed_pos = reinterpret_cast<const int64_t*>(ws + L.fixed_pos);
  p.sup_off = reinterpret_cast<const int64_t*>(ws + L.sup_off);
  p.sup_cls = reinterpret_cast<const uint32_t*>(ws + L.sup_cls);
  p.base_mass = reinterpret_cast<const int64_t*>(ws + L.base_mass);
  p.tl_off = reinterpret_cast<const int64_t*>(ws + L.tl_off);
  p.tl = reinterpret_cast<const BwTimeline*>(ws + L.tl);
  p.gmass = reinterpret_cast<unsigned long long*>(ws + L.gmass);
  p.out = events;
  p.smem_classes = (uint32_t)(smem / 8);
  if (c->n_fixed) {
    const int64_t blocks = (c->n_fixed + 255) / 256;
    k_fixed<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, st>>>(p);
    if ((rc = expand_report(cudaGetLastError(), "fixed launch"))) return rc;
  }
  k_expand<<<(unsigned)G, kExpThreads, smem, st>>>(p);
  return expand_report(cudaGetLastError(), "expand launch");
}
