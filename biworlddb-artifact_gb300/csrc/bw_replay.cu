// bw_replay.cu -- C ABI of the plain (one-tree) event-model replay.
//
// The replay of one version tree is the forest pipeline of bw_pipeline.cu with a
// single tree: the tree's table row is written by the first kernel from the scalar
// arguments, so a launch needs no host-to-device copy and, like the reference's
// gpu_v7_launch (gpu_v7.cu:98-113), only enqueues work on the caller's stream.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <vector>

#include "bw_gpu.h"
#include "bw_common.cuh"
#include "bw_pipeline.cuh"
#include "bw_chain.cuh"

namespace bw {
namespace {

struct LastInfo { int32_t kernels = 0, blocks = 0, chain = 0; };
std::mutex g_info_mu;
LastInfo g_last;

// Stage timing (BW_REPLAY_TIMING): one set of BW_STAGE_COUNT+1 events per timed
// launch since the last reset; sets are kept for reuse across runs.
std::vector<EventSet> g_sets;
size_t g_sets_used = 0;

int validate_args(const BwReplayArgs* a) {
  if (!a || a->n_states < 1 || a->n_events < 0 || a->n_queries < 0 || a->n_keys < 1) return BW_EINVAL;
  if ((int64_t)a->n_states >= ((int64_t)1 << 30)) return BW_EINVAL;
  if (a->n_events >= ((int64_t)1 << 32) || a->n_queries >= ((int64_t)1 << 32)) return BW_EINVAL;
  return 0;
}

int device_sms(int* sms) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev);
  return report(e, "device query");
}

int spec_of(const BwReplayArgs* a, PipeSpec& s) {
  int sms = 0;
  int rc = device_sms(&sms);
  if (rc) return rc;
  return pipe_spec_one(a->n_states, a->n_keys, a->n_events, a->n_queries, a->blocks,
                       (a->flags & BW_REPLAY_CHAIN_HINT) != 0, Tuning(), sms, s);
}

int chain_spec_of(const BwReplayArgs* a, ChainSpec& s) {
  int sms = 0;
  int rc = device_sms(&sms);
  if (rc) return rc;
  return chain_spec(a, sms, s);
}

}  // namespace
}  // namespace bw

using namespace bw;

extern "C" int bw_replay_workspace_size(const BwReplayArgs* a, size_t* bytes) {
  if (validate_args(a) || !bytes) return BW_EINVAL;
  if (chain_selected(a)) {
    ChainSpec cs;
    int rc = chain_spec_of(a, cs);
    if (rc) return rc;
    *bytes = cs.total;
    return 0;
  }
  PipeSpec s;
  int rc = spec_of(a, s);
  if (rc) return rc;
  Layout L;
  pipe_layout(s, L);
  *bytes = L.total;
  return 0;
}

extern "C" int bw_replay_launch(const BwReplayArgs* a) {
  if (validate_args(a) || !a->workspace || !a->parent || (a->n_events && !a->events) ||
      (a->n_queries && (!a->queries || !a->answers)))
    return BW_EINVAL;
  if ((reinterpret_cast<uintptr_t>(a->workspace) & 255) != 0) return BW_EINVAL;
  const bool chain = chain_selected(a);
  PipeSpec s;
  ChainSpec cs;
  int rc = chain ? chain_spec_of(a, cs) : spec_of(a, s);
  if (rc) return rc;
  size_t need = cs.total;
  if (!chain) {
    Layout L;
    pipe_layout(s, L);
    need = L.total;
  }
  if (a->workspace_bytes < need) {
    std::fprintf(stderr, "bw_replay: workspace %zu < required %zu bytes\n", a->workspace_bytes, need);
    return BW_EINVAL;
  }
  EventSet* evs = nullptr;
  if (a->flags & BW_REPLAY_TIMING) {
    if (g_sets_used == g_sets.size()) {
      EventSet es;
      for (auto& ev : es.ev)
        if ((rc = report(cudaEventCreate(&ev), "event create"))) return rc;
      g_sets.push_back(es);
    }
    evs = &g_sets[g_sets_used++];
  }
  int kernels = 0;
  rc = chain ? chain_enqueue(cs, a, evs, &kernels)
             : pipe_enqueue(s, a->workspace, a->parent, a->events, a->queries, a->answers,
                            static_cast<cudaStream_t>(a->stream), evs, &kernels);
  if (rc) return rc;
  std::lock_guard<std::mutex> g(g_info_mu);
  g_last.kernels = kernels;
  g_last.blocks = chain ? cs.B : s.B;
  g_last.chain = chain ? 1 : 0;
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
  const EventSet& last = g_sets[g_sets_used - 1];
  int rc = report(cudaEventSynchronize(last.ev[last.chain ? BW_STAGE_COUNT + 1 : BW_STAGE_COUNT]), "event sync");
  if (rc) return rc;
  for (size_t k = 0; k < g_sets_used; ++k) {
    const EventSet& es = g_sets[k];
    for (int i = 0; i < BW_STAGE_COUNT; ++i) {
      float t = 0.f;
      if (es.chain && i == BW_STAGE_CARRY)   // the chain's carry follows its sweep
        rc = report(cudaEventElapsedTime(&t, es.ev[BW_STAGE_COUNT], es.ev[BW_STAGE_COUNT + 1]), "event elapsed");
      else if (es.chain && i != BW_STAGE_SWEEP)
        t = 0.f;
      else
        rc = report(cudaEventElapsedTime(&t, es.ev[i], es.ev[i + 1]), "event elapsed");
      if (rc) return rc;
      ms[i] += t;
    }
  }
  return 0;
}

extern "C" int bw_replay_status(const BwReplayArgs* a, int32_t* status) {
  if (validate_args(a) || !a->workspace || !status) return BW_EINVAL;
  const int32_t* word = chain_status_word(a->workspace);
  if (!chain_selected(a)) {
    PipeSpec s;
    int rc = spec_of(a, s);
    if (rc) return rc;
    word = pipe_status_word(s, a->workspace);
  }
  cudaStream_t st = static_cast<cudaStream_t>(a->stream);
  int32_t v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, word, 4, cudaMemcpyDeviceToHost, st);
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

extern "C" int bw_replay_path(const BwReplayArgs* a, int32_t* chain) {
  if (validate_args(a) || !chain) return BW_EINVAL;
  *chain = chain_selected(a) ? 1 : 0;
  return 0;
}

extern "C" int bw_device_info(int32_t* sm_count, int32_t* arch_tag) {
  int sms = 0;
  int rc = device_sms(&sms);
  if (rc) return rc;
  if (sm_count) *sm_count = sms;
  if (arch_tag) *arch_tag = BW_ARCH_TAG;
  return 0;
}
