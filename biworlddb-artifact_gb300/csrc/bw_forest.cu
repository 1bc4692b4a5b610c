// bw_forest.cu -- C ABI of the batched forest replay: one plan for thousands of
// independent version trees, launched as one pipeline, captured in a CUDA graph,
// with an autotuner over the block size, the persistent sweep's CTAs per SM and
// the rank-LUT slice width.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "bw_gpu.h"
#include "bw_pipeline.cuh"

using namespace bw;

struct BwForest {
  PipeSpec spec;
  BwForestTuning tuning{};
  std::vector<int64_t> soff, eoff, qoff;
  std::vector<uint32_t> C;
  void* ws = nullptr;
  size_t ws_bytes = 0;
  int kernels = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

int sms_of_device(int* sms) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev);
  return report(e, "device query");
}

Tuning to_tuning(const BwForestTuning* t) {
  Tuning x;
  if (t) {
    x.block_work = t->block_work;
    x.ctas_per_sm = t->ctas_per_sm;
    x.slice_ranks = t->slice_ranks;
    x.tile = t->tile;
  }
  return x;
}

int plan_spec(const BwForestShape* sh, const BwForestTuning* tu, PipeSpec& spec) {
  if (!sh || sh->n_trees < 1 || !sh->state_off || !sh->event_off || !sh->query_off || !sh->n_keys) return BW_EINVAL;
  if (tu && (tu->ctas_per_sm < 0 || tu->ctas_per_sm > 2 || tu->block_work < 0 || tu->slice_ranks < 0 ||
             tu->tile < 0 || tu->tile > kTileMaxId))
    return BW_EINVAL;
  int sms = 0;
  int rc = sms_of_device(&sms);
  if (rc) return rc;
  return pipe_spec_forest(sh->n_trees, sh->state_off, sh->event_off, sh->query_off, sh->n_keys, to_tuning(tu), sms,
                          spec);
}

void drop_graph(BwForest* f) {
  if (f->exec) cudaGraphExecDestroy(f->exec);
  if (f->graph) cudaGraphDestroy(f->graph);
  f->exec = nullptr;
  f->graph = nullptr;
}

// Candidate tunings of the autotuner: CTAs per SM x blocks per CTA at full slice
// width, then narrower slices at the best of those.
std::vector<BwForestTuning> candidates(const BwForestShape* sh, int sms) {
  int64_t W = 0;
  const int32_t T = sh->n_trees;
  for (int32_t t = 0; t < T; ++t)
    W += est_work(sh->state_off[t + 1] - sh->state_off[t], sh->event_off[t + 1] - sh->event_off[t],
                  sh->query_off[t + 1] - sh->query_off[t]);
  std::vector<BwForestTuning> c;
  for (int32_t ctas = 1; ctas <= 2; ++ctas)
    for (int64_t per : {1, 2, 4, 8}) {
      BwForestTuning x{};
      x.ctas_per_sm = ctas;
      x.block_work = W / (per * ctas * (int64_t)sms);
      if (x.block_work < 65536) x.block_work = 65536;
      c.push_back(x);
    }
  return c;
}

}  // namespace

extern "C" int bw_forest_create(const BwForestShape* shape, const BwForestTuning* tuning, BwForest** out) {
  if (!out) return BW_EINVAL;
  *out = nullptr;
  BwForest* f = new BwForest();
  int rc = plan_spec(shape, tuning, f->spec);
  if (rc) {
    delete f;
    return rc;
  }
  if (tuning) f->tuning = *tuning;
  f->tuning.block_work = tuning && tuning->block_work ? tuning->block_work : 0;
  f->tuning.ctas_per_sm = f->spec.ctas_per_sm;
  f->tuning.slice_ranks = tuning ? tuning->slice_ranks : 0;
  f->tuning.tile = f->spec.tile;
  f->tuning.reserved = 0;
  const int32_t T = shape->n_trees;
  f->soff.assign(shape->state_off, shape->state_off + T + 1);
  f->eoff.assign(shape->event_off, shape->event_off + T + 1);
  f->qoff.assign(shape->query_off, shape->query_off + T + 1);
  f->C.assign(shape->n_keys, shape->n_keys + T);
  *out = f;
  return 0;
}

extern "C" int bw_forest_workspace_size(const BwForest* f, size_t* bytes) {
  if (!f || !bytes) return BW_EINVAL;
  Layout L;
  pipe_layout(f->spec, L);
  *bytes = L.total;
  return 0;
}

extern "C" int bw_forest_bind(BwForest* f, void* workspace, size_t workspace_bytes, void* stream) {
  if (!f || !workspace || (reinterpret_cast<uintptr_t>(workspace) & 255) != 0) return BW_EINVAL;
  Layout L;
  pipe_layout(f->spec, L);
  if (workspace_bytes < L.total) {
    std::fprintf(stderr, "bw_forest: workspace %zu < required %zu bytes\n", workspace_bytes, L.total);
    return BW_EINVAL;
  }
  drop_graph(f);
  int rc = pipe_bind(f->spec, workspace, static_cast<cudaStream_t>(stream));
  if (rc) return rc;
  f->ws = workspace;
  f->ws_bytes = workspace_bytes;
  return 0;
}

extern "C" int bw_forest_launch(BwForest* f, const int32_t* parent, const BwEvent* events, const BwQuery* queries,
                                int64_t* answers, void* stream) {
  if (!f || !f->ws || !parent || (f->spec.E && !events) || (f->spec.Q && (!queries || !answers))) return BW_EINVAL;
  return pipe_enqueue(f->spec, f->ws, parent, events, queries, answers, static_cast<cudaStream_t>(stream), nullptr,
                      &f->kernels);
}

extern "C" int bw_forest_capture(BwForest* f, const int32_t* parent, const BwEvent* events, const BwQuery* queries,
                                 int64_t* answers, void* stream) {
  if (!f || !f->ws || !stream || !parent || (f->spec.E && !events) || (f->spec.Q && (!queries || !answers)))
    return BW_EINVAL;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  drop_graph(f);
  int rc = report(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
  if (rc) return rc;
  const int erc = pipe_enqueue(f->spec, f->ws, parent, events, queries, answers, st, nullptr, &f->kernels);
  cudaGraph_t g = nullptr;
  rc = report(cudaStreamEndCapture(st, &g), "end capture");
  if (erc || rc) {
    if (g) cudaGraphDestroy(g);
    return erc ? erc : rc;
  }
  f->graph = g;
  rc = report(cudaGraphInstantiate(&f->exec, g, 0), "graph instantiate");
  if (rc) drop_graph(f);
  return rc;
}

extern "C" int bw_forest_graph_launch(BwForest* f, void* stream) {
  if (!f || !f->exec) return BW_EINVAL;
  return report(cudaGraphLaunch(f->exec, static_cast<cudaStream_t>(stream)), "graph launch");
}

extern "C" int bw_forest_launch_timed(BwForest* f, const int32_t* parent, const BwEvent* events,
                                      const BwQuery* queries, int64_t* answers, void* stream, float* ms) {
  if (!f || !f->ws || !ms || !parent || (f->spec.E && !events) || (f->spec.Q && (!queries || !answers)))
    return BW_EINVAL;
  EventSet es;
  int rc = 0, made = 0;
  for (auto& ev : es.ev) {
    if ((rc = report(cudaEventCreate(&ev), "event create"))) break;
    ++made;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!rc) rc = pipe_enqueue(f->spec, f->ws, parent, events, queries, answers, st, &es, &f->kernels);
  if (!rc) rc = report(cudaEventSynchronize(es.ev[BW_STAGE_COUNT]), "event sync");
  for (int i = 0; i < BW_STAGE_COUNT && !rc; ++i) {
    ms[i] = 0.f;
    rc = report(cudaEventElapsedTime(&ms[i], es.ev[i], es.ev[i + 1]), "event elapsed");
  }
  for (int i = 0; i < made; ++i) cudaEventDestroy(es.ev[i]);
  return rc;
}

extern "C" int bw_forest_status(BwForest* f, void* stream, int32_t* status) {
  if (!f || !f->ws || !status) return BW_EINVAL;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int32_t v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, pipe_status_word(f->spec, f->ws), 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return report(e, "status read");
  *status = v;
  return 0;
}

extern "C" int bw_forest_info(const BwForest* f, int32_t* blocks, int32_t* kernels, BwForestTuning* tuning) {
  if (!f) return BW_EINVAL;
  if (blocks) *blocks = f->spec.B;
  if (kernels) *kernels = f->kernels;
  if (tuning) *tuning = f->tuning;
  return 0;
}

extern "C" int bw_forest_destroy(BwForest* f) {
  if (!f) return 0;
  drop_graph(f);
  delete f;
  return 0;
}

extern "C" int bw_forest_plan_stats(const BwForestShape* sh, const BwForestTuning* tu, int32_t sms, int32_t* blocks,
                                    size_t* workspace_bytes, size_t* carry_bytes) {
  if (!sh || sh->n_trees < 1 || !sh->state_off || !sh->event_off || !sh->query_off || !sh->n_keys || sms < 1)
    return BW_EINVAL;
  if (tu && (tu->ctas_per_sm < 0 || tu->ctas_per_sm > 2 || tu->block_work < 0 || tu->slice_ranks < 0 ||
             tu->tile < 0 || tu->tile > kTileMaxId))
    return BW_EINVAL;
  PipeSpec s;
  const int rc = pipe_spec_forest(sh->n_trees, sh->state_off, sh->event_off, sh->query_off, sh->n_keys, to_tuning(tu),
                                  sms, s);
  if (rc) return rc;
  Layout L;
  pipe_layout(s, L);
  if (blocks) *blocks = s.B;
  if (workspace_bytes) *workspace_bytes = L.total;
  if (carry_bytes) *carry_bytes = (size_t)s.carry_words * 8;
  return 0;
}

extern "C" int bw_forest_autotune_workspace(const BwForestShape* shape, size_t* bytes) {
  if (!shape || !bytes) return BW_EINVAL;
  int sms = 0;
  int rc = sms_of_device(&sms);
  if (rc) return rc;
  size_t best = 0;
  for (const BwForestTuning& c : candidates(shape, sms)) {
    for (int32_t sr : {0, 8192}) {
      BwForestTuning x = c;
      x.slice_ranks = sr;
      PipeSpec s;
      if ((rc = plan_spec(shape, &x, s))) return rc;
      Layout L;
      pipe_layout(s, L);
      if (L.total > best) best = L.total;
    }
  }
  *bytes = best;
  return 0;
}

extern "C" int bw_forest_autotune(const BwForestShape* shape, const int32_t* parent, const BwEvent* events,
                                  const BwQuery* queries, int64_t* answers, void* workspace, size_t workspace_bytes,
                                  void* stream, int32_t reps, BwForestTuning* best, float* best_ms) {
  if (!shape || !best || reps < 1) return BW_EINVAL;
  int sms = 0;
  int rc = sms_of_device(&sms);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0, e1;
  if ((rc = report(cudaEventCreate(&e0), "event create"))) return rc;
  if ((rc = report(cudaEventCreate(&e1), "event create"))) {
    cudaEventDestroy(e0);
    return rc;
  }
  float best_t = -1.f;
  // one candidate: plan, bind, a warm-up launch whose device status must be clean
  // (a rejected candidate is skipped), then `reps` timed launches
  auto trial = [&](const BwForestTuning& x) -> int {
    BwForest* f = nullptr;
    int r = bw_forest_create(shape, &x, &f);
    if (r) return r;
    int32_t status = 0;
    if (!(r = bw_forest_bind(f, workspace, workspace_bytes, stream)) &&
        !(r = bw_forest_launch(f, parent, events, queries, answers, stream)) &&
        !(r = bw_forest_status(f, stream, &status)) && status == 0 &&
        !(r = report(cudaEventRecord(e0, st), "event record"))) {
      for (int32_t i = 0; i < reps && !r; ++i) r = bw_forest_launch(f, parent, events, queries, answers, stream);
      if (!r) r = report(cudaEventRecord(e1, st), "event record");
      if (!r) r = report(cudaEventSynchronize(e1), "event sync");
      float ms = 0.f;
      if (!r) r = report(cudaEventElapsedTime(&ms, e0, e1), "event elapsed");
      ms /= (float)reps;
      if (!r && (best_t < 0.f || ms < best_t)) {
        best_t = ms;
        *best = f->tuning;
      }
    }
    bw_forest_destroy(f);
    return r;
  };
  for (const BwForestTuning& c : candidates(shape, sms))
    if ((rc = trial(c))) break;
  if (!rc && best_t >= 0.f) {   // the other tile geometries at the best block work
    const BwForestTuning base = *best;
    for (int32_t tile = 1; tile <= kTileMaxId && !rc; ++tile) {
      if (tile == base.tile) continue;
      BwForestTuning x = base;
      x.tile = tile;
      if (tile >= 3) x.ctas_per_sm = 1;
      rc = trial(x);
    }
  }
  if (!rc && best_t >= 0.f) {
    const BwForestTuning base = *best;
    for (int32_t sr : {8192, 16384}) {
      BwForestTuning x = base;
      x.slice_ranks = sr;
      if ((rc = trial(x))) break;
    }
  }
  if (!rc && best_t < 0.f) {
    std::fprintf(stderr, "bw_forest_autotune: the device rejected every candidate (invalid input)\n");
    rc = BW_EINVAL;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!rc && best_ms) *best_ms = best_t;
  return rc;
}
