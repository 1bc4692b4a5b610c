// worker_main.cpp -- bw_worker: one timed measurement process with the reference
// GPU worker's contract (panel_batch_gpu.cpp:41-299), so a harness that runs the
// reference's workers as subprocesses (reproduce.py:87-105) can run this one:
//
//   bw_worker --fixture PATH --base-id ID --topology T --seed S --factor-period P
//             --q Q --repeat R --answers A --json J [--arm gb300|gpu_v7]
//             [--states N] [--blocks B]
//
// * the range scope comes from BWH_RANGE_SCOPE ("per_state", anything else shared),
//   the state count from --states, else BWH_STATES, else 2049 (the reference fixes it
//   at compile time), the v7 block count from --blocks, else BWH_V7_BLOCKS, else 128;
// * exit codes: 2 bad arguments, 3 unreadable fixture or unsupported case, 4 answer
//   or JSON write failure, 5 CUDA error (panel_batch_gpu.cpp:32-39, 61-80, 228-232);
// * phases load / setup / execute / extract / cleanup; the answers go raw to
//   --answers, the record to --json written as <json>.tmp and renamed
//   (panel_batch_gpu.cpp:274-293), with answers_sha256, answers_fn, phases_ns, a
//   "gpu" object, full_ns and peak_rss_kb, plus answers_per_s and hbm_gbps.
//
// Arms: "gb300" (default) compiles the declared workload into the event model on the
// host (bw_native_build) and replays it with bw_replay_launch (any topology);
// "gpu_v7" builds the reference's v7 chain plan (bw_v7_plan_build) and drives the
// gpu_v7.h drop-in entries: gpu_v7_launch, the carry on the device
// (bw_v7_carry_launch, where the reference worker does it on the host), and
// gpu_combine_launch.
#include <cuda_runtime.h>

#include <chrono>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "bw_gpu.h"
#include "bw_host.h"

namespace {

using clk = std::chrono::steady_clock;
int64_t ns_between(clk::time_point a, clk::time_point b) {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(b - a).count();
}

#define CUDA_OR_5(x)                                                                    \
  do {                                                                                  \
    const cudaError_t e_ = (x);                                                         \
    if (e_ != cudaSuccess) {                                                            \
      std::fprintf(stderr, "CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return 5;                                                                         \
    }                                                                                   \
  } while (0)
#define BW_OR_5(x, what)                                                                \
  do {                                                                                  \
    const int rc_ = (x);                                                                \
    if (rc_) {                                                                          \
      std::fprintf(stderr, "%s failed with code %d\n", what, rc_);                      \
      return rc_ == BW_EINVAL ? 3 : 5;                                                  \
    }                                                                                   \
  } while (0)

int64_t peak_rss_kb() {
  FILE* s = std::fopen("/proc/self/status", "r");
  int64_t kb = 0;
  if (!s) return 0;
  char line[256];
  while (std::fgets(line, sizeof(line), s)) {
    long v = 0;
    if (std::sscanf(line, "VmHWM: %ld kB", &v) == 1) { kb = v; break; }
  }
  std::fclose(s);
  return kb;
}

struct Timings {
  int64_t upload = 0, kernel = 0, carry = 0, combine = 0, download = 0;
  int32_t blocks = 0, threads = 0, shared = 0, kernels = 0;
  double algorithmic_bytes = 0;
};

template <typename T>
int upload(T** dst, const T* src, size_t n) {
  CUDA_OR_5(cudaMalloc(reinterpret_cast<void**>(dst), (n ? n : 1) * sizeof(T)));
  if (n) CUDA_OR_5(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}

// The event-model replay of a declared workload (any topology).
int run_event_arm(const BwNativeWorkload* w, int32_t blocks, std::vector<int64_t>& answers, Timings& tm) {
  const auto u0 = clk::now();
  int32_t* d_parent = nullptr;
  BwEvent* d_ev = nullptr;
  BwQuery* d_q = nullptr;
  int64_t* d_ans = nullptr;
  void* ws = nullptr;
  int rc = upload(&d_parent, w->parent, (size_t)w->n_states);
  if (!rc) rc = upload(&d_ev, w->events, (size_t)w->n_events);
  if (!rc) rc = upload(&d_q, w->queries, (size_t)w->n_queries);
  if (rc) return rc;
  CUDA_OR_5(cudaMalloc(&d_ans, (size_t)(w->n_queries ? w->n_queries : 1) * 8));
  bool chain = true;
  for (int32_t v = 1; v < w->n_states; ++v) chain = chain && w->parent[v] == v - 1;
  BwReplayArgs a{};
  a.n_states = w->n_states;
  a.parent = d_parent;
  a.n_keys = w->n_keys;
  a.n_events = w->n_events;
  a.events = d_ev;
  a.n_queries = w->n_queries;
  a.queries = d_q;
  a.answers = d_ans;
  a.blocks = blocks;
  a.flags = chain ? BW_REPLAY_CHAIN_HINT : 0;
  size_t need = 0;
  BW_OR_5(bw_replay_workspace_size(&a, &need), "bw_replay_workspace_size");
  CUDA_OR_5(cudaMalloc(&ws, need ? need : 256));
  a.workspace = ws;
  a.workspace_bytes = need ? need : 256;
  CUDA_OR_5(cudaDeviceSynchronize());
  const auto u1 = clk::now();
  cudaEvent_t e0, e1;
  CUDA_OR_5(cudaEventCreate(&e0));
  CUDA_OR_5(cudaEventCreate(&e1));
  CUDA_OR_5(cudaEventRecord(e0));
  BW_OR_5(bw_replay_launch(&a), "bw_replay_launch");
  CUDA_OR_5(cudaEventRecord(e1));
  CUDA_OR_5(cudaEventSynchronize(e1));
  float ms = 0.f;
  CUDA_OR_5(cudaEventElapsedTime(&ms, e0, e1));
  int32_t st = 0;
  BW_OR_5(bw_replay_status(&a, &st), "bw_replay_status");
  if (st) {
    std::fprintf(stderr, "the device rejected the workload (status %d)\n", st);
    return 3;
  }
  const auto d0 = clk::now();
  answers.assign((size_t)w->n_queries, 0);
  if (w->n_queries) CUDA_OR_5(cudaMemcpy(answers.data(), d_ans, (size_t)w->n_queries * 8, cudaMemcpyDeviceToHost));
  const auto d1 = clk::now();
  int32_t kernels = 0, nb = 0;
  bw_replay_last_info(&a, &kernels, &nb);
  tm.upload = ns_between(u0, u1);
  tm.kernel = (int64_t)((double)ms * 1e6);
  tm.download = ns_between(d0, d1);
  tm.blocks = nb;
  tm.kernels = kernels;
  tm.threads = 512;
  tm.algorithmic_bytes = 4.0 * w->n_states + 16.0 * (double)w->n_events + 20.0 * (double)w->n_queries;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CUDA_OR_5(cudaFree(ws));
  CUDA_OR_5(cudaFree(d_ans));
  CUDA_OR_5(cudaFree(d_q));
  CUDA_OR_5(cudaFree(d_ev));
  CUDA_OR_5(cudaFree(d_parent));
  return 0;
}

// The gpu_v7.h drop-in path on the reference's v7 chain plan.
int run_v7_arm(const BwV7Plan* p, std::vector<int64_t>& answers, Timings& tm) {
  const int32_t B = p->B, G = p->G, Cp = p->Cpfx, S = p->n_states, q = p->q;
  const int32_t nms = p->ms_off[p->n_active];
  const auto u0 = clk::now();
  GpuV7Node* d_nodes = nullptr;
  int32_t *d_v0 = nullptr, *d_v1 = nullptr, *d_g2row = nullptr, *d_ms_off = nullptr, *d_ms_dev = nullptr,
          *d_qlb = nullptr, *d_qhb = nullptr, *d_bidx = nullptr;
  int64_t *d_fac = nullptr, *d_ms_cls = nullptr, *d_ms_base = nullptr, *d_devbuf = nullptr, *d_need = nullptr,
          *d_vbase = nullptr, *d_lvals = nullptr, *d_dV = nullptr, *d_carry = nullptr, *d_ans = nullptr;
  int rc = upload(&d_nodes, p->nodes, (size_t)S);
  if (!rc) rc = upload(&d_v0, p->block_v0, (size_t)B);
  if (!rc) rc = upload(&d_v1, p->block_v1, (size_t)B);
  if (!rc) rc = upload(&d_fac, p->fac_start, (size_t)B * G);
  if (!rc) rc = upload(&d_g2row, p->g2row, (size_t)G);
  if (!rc) rc = upload(&d_ms_off, p->ms_off, (size_t)p->n_active + 1);
  if (!rc) rc = upload(&d_ms_cls, p->ms_cls, (size_t)nms);
  if (!rc) rc = upload(&d_ms_base, p->ms_base, (size_t)nms);
  if (!rc) rc = upload(&d_ms_dev, p->ms_dev, (size_t)nms);
  if (!rc) rc = upload(&d_devbuf, p->devbuf, (size_t)(p->n_devbuf ? p->n_devbuf : 1));
  if (!rc) rc = upload(&d_need, p->need_off, (size_t)B * G);
  if (!rc) rc = upload(&d_qlb, p->qlb, (size_t)S * q);
  if (!rc) rc = upload(&d_qhb, p->qhb, (size_t)S * q);
  if (!rc) rc = upload(&d_bidx, p->bidx, (size_t)S);
  if (!rc) rc = upload(&d_vbase, p->vbase, (size_t)Cp);
  if (rc) return rc;
  const size_t nans = (size_t)(S - 1) * q;
  CUDA_OR_5(cudaMalloc(&d_lvals, nans * 2 * 8));
  CUDA_OR_5(cudaMalloc(&d_dV, (size_t)B * Cp * 8));
  CUDA_OR_5(cudaMalloc(&d_carry, (size_t)B * Cp * 8));
  CUDA_OR_5(cudaMalloc(&d_ans, nans * 8));
  CUDA_OR_5(cudaDeviceSynchronize());
  const auto u1 = clk::now();
  GpuV7Args a{};
  a.B = B; a.G = G; a.Cpfx = Cp; a.ncls = p->ncls; a.q = q;
  a.nodes = d_nodes; a.block_v0 = d_v0; a.block_v1 = d_v1; a.fac_start = d_fac; a.g2row = d_g2row;
  a.ms_off = d_ms_off; a.ms_cls = d_ms_cls; a.ms_base = d_ms_base; a.ms_dev = d_ms_dev;
  a.devbuf = d_devbuf; a.need_off = d_need; a.qlb = d_qlb; a.qhb = d_qhb; a.lvals = d_lvals; a.dV = d_dV;
  a.threads = 512; a.shared_bytes = 0;
  GpuV7CombineArgs ca{};
  ca.nstates = S - 1; ca.q = q; ca.Cpfx = Cp; ca.qlb = d_qlb; ca.qhb = d_qhb; ca.carrypref = d_carry;
  ca.bidx = d_bidx; ca.lvals = d_lvals; ca.answers = d_ans;
  cudaEvent_t ev[4];
  for (auto& e : ev) CUDA_OR_5(cudaEventCreate(&e));
  CUDA_OR_5(cudaEventRecord(ev[0]));
  BW_OR_5(gpu_v7_launch(&a), "gpu_v7_launch");
  CUDA_OR_5(cudaEventRecord(ev[1]));
  BW_OR_5(bw_v7_carry_launch(B, Cp, d_vbase, d_dV, d_carry, nullptr), "bw_v7_carry_launch");
  CUDA_OR_5(cudaEventRecord(ev[2]));
  BW_OR_5(gpu_combine_launch(&ca), "gpu_combine_launch");
  CUDA_OR_5(cudaEventRecord(ev[3]));
  CUDA_OR_5(cudaEventSynchronize(ev[3]));
  float k_ms = 0, c_ms = 0, m_ms = 0;
  CUDA_OR_5(cudaEventElapsedTime(&k_ms, ev[0], ev[1]));
  CUDA_OR_5(cudaEventElapsedTime(&c_ms, ev[1], ev[2]));
  CUDA_OR_5(cudaEventElapsedTime(&m_ms, ev[2], ev[3]));
  const auto d0 = clk::now();
  answers.assign(nans, 0);
  if (nans) CUDA_OR_5(cudaMemcpy(answers.data(), d_ans, nans * 8, cudaMemcpyDeviceToHost));
  const auto d1 = clk::now();
  tm.upload = ns_between(u0, u1);
  tm.kernel = (int64_t)((double)k_ms * 1e6);
  tm.carry = (int64_t)((double)c_ms * 1e6);
  tm.combine = (int64_t)((double)m_ms * 1e6);
  tm.download = ns_between(d0, d1);
  tm.blocks = B;
  tm.threads = 512;
  tm.shared = (int32_t)(((size_t)Cp + (size_t)G) * 8);
  tm.kernels = 4;
  tm.algorithmic_bytes = 40.0 * S + 8.0 * nans * 3 + 16.0 * B * Cp;
  for (auto& e : ev) cudaEventDestroy(e);
  void* bufs[] = {d_nodes, d_v0, d_v1, d_fac, d_g2row, d_ms_off, d_ms_cls, d_ms_base, d_ms_dev, d_devbuf,
                  d_need, d_qlb, d_qhb, d_bidx, d_vbase, d_lvals, d_dV, d_carry, d_ans};
  for (void* b : bufs) CUDA_OR_5(cudaFree(b));
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  std::string arm = "gb300", fixture_path, base_id, answers_path, json_path;
  int32_t topology = 0, seed = 7, factor_period = 4, q = 2, repeat = 0, states = 0, blocks = 0;
  for (int i = 1; i < argc; ++i) {
    auto next = [&](const char* k) -> std::string {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "missing value for %s\n", k);
        std::exit(2);
      }
      return argv[++i];
    };
    auto num = [&](const char* k) -> int32_t {
      const std::string s = next(k);
      char* end = nullptr;
      const long v = std::strtol(s.c_str(), &end, 10);
      if (s.empty() || *end) {
        std::fprintf(stderr, "bad integer for %s: %s\n", k, s.c_str());
        std::exit(2);
      }
      return (int32_t)v;
    };
    const char* k = argv[i];
    if (!std::strcmp(k, "--arm")) arm = next(k);
    else if (!std::strcmp(k, "--fixture")) fixture_path = next(k);
    else if (!std::strcmp(k, "--base-id")) base_id = next(k);
    else if (!std::strcmp(k, "--topology")) topology = num(k);
    else if (!std::strcmp(k, "--seed")) seed = num(k);
    else if (!std::strcmp(k, "--factor-period")) factor_period = num(k);
    else if (!std::strcmp(k, "--q")) q = num(k);
    else if (!std::strcmp(k, "--repeat")) repeat = num(k);
    else if (!std::strcmp(k, "--answers")) answers_path = next(k);
    else if (!std::strcmp(k, "--json")) json_path = next(k);
    else if (!std::strcmp(k, "--states")) states = num(k);
    else if (!std::strcmp(k, "--blocks")) blocks = num(k);
    else {
      std::fprintf(stderr, "unknown argument %s\n", k);
      return 2;
    }
  }
  if (fixture_path.empty() || answers_path.empty() || json_path.empty()) {
    std::fprintf(stderr, "usage: bw_worker --fixture PATH --base-id ID --topology T --seed S "
                         "--factor-period P --q Q --repeat R --answers A --json J [--arm gb300|gpu_v7] "
                         "[--states N] [--blocks B]\n");
    return 2;
  }
  if (arm != "gb300" && arm != "gpu_v7") {
    std::fprintf(stderr, "unknown arm %s (gb300 or gpu_v7)\n", arm.c_str());
    return 2;
  }
  if (!states) {
    const char* e = std::getenv("BWH_STATES");
    states = e ? std::atoi(e) : 2049;
  }
  if (!blocks) {
    const char* e = std::getenv("BWH_V7_BLOCKS");
    blocks = e ? std::atoi(e) : (arm == "gpu_v7" ? 128 : 0);
  }
  if (q < 1 || q > 64 || states < 3 || topology < 0 || topology > 2 || blocks < 0) {
    std::fprintf(stderr, "unsupported q, state count, topology or block count\n");
    return 2;
  }
  const char* scope_env = std::getenv("BWH_RANGE_SCOPE");
  const bool per_state = scope_env && std::strcmp(scope_env, "per_state") == 0;

  const auto t0 = clk::now();
  BwFixture* fx = nullptr;
  if (bw_fixture_open(fixture_path.c_str(), &fx)) {
    std::fprintf(stderr, "cannot load fixture\n");
    return 3;
  }
  const auto t1 = clk::now();

  // ---- setup: declared workload compiled on the host
  BwNativeSpec spec{states, topology, seed, factor_period, q, per_state ? 1 : 0, -1};
  BwNativeWorkload* w = nullptr;
  BwV7Plan* plan = nullptr;
  if (arm == "gb300") {
    if (bw_native_build(fx, &spec, &w)) {
      std::fprintf(stderr, "workload build failed (unsupported case)\n");
      return 3;
    }
  } else {
    if (topology != 0 || bw_v7_plan_build(fx, &spec, blocks, &plan)) {
      std::fprintf(stderr, "v7 plan build failed (unsupported case: the v7 block path takes chains)\n");
      return 3;
    }
  }
  const auto t2 = clk::now();

  // ---- execute: upload, replay, download
  CUDA_OR_5(cudaSetDevice(0));
  CUDA_OR_5(cudaFree(nullptr));   // context creation is not a copy cost
  std::vector<int64_t> answers;
  Timings tm;
  const auto te0 = clk::now();
  const int rc = arm == "gb300" ? run_event_arm(w, blocks, answers, tm) : run_v7_arm(plan, answers, tm);
  if (rc) return rc;
  const auto t3 = clk::now();

  // ---- extract
  FILE* out = std::fopen(answers_path.c_str(), "wb");
  if (!out) {
    std::fprintf(stderr, "cannot write answers\n");
    return 4;
  }
  const bool wok = std::fwrite(answers.data(), 8, answers.size(), out) == answers.size();
  std::fclose(out);
  if (!wok) {
    std::fprintf(stderr, "short answer write\n");
    return 4;
  }
  const uint64_t fn = bw_fnv1a(answers.data(), answers.size() * 8);
  char sha[65];
  bw_sha256_hex(answers.data(), answers.size() * 8, sha);
  const auto t4 = clk::now();

  // ---- cleanup
  if (w) bw_native_free(w);
  if (plan) bw_v7_plan_free(plan);
  bw_fixture_close(fx);
  const auto t5 = clk::now();

  const int64_t load_ns = ns_between(t0, t1), setup_ns = ns_between(t1, t2), execute_ns = ns_between(te0, t3),
                extract_ns = ns_between(t3, t4), cleanup_ns = ns_between(t4, t5);
  const int64_t full_ns = load_ns + setup_ns + execute_ns + extract_ns + cleanup_ns;
  const int64_t kernel_total = tm.kernel + tm.carry + tm.combine;
  std::string devname = "n/a";
  {
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, 0) == cudaSuccess) devname.assign(prop.name, strnlen(prop.name, sizeof(prop.name)));
  }
  const std::string tmp = json_path + ".tmp";
  FILE* jf = std::fopen(tmp.c_str(), "w");
  if (!jf) {
    std::fprintf(stderr, "cannot write json\n");
    return 4;
  }
  std::fprintf(jf, "{\n  \"arm\": \"%s\",\n  \"base_id\": \"%s\",\n", arm.c_str(), base_id.c_str());
  std::fprintf(jf, "  \"fixture\": \"%s\",\n  \"topology\": %d,\n  \"seed\": %d,\n  \"factor_period\": %d,\n",
               fixture_path.c_str(), topology, seed, factor_period);
  std::fprintf(jf, "  \"q\": %d,\n  \"repeat\": %d,\n  \"n_states\": %d,\n  \"n_answers\": %zu,\n", q, repeat, states,
               answers.size());
  std::fprintf(jf, "  \"range_scope\": \"%s\",\n", per_state ? "per_state" : "shared");
  std::fprintf(jf, "  \"answers_fn\": \"%016" PRIx64 "\",\n  \"answers_sha256\": \"%s\",\n", fn, sha);
  std::fprintf(jf,
               "  \"phases_ns\": {\"load\": %" PRId64 ", \"setup\": %" PRId64 ", \"execute\": %" PRId64
               ", \"extract\": %" PRId64 ", \"cleanup\": %" PRId64 "},\n",
               load_ns, setup_ns, execute_ns, extract_ns, cleanup_ns);
  std::fprintf(jf,
               "  \"gpu\": {\"device\": \"%s\", \"blocks\": %d, \"threads\": %d, \"shared_bytes\": %d, \"kernels\": %d, "
               "\"upload_ns\": %" PRId64 ", \"kernel_ns\": %" PRId64 ", \"carry_ns\": %" PRId64
               ", \"combine_ns\": %" PRId64 ", \"download_ns\": %" PRId64 "},\n",
               devname.c_str(), tm.blocks, tm.threads, tm.shared, tm.kernels, tm.upload, tm.kernel, tm.carry, tm.combine,
               tm.download);
  std::fprintf(jf, "  \"answers_per_s\": %.6g,\n  \"hbm_gbps\": %.6g,\n",
               kernel_total ? (double)answers.size() / ((double)kernel_total * 1e-9) : 0.0,
               kernel_total ? tm.algorithmic_bytes / (double)kernel_total : 0.0);
  std::fprintf(jf, "  \"full_ns\": %" PRId64 ",\n  \"peak_rss_kb\": %" PRId64 "\n}\n", full_ns, peak_rss_kb());
  std::fclose(jf);
  if (std::rename(tmp.c_str(), json_path.c_str()) != 0) return 4;
  std::printf("arm=%s base=%s t%d s%d f%d q%d r%d blocks=%d kernel_ms=%.3f full_ns=%" PRId64 "\n", arm.c_str(),
              base_id.c_str(), topology, seed, factor_period, q, repeat, tm.blocks, (double)kernel_total / 1e6,
              full_ns);
  return 0;
}
