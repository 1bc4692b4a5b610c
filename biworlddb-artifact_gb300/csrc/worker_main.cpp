// worker_main.cpp -- bw_worker: one timed measurement process with the reference
// GPU worker's contract (panel_batch_gpu.cpp:41-299), so a harness that runs the
// reference's workers as subprocesses (reproduce.py:87-105) can run this one:
//
//   bw_worker --fixture PATH --base-id ID --topology T --seed S --factor-period P
//             --q Q --repeat R --answers A --json J [--arm gb300|gpu_v7]
//             [--states N] [--blocks B] [--events STREAM]
//
// * --events takes the workload from a BWLEV001 event stream over the fixture (the
//   reference's emit_events.cpp output) instead of the declared generator: the
//   stream compiles into a linear-chain event workload (bw_stream_build), replays on
//   the gb300 arm, and its answers go back to (state, k) order on the device
//   (bw_scatter_answers); --topology/--seed/--factor-period/--q are then only echoed;
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

#include <algorithm>
#include <chrono>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <string>
#include <thread>
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

// Answers an arm leaves on the device for the extract phase, and every device
// buffer of the run (freed at cleanup).
struct DeviceAnswers {
  int64_t* d = nullptr;
  size_t n = 0;
  std::vector<void*> owned;
  ~DeviceAnswers() {
    for (void* b : owned) cudaFree(b);
  }
};

template <typename T>
int upload(T** dst, const T* src, size_t n) {
  CUDA_OR_5(cudaMalloc(reinterpret_cast<void**>(dst), (n ? n : 1) * sizeof(T)));
  if (n) CUDA_OR_5(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}

// The event-model replay of a declared workload (any topology).
// wide: the chain path's int64 histogram (deltas mostly outside the int32 window);
// d_events: events already on the device (the device-side chain setup), else they
// are uploaded from w->events.
int run_event_arm(const BwNativeWorkload* w, int32_t blocks, bool wide, BwEvent* d_events, DeviceAnswers& out,
                  Timings& tm) {
  const auto u0 = clk::now();
  int32_t* d_parent = nullptr;
  BwEvent* d_ev = d_events;
  BwQuery* d_q = nullptr;
  int64_t* d_ans = nullptr;
  void* ws = nullptr;
  int rc = upload(&d_parent, w->parent, (size_t)w->n_states);
  out.owned.push_back(d_parent);
  if (!rc && !d_ev) {
    rc = upload(&d_ev, w->events, (size_t)w->n_events);
    out.owned.push_back(d_ev);
  }
  if (!rc) rc = upload(&d_q, w->queries, (size_t)w->n_queries);
  out.owned.push_back(d_q);
  if (rc) return rc;
  CUDA_OR_5(cudaMalloc(&d_ans, (size_t)(w->n_queries ? w->n_queries : 1) * 8));
  out.owned.push_back(d_ans);
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
  a.flags = chain ? (BW_REPLAY_CHAIN_HINT | (wide ? BW_REPLAY_WIDE : 0)) : 0;
  size_t need = 0;
  BW_OR_5(bw_replay_workspace_size(&a, &need), "bw_replay_workspace_size");
  CUDA_OR_5(cudaMalloc(&ws, need ? need : 256));
  out.owned.push_back(ws);
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
  out.d = d_ans;
  out.n = (size_t)w->n_queries;
  int32_t kernels = 0, nb = 0;
  bw_replay_last_info(&a, &kernels, &nb);
  tm.upload = ns_between(u0, u1);
  tm.kernel = (int64_t)((double)ms * 1e6);
  tm.blocks = nb;
  tm.kernels = kernels;
  tm.threads = 512;
  tm.algorithmic_bytes = 4.0 * w->n_states + 16.0 * (double)w->n_events + 20.0 * (double)w->n_queries;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return 0;
}

// More than one delta in 64 outside (-2^19, 2^19): the chain path's int32 windows
// would take the wide-tile route most of the time, so its int64 histogram is used.
bool wide_deltas(const BwEvent* ev, int64_t n) {
  int64_t big = 0;
  for (int64_t i = 0; i < n; ++i) big += (ev[i].delta >= (1 << 19) || ev[i].delta <= -(1 << 19)) ? 1 : 0;
  return big * 64 > n;
}

// The gpu_v7.h drop-in path on the reference's v7 chain plan.
int run_v7_arm(const BwV7Plan* p, DeviceAnswers& out, Timings& tm) {
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
  for (void* b : {(void*)d_nodes, (void*)d_v0, (void*)d_v1, (void*)d_fac, (void*)d_g2row, (void*)d_ms_off,
                  (void*)d_ms_cls, (void*)d_ms_base, (void*)d_ms_dev, (void*)d_devbuf, (void*)d_need, (void*)d_qlb,
                  (void*)d_qhb, (void*)d_bidx, (void*)d_vbase})
    if (b) out.owned.push_back(b);
  if (rc) return rc;
  const size_t nans = (size_t)(S - 1) * q;
  CUDA_OR_5(cudaMalloc(&d_lvals, nans * 2 * 8));
  out.owned.push_back(d_lvals);
  CUDA_OR_5(cudaMalloc(&d_dV, (size_t)B * Cp * 8));
  out.owned.push_back(d_dV);
  CUDA_OR_5(cudaMalloc(&d_carry, (size_t)B * Cp * 8));
  out.owned.push_back(d_carry);
  CUDA_OR_5(cudaMalloc(&d_ans, nans * 8));
  out.owned.push_back(d_ans);
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
  out.d = d_ans;
  out.n = nans;
  tm.upload = ns_between(u0, u1);
  tm.kernel = (int64_t)((double)k_ms * 1e6);
  tm.carry = (int64_t)((double)c_ms * 1e6);
  tm.combine = (int64_t)((double)m_ms * 1e6);
  tm.blocks = B;
  tm.threads = 512;
  tm.shared = (int32_t)(((size_t)Cp + (size_t)G) * 8);
  tm.kernels = 4;
  tm.algorithmic_bytes = 40.0 * S + 8.0 * nans * 3 + 16.0 * B * Cp;
  for (auto& e : ev) cudaEventDestroy(e);
  return 0;
}

// Extract: the answers come down in 2 MiB chunks through a ring of pinned buffers
// on a copy stream, and each landed chunk is digested while the next ones copy:
// SHA-256 on this thread, FNV-1a and the raw answer-file write on a helper thread.
// The digests equal the one-shot ones over the whole vector.  Returns 4 when the
// answer file cannot be written, 5 on a CUDA error.
struct ExtractResult {
  char sha[65] = {0};
  uint64_t fnv = 0;
  int64_t download_ns = 0;   // summed device time of the chunk copies
};

int extract_answers(const DeviceAnswers& da, const std::string& path, ExtractResult& r) {
  FILE* out = std::fopen(path.c_str(), "wb");
  if (!out) return 4;
  constexpr size_t kChunk = (size_t)1 << 18;   // answers per chunk
  constexpr int kRing = 4;
  const size_t nchunks = (da.n + kChunk - 1) / kChunk;
  struct Ring {
    int64_t* host[kRing] = {};
    cudaEvent_t beg[kRing] = {}, end[kRing] = {};
    cudaStream_t s = nullptr;
    ~Ring() {
      for (int k = 0; k < kRing; ++k) {
        if (host[k]) cudaFreeHost(host[k]);
        if (beg[k]) cudaEventDestroy(beg[k]);
        if (end[k]) cudaEventDestroy(end[k]);
      }
      if (s) cudaStreamDestroy(s);
    }
  } ring;
  auto fail = [&](cudaError_t e) {
    std::fprintf(stderr, "CUDA error %s in the answer extract\n", cudaGetErrorString(e));
    std::fclose(out);
    return 5;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&ring.s, cudaStreamNonBlocking);
  for (int k = 0; e == cudaSuccess && k < kRing && (size_t)k < nchunks; ++k) {
    e = cudaHostAlloc(reinterpret_cast<void**>(&ring.host[k]), kChunk * 8, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaEventCreate(&ring.beg[k]);
    if (e == cudaSuccess) e = cudaEventCreate(&ring.end[k]);
  }
  if (e != cudaSuccess) return fail(e);
  auto chunk_len = [&](size_t c) { return std::min(kChunk, da.n - c * kChunk); };
  auto issue = [&](size_t c) {
    const int k = (int)(c % kRing);
    cudaError_t x = cudaEventRecord(ring.beg[k], ring.s);
    if (x == cudaSuccess)
      x = cudaMemcpyAsync(ring.host[k], da.d + c * kChunk, chunk_len(c) * 8, cudaMemcpyDeviceToHost, ring.s);
    if (x == cudaSuccess) x = cudaEventRecord(ring.end[k], ring.s);
    return x;
  };
  for (size_t c = 0; e == cudaSuccess && c < nchunks && c < (size_t)kRing; ++c) e = issue(c);
  if (e != cudaSuccess) return fail(e);
  BwSha256 sh;
  bw_sha256_init(&sh);
  uint64_t fn = BW_FNV1A_BASIS;
  bool wok = true;
  double copy_ms = 0;
  for (size_t c = 0; c < nchunks; ++c) {
    const int k = (int)(c % kRing);
    if ((e = cudaEventSynchronize(ring.end[k])) != cudaSuccess) return fail(e);
    float ms = 0.f;
    if ((e = cudaEventElapsedTime(&ms, ring.beg[k], ring.end[k])) != cudaSuccess) return fail(e);
    copy_ms += ms;
    const int64_t* buf = ring.host[k];
    const size_t n = chunk_len(c);
    std::thread side([&fn, &wok, buf, n, out] {
      fn = bw_fnv1a_update(fn, buf, n * 8);
      wok = std::fwrite(buf, 8, n, out) == n && wok;
    });
    bw_sha256_update(&sh, buf, n * 8);
    side.join();
    if (c + kRing < nchunks && (e = issue(c + kRing)) != cudaSuccess) return fail(e);
  }
  wok = std::fclose(out) == 0 && wok;
  bw_sha256_final(&sh, r.sha);
  r.fnv = fn;
  r.download_ns = (int64_t)(copy_ms * 1e6);
  if (!wok) {
    std::fprintf(stderr, "short answer write\n");
    return 4;
  }
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  std::string arm = "gb300", fixture_path, base_id, answers_path, json_path, events_path;
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
    else if (!std::strcmp(k, "--events")) events_path = next(k);
    else {
      std::fprintf(stderr, "unknown argument %s\n", k);
      return 2;
    }
  }
  if (fixture_path.empty() || answers_path.empty() || json_path.empty()) {
    std::fprintf(stderr, "usage: bw_worker --fixture PATH --base-id ID --topology T --seed S "
                         "--factor-period P --q Q --repeat R --answers A --json J [--arm gb300|gpu_v7] "
                         "[--states N] [--blocks B] [--events STREAM]\n");
    return 2;
  }
  if (arm != "gb300" && arm != "gpu_v7") {
    std::fprintf(stderr, "unknown arm %s (gb300 or gpu_v7)\n", arm.c_str());
    return 2;
  }
  if (!events_path.empty() && arm != "gb300") {
    std::fprintf(stderr, "--events replays on the gb300 arm only\n");
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
  BwStreamWorkload* sw = nullptr;
  BwNativeCompact* cp = nullptr;   // device-side chain setup
  BwNativeWorkload cw{};           // its chain view (events on the device)
  BwEvent* d_events = nullptr;
  void* d_xws = nullptr;
  bool wide = false;
  const char* dev_setup = std::getenv("BWH_DEVICE_SETUP");
  const bool device_setup = arm == "gb300" && events_path.empty() && topology == 0 &&
                            !(dev_setup && std::strcmp(dev_setup, "0") == 0);
  if (device_setup) {   // the CUDA context is process start-up, not a workload phase
    CUDA_OR_5(cudaSetDevice(0));
    CUDA_OR_5(cudaFree(nullptr));
  }
  const auto t1s = clk::now();
  if (!events_path.empty()) {
    std::ifstream in(events_path, std::ios::binary);
    const std::vector<char> img((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    if (!in.good() && !in.eof()) {
      std::fprintf(stderr, "cannot read event stream\n");
      return 3;
    }
    if (bw_stream_build(fx, img.data(), img.size(), &sw)) {
      std::fprintf(stderr, "malformed event stream\n");
      return 3;
    }
    w = &sw->chain;
    q = sw->q;
    if (q > 0) states = (int32_t)(sw->n_answers / q) + 1;
  } else if (device_setup) {
    // chain setup on the device: compact form on the host, factor expansion on the GPU
    if (bw_native_build_compact(fx, &spec, &cp)) {
      std::fprintf(stderr, "workload build failed (unsupported case)\n");
      return 3;
    }
    size_t xbytes = 0;
    BW_OR_5(bw_native_expand_workspace(cp, &xbytes), "bw_native_expand_workspace");
    CUDA_OR_5(cudaMalloc(&d_xws, xbytes ? xbytes : 256));
    CUDA_OR_5(cudaMalloc(&d_events, (size_t)(cp->n_events ? cp->n_events : 1) * sizeof(BwEvent)));
    BW_OR_5(bw_native_expand(cp, d_events, d_xws, xbytes ? xbytes : 256, nullptr), "bw_native_expand");
    CUDA_OR_5(cudaDeviceSynchronize());
    CUDA_OR_5(cudaFree(d_xws));
    d_xws = nullptr;
    cw.n_states = cp->n_states;
    cw.n_keys = cp->n_keys;
    cw.n_events = cp->n_events;
    cw.n_queries = cp->n_queries;
    cw.parent = cp->parent;
    cw.queries = cp->queries;
    w = &cw;
    wide = wide_deltas(cp->fixed, cp->n_fixed);
  } else if (arm == "gb300") {
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
  DeviceAnswers da;
  Timings tm;
  const auto te0 = clk::now();
  if (w && !cp) wide = wide_deltas(w->events, w->n_events);
  if (d_events) da.owned.push_back(d_events);
  const int rc = arm == "gb300" ? run_event_arm(w, blocks, wide, d_events, da, tm) : run_v7_arm(plan, da, tm);
  if (rc) return rc;
  if (sw) {   // chain answers (stream order) -> the (state, k) answer vector
    int64_t *d_slot = nullptr, *d_out = nullptr;
    const size_t nq = (size_t)sw->chain.n_queries, na = (size_t)sw->n_answers;
    if (upload(&d_slot, sw->slot, nq)) return 5;
    da.owned.push_back(d_slot);
    CUDA_OR_5(cudaMalloc(&d_out, (na ? na : 1) * 8));
    da.owned.push_back(d_out);
    CUDA_OR_5(cudaMemset(d_out, 0, (na ? na : 1) * 8));
    BW_OR_5(bw_scatter_answers(da.d, d_slot, (int64_t)nq, d_out, (int64_t)na, nullptr), "bw_scatter_answers");
    CUDA_OR_5(cudaDeviceSynchronize());
    da.d = d_out;
    da.n = na;
  }
  const auto t3 = clk::now();

  // ---- extract: pipelined download, digests and answer file
  ExtractResult xr;
  const int xrc = extract_answers(da, answers_path, xr);
  if (xrc) {
    if (xrc == 4) std::fprintf(stderr, "cannot write answers\n");
    return xrc;
  }
  tm.download = xr.download_ns;
  const uint64_t fn = xr.fnv;
  const char* sha = xr.sha;
  const size_t n_answers = da.n;
  const auto t4 = clk::now();

  // ---- cleanup
  for (void* b : da.owned) cudaFree(b);
  da.owned.clear();
  if (sw) bw_stream_free(sw);
  else if (cp) bw_native_compact_free(cp);
  else if (w) bw_native_free(w);
  if (plan) bw_v7_plan_free(plan);
  bw_fixture_close(fx);
  const auto t5 = clk::now();

  const int64_t load_ns = ns_between(t0, t1), setup_ns = ns_between(t1s, t2), execute_ns = ns_between(te0, t3),
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
               n_answers);
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
               kernel_total ? (double)n_answers / ((double)kernel_total * 1e-9) : 0.0,
               kernel_total ? tm.algorithmic_bytes / (double)kernel_total : 0.0);
  std::fprintf(jf, "  \"full_ns\": %" PRId64 ",\n  \"peak_rss_kb\": %" PRId64 "\n}\n", full_ns, peak_rss_kb());
  std::fclose(jf);
  if (std::rename(tmp.c_str(), json_path.c_str()) != 0) return 4;
  std::printf("arm=%s base=%s t%d s%d f%d q%d r%d blocks=%d kernel_ms=%.3f full_ns=%" PRId64 "\n", arm.c_str(),
              base_id.c_str(), topology, seed, factor_period, q, repeat, tm.blocks, (double)kernel_total / 1e6,
              full_ns);
  return 0;
}
