// bw_chain.cuh -- single-pass replay of a linear version chain (parent[v] = v-1).
//
// For a chain the Euler tour of the general pipeline is unnecessary: the events
// grouped by state are already in replay order, and the answer of a query at
// state s is the sum over the events with state <= s whose key lies in [lo, hi).
// The chain path reads each event once: persistent CTAs take contiguous event
// ranges (state blocks), stream them through shared memory with bulk async copies
// completed on mbarriers, keep the block's running key histogram in shared memory
// and answer the block's queries at tile granularity; a column scan of the
// blocks' histograms (the reference's serial carry, batch_engine_v7.hpp:936-945)
// and a per-block fix-up (its combine, :948-961) add the carry of the preceding
// blocks.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "bw_gpu.h"
#include "bw_pipeline.cuh"

namespace bw {

constexpr int kChainThreads = 512;                              // largest sweep CTA (and the fix-up CTA)
constexpr int kChainTile = 1024;                                // largest tile, events (16 KiB)
constexpr int kChainQBuf = 64;                                  // query records staged per tile
constexpr uint32_t kChainMaxKeys = 32768;                       // key domain held in shared memory
constexpr uint32_t kChainMaxKeys64 = 16384;                     // ... with the int64 window
constexpr int kChainSegRows = 16;                               // block rows per column-scan segment
constexpr int64_t kChainMinBlockEvents = 8192;

struct ChainSpec {
  int32_t S = 0;
  uint32_t C = 0;
  int64_t E = 0, Q = 0;
  int32_t B = 1;          // state blocks (= sweep CTAs)
  int32_t nch = 1;        // 32-key chunks of the window's chunk totals
  int32_t nseg = 1;       // column-scan segments
  int32_t ctas_per_sm = 1;
  bool w64 = false;       // int64 window (BW_REPLAY_WIDE)
  int32_t geometry = 2;   // sweep geometry: index, threads per CTA, events per thread
  int32_t threads = 512;
  int32_t ept = 2;
  size_t smem = 0;        // dynamic shared memory of the sweep
  size_t off_btab = 0, off_rows = 0, off_wide = 0, off_seg = 0, total = 0;   // workspace layout
};

// Whether a replay takes the chain path: the caller asserts a chain
// (BW_REPLAY_CHAIN_HINT), the key domain fits shared memory, the events are
// 16-byte aligned (bulk copies), and either the workload is event-heavy (at most
// one query per 8 events) or the caller forces the chain kernel.
bool chain_selected(const BwReplayArgs* a);
int chain_spec(const BwReplayArgs* a, int sms, ChainSpec& s);
int chain_enqueue(const ChainSpec& s, const BwReplayArgs* a, EventSet* timing, int* kernels);
inline const int32_t* chain_status_word(const void* workspace) { return static_cast<const int32_t*>(workspace); }

}  // namespace bw
