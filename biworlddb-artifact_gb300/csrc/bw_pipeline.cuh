// bw_pipeline.cuh -- the version-forest replay pipeline shared by the plain entry
// (bw_replay_*, one tree) and the batched entry (bw_forest_*, many trees).
//
// A forest is a concatenation of independent version trees.  Tree t owns global
// states [s0, s0 + ns), events [e0, e0 + ne), queries [q0, q0 + nq) and a key
// domain [0, C); its parent array, event states and query states are local to the
// tree (parent[local 0] = -1, parent[l] < l).  The pipeline lays every tree's
// Euler tour out at steps [2 s0, 2 s0 + 2 ns), cuts each tree into nb equal-work
// state blocks that never span trees, and replays all blocks of all trees with
// persistent CTAs that take blocks from a shared queue (largest first).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

#include "bw_gpu.h"

namespace bw {

// ------------------------------------------------------------------ constants
constexpr int kPrepThreads = 512;             // CTA width of the prepare kernel (two per SM)
constexpr int kWinBits = 18;                  // rank window: 2^18 keys per smem bitmap
constexpr int kWinWords = 1 << (kWinBits - 6);
constexpr int kMaxSlices = 256;               // key slices per block
constexpr int kSmemLimit = 232448;            // 227 KiB dynamic smem per CTA on sm_100/103
constexpr int kSmemPerSM = 233472;            // 228 KiB shared memory per SM
constexpr int kCarryGroup = 16;               // rows per group of the carry scan
constexpr int kCarryChunk = 256;              // columns per carry unit
constexpr int64_t kStepCost = 4;              // fixed cost of an Euler step, in event units
constexpr int64_t kQueryStepCost = 64;        // extra cost of a step with queries (two CTA barriers)
constexpr int64_t kQueryCost = 2;             // a query is two prefix probes

// Estimated sweep work of a tree (or a whole forest) from its sizes: every event is
// applied on enter and on exit, every state is entered and left, and at most
// min(S, Q) steps carry queries.
__host__ __device__ inline int64_t est_work(int64_t S, int64_t E, int64_t Q) {
  return 2 * E + kQueryCost * Q + 2 * kStepCost * S + kQueryStepCost * (S < Q ? S : Q);
}

// Sweep geometry (see bw_pipeline.cu).
constexpr int kChunk = 256;
constexpr int kChunkBits = 8;
constexpr int kChunkLevels = 8;
constexpr int kChunkStride = 257;
constexpr int kMaxChunks = 128;
constexpr int kRebuildPer = 5;
constexpr int64_t kOfflinePairs = 32768;      // tile (queries x events) below which probes are batched
constexpr int kOfflineQ = 128;                // and at most this many queries (their sums live in smem)

// Sweep tile geometry: THREADS per CTA, EV events and QP queries staged per thread
// per tile, at most STEPS steps per tile, a ring of RING step descriptors refilled
// RING - 3 * STEPS (rounded down to whole warps) at a time: a refill during a tile's
// probes keeps the slots of that tile and the next two.
// COOP: the tile is staged cooperatively and made visible by a barrier (suits many
// small steps); otherwise every thread stages the items it will apply and probe
// itself and waits for its own copies only (suits few large, query-heavy steps).
// FLAT: the rank structure keeps plain values per rank with chunk totals (two
// atomics per update, probes summed by a warp: suits few queries per many events);
// otherwise a Fenwick tree inside every chunk (<= 9 atomics per update, probes by one
// thread: suits many queries).
// SPEC: warp-specialised: the last warp cuts and stages tiles (ring, tile cut,
// cp.async of events and queries) two tiles ahead into three buffers while the
// other warps replay, synchronised by one CTA barrier per tile and a consumer-only
// named barrier (flat chunks only).
template <int EV, int QP, int STEPS, int RING, int THREADS, bool COOP, bool FLAT, bool SPEC = false>
struct TileCfg {
  static constexpr bool kCoop = COOP, kFlat = FLAT, kSpec = SPEC;
  static constexpr int kBufs = SPEC ? 3 : 2;
  static constexpr int kEvPer = EV, kQPer = QP, kTileSteps = STEPS, kRing = RING,
                       kRingFill = (RING - 3 * STEPS) / 32 * 32;
  static constexpr int kThreads = THREADS, kWarps = THREADS / 32, kMinBlocks = THREADS >= 512 ? 1 : 2;
  static constexpr int kTileEv = EV * THREADS, kTileQ = QP * THREADS;
  static_assert((RING & (RING - 1)) == 0 && kRingFill >= STEPS && STEPS <= 128 && STEPS % 32 == 0,
                "tile ring too small");
  static_assert(!SPEC || (FLAT && !COOP && THREADS >= 128), "specialised tiles are flat, own staging");
};
using TileNarrow = TileCfg<2, 2, 32, 128, 256, false, false>;      // query-heavy steps: small staging, Fenwick
using TileWide = TileCfg<4, 1, 64, 256, 256, true, true>;          // event-heavy steps: deep staging, flat
using TileNarrow512 = TileCfg<2, 1, 128, 512, 512, false, true>;   // 16 warps (one CTA per SM), own staging, flat
using TileWide512 = TileCfg<2, 1, 64, 256, 512, true, true>;
using TileSpec512 = TileCfg<1, 1, 64, 512, 512, false, true, true>;   // 15 replay warps + 1 staging warp
// kTileEulerId: the Euler-tile sweep of bw_esweep.cu (bulk-copied signed event tiles,
// flat window, a producer warp; one CTA per SM) instead of k_sweep.
enum { kTileAuto = 0, kTileNarrowId = 1, kTileWideId = 2, kTileNarrow512Id = 3, kTileWide512Id = 4, kTileSpec512Id = 5,
       kTileEulerId = 6 };
constexpr int kTileMaxId = 6;
// Window capacity of the Euler-tile sweep: int32 entries, or int64 ones in the same
// bytes (the prepare pass cuts its rank slices with the k_sweep window's capacities,
// 27,904 and 13,824 entries, which both fit).
constexpr uint32_t kEsCap32 = 27904;
constexpr uint32_t kEsCap64 = 13952;

// ------------------------------------------------------------------ records
struct StepDesc {        // one Euler step, 16 bytes
  uint32_t e0;           // first event of the node (global index)
  uint32_t q0;           // first query of the node (enter steps)
  int32_t ne;            // event count
  int32_t nq;            // query count on enter, -1 on exit
};

struct Slice {           // contiguous key range with <= cap distinct block keys
  int32_t word_lo, word_hi;  // bitmap words [word_lo, word_hi)
  uint32_t rank_lo;          // block-local rank of the first key of the slice
  uint32_t n;                // distinct keys in the slice
};

struct BlockTab {        // one state block, written on the device per launch
  int32_t tree, idx;     // tree and block index inside the tree
  int32_t t0, t1;        // steps [t0, t1)
  uint32_t C;            // key domain of the tree
  int32_t nwords;        // bitmap words of the domain
  int64_t bits_off;      // first bitmap word (rank table: bits_off + block index)
  int64_t carry_in;      // carry row read by the sweep (-1: the block starts its tree)
  int64_t carry_out;     // net-delta row written by prepare (-1: last block of its tree)
};

struct CarryUnit {       // 256 columns of one row group of one tree's carry rows
  int32_t tree, group, chunk, pad;
};

// Device-side tree tables (in the workspace).
struct TreeTabs {
  int32_t* soff;         // T+1 first global state
  int64_t* eoff;         // T+1 first event
  int64_t* qoff;         // T+1 first query
  uint32_t* C;           // T   key domain
  int32_t* boff;         // T+1 first block
  int64_t* bits;         // T   first bitmap word of the tree's blocks
  int64_t* carry;        // T   first carry word of the tree's rows
  int64_t* gsum;         // T   first group-sum word
  int32_t* last_q;       // T   last step answering a query + 1 (0: none)
};

// Shared-memory layout of the sweep for a rank-table window of `ww` words.
struct SweepLayout {
  int32_t ww;
  int32_t nch32, nch64;
  uint32_t cap32, cap64;
  size_t off_rl, off_fine, off_T, off_P, off_ring, off_pdesc, off_epre, off_qpre, off_ev, off_emeta, off_q, off_qmeta,
      off_corr, off_tiles, bytes;
};
template <typename Cfg>
__host__ __device__ inline SweepLayout sweep_layout(int32_t nwords, size_t budget) {
  SweepLayout L;
  L.ww = nwords < kWinWords ? nwords : kWinWords;
  auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
  const size_t staging = sizeof(StepDesc) * (Cfg::kRing + Cfg::kRingFill) + 2 * 8 * (size_t)Cfg::kRing +
                         Cfg::kBufs * (size_t)Cfg::kTileEv * 16 + al(Cfg::kBufs * (size_t)Cfg::kTileEv) +
                         al(Cfg::kBufs * (size_t)Cfg::kTileQ * 12) + al(Cfg::kBufs * (size_t)Cfg::kTileQ) +
                         (size_t)kOfflineQ * 8 + 3 * 32;
  // per-warp copies of the chunk-total prefix: Fenwick chunks only (flat chunks
  // probe the chunk totals directly)
  const size_t pcopies = Cfg::kFlat ? 0 : (size_t)Cfg::kWarps * (kMaxChunks + 1) * 8;
  const size_t fixed = al((size_t)L.ww * 8) + al(((size_t)L.ww + 2) * 4) + staging + pcopies + 128;
  const size_t per32 = (size_t)kChunkStride * 4 + 8;  // int32 nodes + chunk total
  int32_t n32 = budget > fixed ? (int32_t)((budget - fixed) / per32) : 0;
  if (n32 > kMaxChunks) n32 = kMaxChunks;
  L.nch32 = n32;
  L.nch64 = (int32_t)(((size_t)n32 * kChunkStride * 4) / ((size_t)kChunkStride * 8));
  L.cap32 = (uint32_t)L.nch32 * kChunk;
  L.cap64 = (uint32_t)L.nch64 * kChunk;
  size_t o = al((size_t)L.ww * 8);
  L.off_rl = o;   o = al(o + ((size_t)L.ww + 2) * 4);
  L.off_fine = o; o = al(o + (size_t)n32 * kChunkStride * 4);
  L.off_T = o;    o = al(o + (size_t)n32 * 8);
  L.off_P = o;    o = al(o + pcopies);
  L.off_ring = o; o = al(o + sizeof(StepDesc) * Cfg::kRing);
  L.off_pdesc = o; o = al(o + sizeof(StepDesc) * Cfg::kRingFill);
  L.off_epre = o; o = al(o + 8 * (size_t)Cfg::kRing);
  L.off_qpre = o; o = al(o + 8 * (size_t)Cfg::kRing);
  L.off_ev = o;   o = al(o + Cfg::kBufs * (size_t)Cfg::kTileEv * 16);
  L.off_emeta = o; o = al(o + Cfg::kBufs * (size_t)Cfg::kTileEv);
  L.off_q = o;    o = al(o + Cfg::kBufs * (size_t)Cfg::kTileQ * 12);
  L.off_qmeta = o; o = al(o + Cfg::kBufs * (size_t)Cfg::kTileQ);
  L.off_corr = o; o = al(o + (size_t)kOfflineQ * 8);
  L.off_tiles = o; o = al(o + 3 * 32);
  L.bytes = o;
  return L;
}

// ------------------------------------------------------------------ host plan
// Tunable knobs of a pipeline (picked by the caller or the forest autotuner).
struct Tuning {
  int64_t block_work = 0;   // target work per state block (est_work units); 0 = auto
  int32_t ctas_per_sm = 0;  // persistent sweep CTAs per SM (1 or 2); 0 = auto
  int32_t slice_ranks = 0;  // cap on the ranks of one LUT slice (0 = all that fit shared memory)
  int32_t tile = 0;         // sweep tile geometry: kTileNarrowId, kTileWideId, 0 = by query/event ratio
};

// Everything the enqueue needs that does not depend on the data.  Built on the
// host from the tree shapes (for one tree: from the scalar arguments).
struct PipeSpec {
  int32_t T = 1;
  int32_t S = 0;                // total states
  int64_t E = 0, Q = 0;
  uint32_t Cmax = 1;
  int32_t Smax = 1;             // largest tree (bounds the list-ranking rounds)
  int32_t B = 1;                // total blocks
  int64_t bits_words = 0;       // sum over blocks of bitmap words
  int64_t carry_words = 0;      // sum over trees of (nb - 1) * (C + 1)
  int64_t gsum_words = 0;       // sum over trees with > kCarryGroup rows of groups * (C + 1)
  int32_t n_units = 0;          // carry units
  bool group_pass = false;      // some tree has more than one row group
  int32_t ctas_per_sm = 2;
  int32_t tile = kTileNarrowId;
  int32_t sms = 0;
  SweepLayout SL{};
  bool chain_hint = false;
  // one-tree scalars (T == 1): tables are written by a kernel at each launch
  int32_t nb1 = 1;
  // forest host tables, uploaded once by bind (empty for the plain one-tree spec)
  std::vector<int32_t> h_soff, h_boff;
  std::vector<int64_t> h_eoff, h_qoff, h_bits, h_carry, h_gsum;
  std::vector<uint32_t> h_C;
  std::vector<CarryUnit> h_units;
  std::vector<int32_t> h_order;
};

struct Layout {
  size_t off[40];
  size_t total;
};

enum {
  W_TSOFF, W_TEOFF, W_TQOFF, W_TC, W_TBOFF, W_TBITS, W_TCARRY, W_TGSUM, W_LASTQ, W_UNITS, W_ORDER,
  W_MISC, W_EOFF, W_QOFF, W_GPAR, W_FORK, W_NEXT, W_CNT, W_EHEAD, W_XHEAD, W_RANKA, W_RANKB,
  W_STEPS, W_DESC, W_TIN, W_TOUT, W_WORK, W_SCAN, W_BLOCKS, W_BMODE, W_BITS, W_RLUT, W_SLICES,
  W_NSLICES, W_CARRY, W_GSUM, W_COUNT
};

// misc words
enum { M_STATUS = 0, M_PREP_TICKET = 1, M_SWEEP_TICKET = 2, M_CHAIN = 3, M_PREPB_TICKET = 4, M_ROUNDS = 32 };  // 64 words

// Stage timing events of one launch: stage i runs from ev[i] to ev[i + 1]; a chain
// launch (chain = 1) records the sweep from ev[BW_STAGE_SWEEP] to ev[BW_STAGE_SWEEP+1]
// and the carry that follows it up to ev[BW_STAGE_COUNT + 1].
struct EventSet {
  cudaEvent_t ev[BW_STAGE_COUNT + 2];
  int chain = 0;
};

// Build the spec of a forest (tree shapes on the host).  Returns 0 or BW_EINVAL.
int pipe_spec_forest(int32_t T, const int64_t* soff, const int64_t* eoff, const int64_t* qoff,
                     const uint32_t* C, const Tuning& tune, int sms, PipeSpec& spec);
// Spec of one tree (the plain replay).
int pipe_spec_one(int32_t S, uint32_t C, int64_t E, int64_t Q, int32_t blocks, bool chain, const Tuning& tune,
                  int sms, PipeSpec& spec);
void pipe_layout(const PipeSpec& spec, Layout& L);
// Upload the forest tables into the workspace (no-op for one tree).  Synchronous.
int pipe_bind(const PipeSpec& spec, void* workspace, cudaStream_t st);
// Enqueue the whole pipeline (kernels and memsets only: capturable in a CUDA graph).
int pipe_enqueue(const PipeSpec& spec, void* workspace, const int32_t* parent, const BwEvent* events,
                 const BwQuery* queries, int64_t* answers, cudaStream_t st, EventSet* timing, int* kernels);
// Euler-tile sweep (bw_esweep.cu): the inputs of k_sweep, the rank capacities the
// prepare pass cut the slices with, events as 16-byte records (16-byte aligned).
struct EsParams {
  const uint4* ev;
  const BwQuery* qs;
  const StepDesc* desc;
  const BlockTab* blocks;
  const int32_t* order;   // queue order (NULL: identity)
  int32_t B;
  uint32_t cap32, cap64;
  const uint64_t* bits;
  const uint32_t* rlut;
  const Slice* slices;
  const int32_t* nslices;
  const int64_t* carry;
  int64_t* answers;
  int32_t* status;
  const int32_t* bmode;
  int32_t* ticket;
};
int esweep_attrs();   // one-time shared-memory opt-in (cudaError_t as int)
int esweep_launch(const EsParams& p, int grid, cudaStream_t st);

// Device address of the status word inside a workspace laid out for `spec`.
const int32_t* pipe_status_word(const PipeSpec& spec, const void* workspace);
int report(cudaError_t e, const char* what);

}  // namespace bw
