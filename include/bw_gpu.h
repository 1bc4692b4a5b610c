/*
 * bw_gpu.h -- C ABI of the GB300 (sm_103a) version-tree range-sum executor.
 *
 * Plain C types only (no CUDA or torch types), so the header is includable from
 * gcc, g++ and nvcc, like the reference's gpu_v7.h:1-2.  Every pointer named
 * "device" is device memory owned by the caller.  Every entry returns 0 on
 * success or the cudaError_t value of the failing CUDA call (as the reference's
 * *_launch functions do, gpu_v7.cu:98-121), after printing a one-line
 * diagnostic to stderr; argument errors return BW_EINVAL.  Launches are
 * asynchronous on the given stream (NULL = legacy default stream, as the
 * reference launches).
 *
 * Two families of entry points:
 *
 *  1. Drop-in replacements for the reference's GPU v7 interface
 *     (gpu_v7.h:7-50): same struct layouts, same argument meaning, same
 *     outputs (local endpoint prefixes `lvals`, dense block leaf deltas `dV`,
 *     answers of the combine), so the reference worker panel_batch_gpu.cpp can
 *     link this library unchanged.
 *
 *  2. The event-model replay (bw_replay_*): a version tree (parent array),
 *     int64 delta events (state, key, delta) grouped by state and range-sum
 *     queries (state, lo, hi) grouped by state.  The answer of query j is the
 *     wrapping int64 sum of the deltas of every event whose state lies on the
 *     root path of queries[j].state (inclusive) and whose key lies in [lo, hi);
 *     0 when hi <= lo.  This is the reference's per-state answer
 *     (oracle.cpp:357-422) restated over endpoint classes: a row edit or factor
 *     edit becomes class-delta events (batch_engine_v7.hpp:884-929), a query
 *     becomes the class interval [qlb, qhb) (batch_engine_v7.hpp:666-698).
 */
#ifndef BW_GPU_H
#define BW_GPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BW_EINVAL 1001

/* ===================================================================== v7 drop-in
 * Layouts identical to the reference (gpu_v7.h:7-47). */
struct GpuV7Node {  /* one edited state (node 0 is unused) */
  int32_t kind;     /* 1 row, 2 factor */
  int32_t g_old, c_old, ti_old;
  int32_t g_new, c_new, ti_new;
  int64_t amt_old, amt_new, fac_val, fac_prev;
  uint8_t ex_old, ex_new;
  uint8_t pad[6];
};

struct GpuV7Args {
  int B, G, Cpfx, ncls, q;
  const struct GpuV7Node* nodes; /* device, kStates entries */
  const int32_t* block_v0;       /* device, B */
  const int32_t* block_v1;       /* device, B */
  const int64_t* fac_start;      /* device, B*G factor vector at each block start */
  const int32_t* g2row;          /* device, G (-1: group never factor-edited) */
  const int32_t* ms_off;         /* device, n_active+1 merged-support offsets */
  const int64_t* ms_cls;         /* device, support classes */
  const int64_t* ms_base;        /* device, base mass at support classes */
  const int32_t* ms_dev;         /* device, deviation index or -1 */
  int64_t* devbuf;               /* device in/out, block-start deviation snapshots */
  const int64_t* need_off;       /* device, B*G offsets into devbuf, -1 when not needed */
  const int32_t* qlb;            /* device, kStates*q lower endpoint classes */
  const int32_t* qhb;            /* device, kStates*q upper endpoint classes */
  int64_t* lvals;                /* device out, (kStates-1)*2q local endpoint prefixes */
  int64_t* dV;                   /* device out, B*Cpfx dense block leaf deltas */
  int threads;                   /* hint only; the GB300 kernel picks its own width */
  int shared_bytes;              /* hint only */
};

struct GpuV7CombineArgs {
  int nstates;               /* kStates-1 */
  int q;
  int Cpfx;
  const int32_t* qlb;        /* device */
  const int32_t* qhb;        /* device */
  const int64_t* carrypref;  /* device, B*Cpfx */
  const int32_t* bidx;       /* device, kStates state -> block */
  const int64_t* lvals;      /* device */
  int64_t* answers;          /* device out, nstates*q */
};

/* Replaces gpu_v7_launch (gpu_v7.h:49, gpu_v7.cu:98-113): per state block, replay
 * the block's nodes from a zero local prefix, record the local prefix at both
 * declared endpoints of every query, and emit the block's dense leaf delta.
 * Updates devbuf exactly as the reference kernel does (gpu_v7.cu:29-37). */
int gpu_v7_launch(const struct GpuV7Args* a);
/* Replaces gpu_combine_launch (gpu_v7.h:50, gpu_v7.cu:115-121):
 * answers = carry prefix difference + local prefix difference. */
int gpu_combine_launch(const struct GpuV7CombineArgs* a);
/* Device-side replacement of the worker's host carry pass
 * (panel_batch_gpu.cpp:191-202): carrypref[b][k] = sum_{c<k} vstart_b[c],
 * vstart_0 = vbase, vstart_{b+1} = vstart_b + dV[b].  Same stream semantics. */
int bw_v7_carry_launch(int B, int Cpfx, const int64_t* vbase, const int64_t* dV,
                       int64_t* carrypref, void* stream);

/* ------------------------------------------------------------ v7b drop-in
 * Layouts identical to the reference's compact plan (gpu_v7b.h:6-48): a 40-byte node
 * (kind bits: 1 row, 2 factor, bit 2 ex_old, bit 3 ex_new; a, b = amt_old, amt_new
 * for a row edit, fac_val, fac_prev for a factor edit) and block-start deviation
 * snapshots made on the device by the snapshot entry. */
struct GpuV7bNode {
  uint8_t kind;
  int16_t g_old, g_new;
  int32_t c_old, c_new;
  int32_t ti_old, ti_new;
  int64_t a, b;
};

struct GpuV7bSnapArgs {
  int nstates;                  /* kStates */
  const struct GpuV7bNode* nodes;
  const int32_t* bidx;          /* state -> block */
  const int32_t* gb_off;        /* G+1 */
  const int32_t* gb_block;      /* per (group, block) occurrence, ascending blocks per group */
  const int64_t* gb_reg;        /* devbuf offset of the group's region in that block */
  int64_t* devbuf;              /* in/out: snapshots accumulate into it (caller zeroes it) */
};

struct GpuV7bArgs {
  int B, G, Cpfx, ncls, q;
  const struct GpuV7bNode* nodes;
  const int32_t *bv0, *bv1;
  const int64_t* fac_start;     /* B*G */
  const int32_t* g2row;         /* G */
  const int32_t* ms_off;        /* n_active+1 */
  const int64_t *ms_cls, *ms_base;
  const int32_t* ms_dev;
  int64_t* devbuf;
  const int64_t* need_off;      /* B*G */
  const int32_t *qlb, *qhb;
  int64_t *lvals, *dV;
  int threads;                  /* hint only */
  int shared_bytes;             /* hint only */
};

struct GpuV7bCombineArgs {      /* same layout as GpuV7CombineArgs */
  int nstates, q, Cpfx;
  const int32_t *qlb, *qhb;
  const int64_t* carrypref;     /* B*Cpfx */
  const int32_t* bidx;
  const int64_t* lvals;
  int64_t* answers;
};

/* Replace gpu_v7b_snap_launch / gpu_v7b_launch / gpu_v7b_combine_launch
 * (gpu_v7b.h:50-52, gpu_v7b.cu:13-141): the snapshot entry adds every row edit's
 * deviation delta into the regions of the later blocks that need its group; the
 * block and combine entries are those of gpu_v7.h on the compact node.  Default
 * stream, asynchronous. */
int gpu_v7b_snap_launch(const struct GpuV7bSnapArgs* a);
int gpu_v7b_launch(const struct GpuV7bArgs* a);
int gpu_v7b_combine_launch(const struct GpuV7bCombineArgs* a);

/* ------------------------------------------------------------ session drop-in
 * Layouts identical to the reference's session backend (gpu_session.h:4-20): the
 * prefix structure of each block lives in caller-owned global memory (fen, leaf:
 * B*Cpfx int64 each), so the class domain is not bounded by shared memory; a
 * session uploads once and reruns run + combine per query batch. */
struct GpuSessNode { uint8_t kind; int16_t g_old, g_new; int32_t c_old, c_new, ti_old, ti_new; int64_t a, b; };
struct GpuSessResetArgs { int B, Cpfx; int64_t* fen; int64_t* leaf; };
struct GpuSessRunArgs {
  int B, G, Cpfx, ncls, q;
  const struct GpuSessNode* nodes;
  const int32_t *bv0, *bv1;
  const int64_t* fac_start;
  const int32_t* g2row;
  const int32_t* ms_off; const int64_t *ms_cls, *ms_base; const int32_t* ms_dev;
  int64_t* devbuf; const int64_t* need_off;
  const int32_t *qlb, *qhb;
  int64_t* lvals; int64_t* dV;
  int64_t* fen; int64_t* leaf;  /* B*Cpfx each */
  int threads;                  /* hint only */
};
struct GpuSessCombineArgs { int nstates, q, Cpfx; const int32_t *qlb, *qhb; const int64_t* carrypref;
                            const int32_t* bidx; const int64_t* lvals; int64_t* answers; };
struct GpuSessSnapArgs { int nstates; const struct GpuSessNode* nodes; const int32_t* bidx; const int32_t* gb_off;
                         const int32_t* gb_block; const int64_t* gb_reg; int64_t* devbuf; };

/* Replace gpu_sess_reset_launch / gpu_sess_run_launch / gpu_sess_snap_launch /
 * gpu_sess_combine_launch (gpu_session.h:21-24): reset zeroes fen and leaf, run
 * replays every block with its prefix structure in fen/leaf and writes lvals, the
 * block leaf deltas into both leaf and dV, and devbuf as gpu_v7_launch does;
 * snap and combine are the v7b ones. */
int gpu_sess_reset_launch(const struct GpuSessResetArgs* a);
int gpu_sess_run_launch(const struct GpuSessRunArgs* a);
int gpu_sess_snap_launch(const struct GpuSessSnapArgs* a);
int gpu_sess_combine_launch(const struct GpuSessCombineArgs* a);

/* ===================================================================== event model */
typedef struct { uint32_t state, key; int64_t delta; } BwEvent;   /* 16 bytes */
typedef struct { uint32_t state, lo, hi; } BwQuery;               /* 12 bytes */

typedef struct {
  int32_t n_states;          /* states 0..n_states-1; state 0 is the root */
  const int32_t* parent;     /* device, n_states; parent[0] = -1, parent[v] < v */
  uint32_t n_keys;           /* key domain [0, n_keys); query bounds lie in [0, n_keys] */
  int64_t n_events;
  const BwEvent* events;     /* device, grouped by state (non-decreasing state), 16-byte aligned
                                (misaligned events are refused: BW_EINVAL) */
  int64_t n_queries;
  const BwQuery* queries;    /* device, grouped by state (non-decreasing state) */
  int64_t* answers;          /* device out, n_queries */
  void* workspace;           /* device, >= bw_replay_workspace_size(); 256-byte aligned */
  size_t workspace_bytes;
  void* stream;              /* cudaStream_t or NULL */
  int32_t blocks;            /* state blocks; 0 = pick from the device and the workload */
  int32_t flags;             /* BW_REPLAY_* */
} BwReplayArgs;

#define BW_REPLAY_CHAIN_HINT 1  /* caller asserts parent[v] == v-1; any fork is rejected (BW_STATUS_BAD_PARENT) */
#define BW_REPLAY_TIMING 2      /* record CUDA events between pipeline stages (see below) */
/* With BW_REPLAY_CHAIN_HINT, a key domain of at most 32,768 keys and 16-byte aligned
 * events, the replay takes the single-pass chain path (each event read once, no
 * Euler tour) when the workload has at most one query per 8 events; these flags
 * force either path instead (tests, benchmarks). */
#define BW_REPLAY_CHAIN_KERNEL 4
#define BW_REPLAY_GENERAL 8
/* Chain path: keep the running key histogram as int64 (exact at any delta size, two
 * 32-bit shared atomics per update) instead of int32 windows -- for chains whose
 * deltas mostly lie outside (-2^19, 2^19), e.g. amount x factor products of the
 * reference-native workloads.  Key domains up to 16,384 keys; ignored above. */
#define BW_REPLAY_WIDE 16

/* Pipeline stages timed under BW_REPLAY_TIMING, in order (the chain path has only
 * the sweep, which reads the events, and the carry scan with the answer fix-up that
 * follows it; its other stages read 0). */
enum {
  BW_STAGE_INGEST = 0,     /* per-state offsets + validation */
  BW_STAGE_LINEARISE = 1,  /* Euler tour / chain layout */
  BW_STAGE_BLOCKS = 2,     /* work prefix + block cut */
  BW_STAGE_PREPARE = 3,    /* block rank tables, slices, net key-prefix rows */
  BW_STAGE_CARRY = 4,      /* carry scan over blocks */
  BW_STAGE_SWEEP = 5,      /* block sweep and answers */
  BW_STAGE_COUNT = 6
};

/* Input errors found on the device are reported through bw_replay_status(). */
enum {
  BW_STATUS_OK = 0,
  BW_STATUS_EVENTS_UNSORTED = 1,
  BW_STATUS_EVENT_KEY_RANGE = 2,
  BW_STATUS_QUERIES_UNSORTED = 3,
  BW_STATUS_QUERY_RANGE = 4,
  BW_STATUS_BAD_PARENT = 5,
  BW_STATUS_TOO_MANY_SLICES = 6,
  BW_STATUS_STATE_RANGE = 7,
  BW_STATUS_TIMEOUT = 8      /* a bounded device wait gave up (the kernel returned early) */
};

/* Bytes of device workspace needed for these arguments (pointers unused). */
int bw_replay_workspace_size(const BwReplayArgs* a, size_t* bytes);
/* Enqueue the whole replay (ingest offsets, tree linearisation, block plan, carry
 * scan, block sweep) on a->stream.  Reads only the inputs, writes answers and the
 * workspace. */
int bw_replay_launch(const BwReplayArgs* a);
/* Synchronise a->stream and read the device status word written by the last
 * bw_replay_launch with this workspace; *status receives a BW_STATUS_* code. */
int bw_replay_status(const BwReplayArgs* a, int32_t* status);
/* Number of kernels the most recent bw_replay_launch of this process enqueued (any
 * workspace, any thread: the record is process-wide) and the state-block count it
 * used (host-side bookkeeping, no synchronisation). */
int bw_replay_last_info(const BwReplayArgs* a, int32_t* kernels, int32_t* blocks);
/* *chain = 1 when these arguments take the single-pass chain path, 0 for the
 * general pipeline (host-side decision from the sizes, flags and event alignment). */
int bw_replay_path(const BwReplayArgs* a, int32_t* chain);

/* Stage timing over a run of launches made with BW_REPLAY_TIMING (CUDA events
 * recorded on each launch's stream).  bw_replay_timing_reset() starts a new run;
 * bw_replay_stage_times() synchronises on the last recorded event and writes the
 * per-stage milliseconds summed over the run's launches (ms[BW_STAGE_COUNT]) and
 * the number of launches.  Process-wide, for one host thread at a time. */
int bw_replay_timing_reset(void);
int bw_replay_stage_times(float* ms, int32_t* launches);

/* The replay for callers that cannot allocate device memory when they run it (a
 * plugin inside a host engine with a fixed memory budget, a loop that must not
 * block in the allocator).  No counterpart in the reference.  Same arguments and
 * results as bw_replay_launch, except that a->workspace must be NULL and
 * a->workspace_bytes 0: the scratch comes from a fixed 32 MiB region compiled into
 * the library (held by every GPU that loads it until exit); workloads needing more
 * (bw_replay_workspace_size) are rejected with BW_EINVAL.  Nothing is allocated or
 * freed.  Every call looks the region's device address up on the current device
 * (an allocation-free lookup that stays right after a context reset); the first
 * call on a device loads the library's module there and should come before any
 * stream capture.  Calls share the region, so calls overlapping on the GPU race.
 * A non-NULL host `status` makes the call wait for its stream and receive the
 * BW_STATUS_* code; NULL returns once the work is enqueued, and the device's input
 * check is then not reported. */
int bw_replay_launch_noalloc(const BwReplayArgs* a, int32_t* status);

/* ============================================================ one chain across ranks
 * A chain split into contiguous state ranges, one per rank (one process per GPU):
 * each rank replays its range as a chain of its own (local states start at 0), and
 * the only exchange is the carry, an exclusive scan over ranks of each rank's dense
 * key histogram -- the reference's serial carry pass (batch_engine_v7.hpp:936-945)
 * lifted from state blocks to ranks; the carry is then added to the rank's answers
 * inside [lo, hi) as the reference's combine does (batch_engine_v7.hpp:948-961).
 * The scan is the caller's (an identity on one rank; torch.distributed between
 * processes).  Asynchronous on `stream`. */
/* hist[k] = wrapping sum of the deltas of events with key k, k < n_keys (device
 * arrays; the call zeroes hist first; keys >= n_keys are ignored). */
int bw_key_histogram(const BwEvent* events, int64_t n, uint32_t n_keys, int64_t* hist, void* stream);
/* prefix[k] = sum of vec[j] for j < k, k = 0..n (prefix holds n+1 entries). */
int bw_key_prefix(const int64_t* vec, uint32_t n, int64_t* prefix, void* stream);
/* answers[i] += prefix[hi] - prefix[lo] for every query with lo < hi (bounds clamped to
 * n_keys): the carry below the rank inside each query's interval. */
int bw_add_range_carry(const BwQuery* queries, int64_t n, uint32_t n_keys, const int64_t* prefix,
                       int64_t* answers, void* stream);
/* dst[slot[i]] = src[i] for every i with 0 <= slot[i] < n_dst (device arrays): the
 * answers of a BWLEV001 stream workload's chain queries, in stream order, into the
 * reference's (state, k) answer order (bw_stream_build's slot, include/bw_host.h). */
int bw_scatter_answers(const int64_t* src, const int64_t* slot, int64_t n, int64_t* dst, int64_t n_dst,
                       void* stream);

/* ============================================================ grouping by state
 * The replay takes events and queries grouped by state (non-decreasing).  Arrays in
 * another order are grouped on the device by a stable radix sort on the state (8
 * bits per pass over the bits n_states needs).  bw_group_queries also writes
 * order[i] = the input index of output query i, so the answers of the grouped
 * queries go back to input order with bw_scatter_answers(answers, order, ...).  The
 * first pass checks every state against n_states: bw_group_status then reads
 * BW_STATUS_STATE_RANGE (synchronises).  Events must be 16-byte aligned; the input
 * and output arrays must differ. */
int bw_group_workspace_size(int64_t n, int32_t queries, size_t* bytes);
int bw_group_events(const BwEvent* in, int64_t n, int32_t n_states, BwEvent* out, void* workspace,
                    size_t workspace_bytes, void* stream);
int bw_group_queries(const BwQuery* in, int64_t n, int32_t n_states, BwQuery* out, int64_t* order,
                     void* workspace, size_t workspace_bytes, void* stream);
int bw_group_status(const void* workspace, int32_t* status);

/* ============================================================ chain setup on the device
 * The factor expansion of a reference-native chain (the bulk of its events: a factor
 * edit of group g becomes one event per class of g's support) built on the GPU.
 * The host compiles the chain into this compact form (bw_native_build_compact,
 * include/bw_host.h): the events that are copied verbatim (base rows and row edits)
 * with their output positions, every group's support and base mass, and per group
 * the timeline of its mass updates and factor expansions in state order.  The
 * device applies a group's updates between expansions (they commute) and writes
 * each expansion (state, class, ds * mass) at its output range. */
typedef struct {
  int32_t state;
  int32_t idx;        /* support index of a mass update; -1 for an expansion */
  int64_t value;      /* mass delta, or the expansion's factor delta ds */
  int64_t out;        /* expansion: output position of its first event */
} BwTimeline;

typedef struct {
  int32_t n_states, n_groups;
  uint32_t n_keys;
  int64_t n_events;       /* events the expansion writes in all */
  int64_t n_queries;
  int32_t* parent;        /* n_states (a chain) */
  BwQuery* queries;       /* n_queries, reference answer order */
  int64_t n_fixed;
  BwEvent* fixed;         /* events copied verbatim ... */
  int64_t* fixed_pos;     /* ... to these output positions */
  int64_t* sup_off;       /* n_groups + 1 */
  uint32_t* sup_cls;      /* group g's classes: sup_cls[sup_off[g] .. sup_off[g+1]) */
  int64_t* base_mass;     /* parallel to sup_cls */
  int64_t* tl_off;        /* n_groups + 1 */
  BwTimeline* tl;         /* group g's timeline: tl[tl_off[g] .. tl_off[g+1]) */
} BwNativeCompact;

/* Device scratch for bw_native_expand (the compact arrays and per-group masses). */
int bw_native_expand_workspace(const BwNativeCompact* c, size_t* bytes);
/* Upload the compact form (host arrays) into `workspace` and write all n_events
 * events, grouped by state, to `events` (device).  Enqueued on `stream`; the host
 * arrays must stay valid until the stream reaches this point. */
int bw_native_expand(const BwNativeCompact* c, BwEvent* events, void* workspace, size_t workspace_bytes,
                     void* stream);

/* ============================================================ batched version forests
 * Thousands of independent version trees replayed in one pipeline (the reference
 * replays one chain per worker process, panel_batch_gpu.cpp:182-214, and its
 * parallel_jobs.py runs many of those side by side).  Tree t owns states
 * [state_off[t], state_off[t+1]), events [event_off[t], event_off[t+1]), queries
 * [query_off[t], query_off[t+1]) and the key domain [0, n_keys[t]); each tree's
 * slice of `parent`, `events` and `queries` is exactly a plain replay input
 * (tree-local state ids, parent[local 0] = -1, parent[l] < l, events and queries
 * grouped by local state).  answers[j] is the plain answer of query j within its
 * tree.  Every tree is cut into state blocks that never span trees; persistent
 * CTAs take the blocks from one queue, largest estimated work first. */
typedef struct {
  int32_t n_trees;
  const int64_t* state_off;  /* host, n_trees+1 (state_off[0] = 0; every tree has >= 1 state) */
  const int64_t* event_off;  /* host, n_trees+1 */
  const int64_t* query_off;  /* host, n_trees+1 */
  const uint32_t* n_keys;    /* host, n_trees */
} BwForestShape;

typedef struct {
  int64_t block_work;   /* target work of one state block, in event units (an event 2,
                           a query 2, an Euler step 64); 0 = auto */
  int32_t ctas_per_sm;  /* persistent sweep CTAs per SM, 1 or 2; 0 = auto */
  int32_t slice_ranks;  /* cap on the distinct keys of one rank-LUT slice held in
                           shared memory; 0 = as many as fit */
  int32_t tile;         /* sweep tile geometry: 1 narrow (256 threads, 2 events + 2 queries
                           staged per thread, 32 steps), 2 wide (256 threads, 4 events + 1
                           query, 64 steps), 3 and 4 the same tiles on 512 threads (one
                           CTA per SM), 5 the 512-thread tile with one warp staging
                           tiles for the other fifteen, 6 the Euler-tile sweep (a
                           planner and an issuer warp bulk-copy signed event tiles for
                           sixteen consumer warps over a flat shared-memory window; one
                           CTA per SM); 0 = 6 */
  int32_t reserved;
} BwForestTuning;

typedef struct BwForest BwForest;   /* opaque plan: host tables, layout, CUDA graph */

/* Plan a forest (host only; NULL tuning = auto).  BW_EINVAL for malformed shapes. */
int bw_forest_create(const BwForestShape* shape, const BwForestTuning* tuning, BwForest** out);
int bw_forest_workspace_size(const BwForest* f, size_t* bytes);
/* Attach a device workspace (>= bw_forest_workspace_size, 256-byte aligned) and
 * upload the plan's tables into it; synchronises `stream`.  Needed once per
 * workspace, before any launch or capture. */
int bw_forest_bind(BwForest* f, void* workspace, size_t workspace_bytes, void* stream);
/* Enqueue the whole replay on `stream`: kernels and one memset, no host copies. */
int bw_forest_launch(BwForest* f, const int32_t* parent, const BwEvent* events, const BwQuery* queries,
                     int64_t* answers, void* stream);
/* Capture bw_forest_launch with these device pointers into a CUDA graph owned by
 * the plan (stream must not be the legacy default stream); bw_forest_graph_launch
 * replays it. */
int bw_forest_capture(BwForest* f, const int32_t* parent, const BwEvent* events, const BwQuery* queries,
                      int64_t* answers, void* stream);
int bw_forest_graph_launch(BwForest* f, void* stream);
/* One launch with CUDA events between the pipeline stages; synchronises `stream`
 * and writes the milliseconds of each stage (ms[BW_STAGE_COUNT], BW_STAGE_*). */
int bw_forest_launch_timed(BwForest* f, const int32_t* parent, const BwEvent* events, const BwQuery* queries,
                           int64_t* answers, void* stream, float* ms);
/* Synchronise `stream` and read the device status word (BW_STATUS_*). */
int bw_forest_status(BwForest* f, void* stream, int32_t* status);
/* Blocks, kernels per launch, and the tuning in effect. */
int bw_forest_info(const BwForest* f, int32_t* blocks, int32_t* kernels, BwForestTuning* tuning);
int bw_forest_destroy(BwForest* f);
/* Host-only planning (no device call): the blocks, workspace bytes and dense carry
 * bytes bw_forest_create would plan for this shape and tuning on a GPU with `sms`
 * multiprocessors. */
int bw_forest_plan_stats(const BwForestShape* shape, const BwForestTuning* tuning, int32_t sms, int32_t* blocks,
                         size_t* workspace_bytes, size_t* carry_bytes);
/* Autotuner: times candidate tunings on the caller's inputs (sweep CTAs per SM x
 * block work, then the other tile geometry, then narrower LUT slices, each at the
 * best so far) with `reps` launches after a warm-up, skips candidates the device
 * rejects, and returns the fastest in *best (and its mean milliseconds).  The
 * workspace must hold bw_forest_autotune_workspace bytes; answers are overwritten.
 * BW_EINVAL when no candidate ran (invalid input). */
int bw_forest_autotune_workspace(const BwForestShape* shape, size_t* bytes);
int bw_forest_autotune(const BwForestShape* shape, const int32_t* parent, const BwEvent* events,
                       const BwQuery* queries, int64_t* answers, void* workspace, size_t workspace_bytes,
                       void* stream, int32_t reps, BwForestTuning* best, float* best_ms);

/* ============================================================ served version store
 * A device-resident version store answering range-sum queries and creating
 * versions (commits of int64 delta events, forks) as requests arrive, from a
 * persistent request loop (one request per warp) fed through host-mapped memory.
 * It starts from an initial tree (the event-model inputs of bw_replay, on the
 * host).  Every version keeps its own events as a key-sorted overlay; versions on
 * a regular spacing keep a dense key-prefix row of their whole root path
 * (checkpoints), the others read their nearest checkpoint ancestor's row plus the
 * overlays of at most `spacing` member versions.  The spacing is the densest whose
 * store fits hbm_cap_bytes.  No counterpart in the reference, which answers one
 * offline batch per worker process (panel_gpu_session.cpp:110-137 runs repeated
 * batches against one session). */
enum { BW_REQ_QUERY = 0, BW_REQ_COMMIT = 1, BW_REQ_FORK = 2 };

typedef struct {
  uint32_t kind;         /* BW_REQ_* */
  uint32_t version;      /* query: the version read; commit/fork: the parent version */
  uint32_t lo, hi;       /* query: key interval [lo, hi) */
  uint32_t new_version;  /* commit/fork: the next free version id (ids are created in log order) */
  uint32_t n_events;     /* commit: events commit_events[events_off, events_off + n_events), <= 128 */
  uint64_t events_off;
} BwServeRequest;        /* 32 bytes */

typedef struct {
  int32_t n_states;          /* initial tree: states 0..n_states-1 */
  const int32_t* parent;     /* host, n_states (parent[0] = -1, parent[v] < v) */
  uint32_t n_keys;           /* key domain */
  int64_t n_events;
  const BwEvent* events;     /* host, grouped by state */
  int32_t max_versions;      /* capacity: initial states + versions runs may create */
  int64_t max_events;        /* event arena: initial events + events runs may commit */
  size_t hbm_cap_bytes;      /* admission cap of the whole store */
  int32_t chain_limit;       /* largest checkpoint spacing allowed (<= 32; 0 = 32) */
  uint32_t spin_limit;       /* polls (each with a nanosleep backoff of up to ~2 us) before a
                                device wait for an unpublished request or an unfinished version
                                gives up and ends the run with an error; 0 = 2^25 */
} BwServeConfig;

typedef struct {
  int64_t requests, queries, commits, forks;
  double wall_s;             /* first arrival to last completion */
  int32_t checkpoints;       /* dense rows in the store */
  int32_t spacing;           /* checkpoint spacing in versions */
  size_t store_bytes;        /* device bytes of the store */
  int32_t warps;             /* request-loop warps */
  int32_t reserved;
} BwServeStats;

typedef struct BwServe BwServe;

/* Build the store on the current device (allocates it; checkpoint rows are built
 * level by level).  BW_EINVAL for malformed input or a store over the cap. */
int bw_serve_create(const BwServeConfig* cfg, BwServe** out);
/* Forget every version and event created by runs (back to the initial tree). */
int bw_serve_reset(BwServe* s);
/* Serve a request log: request i is published at t0 + arrival_s[i] (NULL: at
 * once) while at most max_inflight requests are unfinished; the persistent loop
 * executes requests concurrently (a request waits only for the versions it reads).
 * answers[i] receives the range sum of query i (0 for commits and forks) and
 * latency_us[i] its completion time minus its arrival time, both on the host
 * clock.  The log is checked first (versions exist before they are read, new ids
 * are consecutive, bounds and keys in range) and admitted only if its commit
 * events fit the free event arena.  Blocks until every request completes or
 * timeout_s elapses, or a device wait reaches its spin_limit (both BW_EINVAL, after
 * the loop has returned; the store stays usable and bw_serve_reset forgets the
 * partial run). */
int bw_serve_run(BwServe* s, const BwServeRequest* reqs, int64_t n, const BwEvent* commit_events,
                 int64_t n_commit_events, const double* arrival_s, int32_t max_inflight, double timeout_s,
                 int64_t* answers, float* latency_us, BwServeStats* stats);
int bw_serve_info(const BwServe* s, BwServeStats* stats);
int bw_serve_destroy(BwServe* s);

/* ============================================================ sparse-key rank index */
/* The CSR rank-LUT of the reference's sparse engine (CsrBase, sparse_engine.hpp:70-102;
 * build_csr_base, sparse_engine.hpp:287-360) over a sparse key universe
 * [0, 2^key_bits): a sorted array of the distinct keys, the cumulative amount prefix
 * over them (pre[i] = sum of the amounts of keys <= keys[i]) and a rank LUT with one
 * u32 entry per bucket of 2^shift keys (lut[b] = number of keys below b << shift).
 * rank(k) = lut[k >> shift] + #(keys in that bucket below k), the reference's
 * rlut[word] + popcount(bits & mask) with buckets in place of 64-key words, so the
 * table fits a byte budget for any universe.  Keys >= 2^key_bits rank as the count. */
typedef struct {
  int32_t key_bits;          /* universe [0, 2^key_bits), 1..63 */
  int32_t shift;             /* bucket width 2^shift */
  int64_t n_buckets;         /* 2^(key_bits - shift) */
  const int64_t* count;      /* device, 1: number of distinct keys m */
  const int32_t* status;     /* device, 1: 0, or 1 when a build key was >= 2^key_bits */
  const uint64_t* keys;      /* device, m ascending distinct keys */
  const int64_t* pre;        /* device, m cumulative amounts (wrapping int64) */
  const uint32_t* lut;       /* device, n_buckets */
  const uint16_t* low;       /* device, m low `shift` bits of the keys (shift <= 16), else NULL */
} BwCsr;

/* Workspace for bw_csr_build over n_items (key, amount) pairs with a LUT budget of
 * lut_budget_bytes (the LUT takes the largest power-of-two bucket count that fits). */
int bw_csr_workspace_size(int64_t n_items, int32_t key_bits, size_t lut_budget_bytes, size_t* bytes);
/* Device radix sort of the pairs by key, run-length merge of equal keys (amounts
 * summed), cumulative amount prefix, and the bucket LUT; all on `stream`,
 * asynchronous.  The index arrays live in the workspace, which must outlive every
 * lookup; *out receives their device addresses.  Keys must be < 2^key_bits: a
 * larger key sets the device status word (bw_csr_status) and leaves the lookups
 * unspecified but in bounds.  BW_EINVAL for n_items >= 2^31. */
int bw_csr_build(const uint64_t* keys, const int64_t* amounts, int64_t n_items, int32_t key_bits,
                 size_t lut_budget_bytes, void* workspace, size_t workspace_bytes, void* stream,
                 BwCsr* out);
/* Point lookups: out[i] = rank(keys[i]) when keys[i] is present, -rank-1 when
 * absent (rank = number of index keys below keys[i]).  Device arrays of n. */
int bw_csr_point(const BwCsr* idx, const uint64_t* keys, int64_t n, int64_t* out, void* stream);
/* Range lookups, CsrBase::range semantics (sparse_engine.hpp:89-97):
 * bounds[2i], bounds[2i+1] = lo, hi; out[2i] = rank(hi) - rank(lo) and
 * out[2i+1] = pre-sum over the keys in [lo, hi) (both negative when hi < lo,
 * as in the reference). */
int bw_csr_range(const BwCsr* idx, const uint64_t* bounds, int64_t n, int64_t* out, void* stream);
/* Synchronise the device and read the build's status word (0 = valid input). */
int bw_csr_status(const BwCsr* idx, int32_t* status);
/* Versioned sparse keys: the event model over the index's ranks, so a version tree
 * whose events carry u64 keys (config 3's chain-with-forks over sparse keys) replays
 * with bw_replay_launch at n_keys = the index's key count.  bw_csr_events: out[i] =
 * (states[i], rank of keys[i], deltas[i]); a key missing from the index gets rank m
 * (the replay then reports BW_STATUS_EVENT_KEY_RANGE).  bw_csr_queries: hi == NULL,
 * point lookups -- (states[i], rank, rank + 1) for a present lo[i], an empty interval
 * for an absent one; else range lookups over keys [lo[i], hi[i]) -- (states[i],
 * rank(lo[i]), rank(hi[i])), empty when hi <= lo.  rank = index keys below the key. */
int bw_csr_events(const BwCsr* idx, const uint32_t* states, const uint64_t* keys, const int64_t* deltas,
                  int64_t n, BwEvent* out, void* stream);
int bw_csr_queries(const BwCsr* idx, const uint32_t* states, const uint64_t* lo, const uint64_t* hi,
                   int64_t n, BwQuery* out, void* stream);

/* Library/device information: SM count of the current device and the library's
 * compile-time architecture tag (e.g. 1030 for sm_103a). */
int bw_device_info(int32_t* sm_count, int32_t* arch_tag);

#ifdef __cplusplus
}
#endif
#endif
