/*
 * bw_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the BiWorldDB version-tree range-sum semantics, used as the
 * checker for the GPU path.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load this library; the product never links or calls it.
 *
 * Two families of checkers live here:
 *
 *  1. Reference-native workloads (fixture BWBASE02 + deterministic declared edits):
 *     bwo_workload_make() restates common.hpp:279-374 (make_workload) and
 *     bwo_direct_scan() restates the independent oracle of oracle.cpp:213-451:
 *     full mutable row state, DFS apply/revert, one direct scan of every row per
 *     state, __int128 accumulation with an int64 overflow check.
 *
 *  2. The generic event model (configs of the GPU path): a version tree, events
 *     (state, key, delta) and queries (state, lo, hi).  The answer of a query is
 *     the wrapping int64 sum of the deltas of every event whose state is an
 *     ancestor-or-self of the query state and whose key lies in [lo, hi); it is 0
 *     when hi <= lo.  bwo_ev_bruteforce() walks ancestors; bwo_ev_sweep() is the
 *     preorder apply/undo Fenwick replay of batch_engine_v7.hpp:1021-1059;
 *     bwo_ev_blocks() is the block-parallel chain executor of
 *     batch_engine_v7.hpp:832-968 (phase 1 local Fenwick per block, phase 2
 *     serial carry, phase 3 combine) used as the timed CPU baseline.
 *
 * Parity is pinned by the reference's committed golden answer vectors
 * (results/general_router_final2_20261102/raw/1d_q{2,8}_oracle_r0.bin) and by
 * hashes of the reference binaries built from source (oracle/ref.mk).
 */
#ifndef BW_ORACLE_H
#define BW_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- digests */
/* SHA-256 (FIPS 180-4) of n bytes; writes 64 lowercase hex chars + NUL. */
void bwo_sha256_hex(const void* data, size_t n, char out_hex[65]);
/* 64-bit FNV-1a, as common.hpp:396-400. */
uint64_t bwo_fnv1a(const void* data, size_t n);

/* ---------------------------------------------------------------- RNG */
uint64_t bwo_splitmix_next(uint64_t* state);

/* ---------------------------------------------------------------- fixture */
typedef struct {
  int64_t n;
  int32_t groups;
  int32_t unit;
  int64_t t_min, t_max;
  const int64_t* row_t;     /* stride 3 int64 words per row: t, amount, (g,pad) */
  const uint8_t* rows;      /* raw 24-byte records */
  const int64_t* factor;    /* groups */
  const int32_t* labels;    /* groups */
} bwo_fixture;

/* Parse a BWBASE02 image held in memory (common.hpp:57-75, 112-155).
 * Returns 0 on success, 3 on a malformed image. */
int bwo_fixture_parse(const void* image, size_t len, bwo_fixture* f);

/* ---------------------------------------------------------------- workload */
enum { BWO_OP_REPLACE = 0, BWO_OP_INSERT = 1, BWO_OP_DELETE = 2, BWO_OP_MOVE = 3, BWO_OP_FACTOR = 4 };

typedef struct {
  int32_t n_states, topology, seed, factor_period, q, per_state, factor_pct;
  int64_t n_base;
  int32_t groups, n_inserted;
  int64_t t_min, t_max;
  int32_t* parent;     /* n_states */
  uint8_t* op;         /* n_states (index 0 unused) */
  int32_t* eg;         /* edit group */
  int64_t* eid;        /* edit row id */
  int64_t* eval;       /* amount or factor */
  int64_t* et;         /* edit timestamp */
  int64_t* qlo;        /* n_states*q (per-state) or q (shared) */
  int64_t* qhi;
  int64_t* ins_t;      /* n_inserted */
  int32_t* ins_g;
  int64_t* endpoints;  /* sorted distinct declared endpoints */
  int64_t n_endpoints;
} bwo_workload;

/* Build the declared workload (common.hpp:279-374); factor_pct < 0 keeps the
 * factor-period pattern.  Returns 0 or an error code. */
int bwo_workload_make(const bwo_fixture* f, int32_t n_states, int32_t topology, int32_t seed,
                      int32_t factor_period, int32_t q, int32_t per_state, int32_t factor_pct,
                      bwo_workload* w);
void bwo_workload_free(bwo_workload* w);

/* Independent direct-scan oracle (oracle.cpp:213-451).  answers: (n_states-1)*q
 * int64 in order v=1..n_states-1, k=0..q-1.  Returns 0, or 6 when an answer
 * does not fit int64 (the reference oracle exits 6 there). */
int bwo_direct_scan(const bwo_fixture* f, const bwo_workload* w, int64_t* answers);

/* ---------------------------------------------------------------- event model */
typedef struct { uint32_t state, key; int64_t delta; } bwo_event;   /* 16 bytes */
typedef struct { uint32_t state, lo, hi; } bwo_query;               /* 12 bytes */

/* Ancestor walk; returns 0, or 6 if some exact answer overflows int64 (the
 * wrapped value is still written). */
int bwo_ev_bruteforce(int32_t n_states, const int32_t* parent, int64_t n_events,
                      const bwo_event* ev, int64_t n_queries, const bwo_query* qs,
                      int64_t* answers);
/* Preorder apply/undo Fenwick replay over key domain [0, n_keys). */
int bwo_ev_sweep(int32_t n_states, const int32_t* parent, uint32_t n_keys, int64_t n_events,
                 const bwo_event* ev, int64_t n_queries, const bwo_query* qs, int64_t* answers);
/* Same sweep restricted to the first `limit_steps` preorder entries (bounded CPU
 * baseline sample); returns the number of queries answered via *answered and the
 * wall time of the replay loop alone (input grouping excluded) via *seconds. */
int bwo_ev_sweep_prefix(int32_t n_states, const int32_t* parent, uint32_t n_keys,
                        int64_t n_events, const bwo_event* ev, int64_t n_queries,
                        const bwo_query* qs, int64_t* answers, int64_t limit_steps,
                        int64_t* answered, double* seconds);
/* Block-parallel chain executor with OpenMP (chains only: parent[v] == v-1).
 * blocks <= 0 picks the thread count.  Returns 0, or 2 if the tree is not a chain. */
int bwo_ev_blocks(int32_t n_states, const int32_t* parent, uint32_t n_keys, int64_t n_events,
                  const bwo_event* ev, int64_t n_queries, const bwo_query* qs,
                  int64_t* answers, int32_t blocks, int32_t threads);
int bwo_max_threads(void);

/* -------------------------------------------------------- sparse-key rank index */
/* CSR build (build_csr_base, sparse_engine.hpp:287-360, over u64 keys): the
 * distinct keys ascending (out_keys) and the cumulative amount prefix over them
 * (out_pre[i] = wrapping sum of the amounts of every key <= out_keys[i]); *m
 * receives the distinct count.  out_* hold n entries. */
int bwo_csr_build(const uint64_t* keys, const int64_t* amounts, int64_t n, uint64_t* out_keys,
                  int64_t* out_pre, int64_t* m);
/* rank(k) = number of index keys below k (CsrBase::rank, sparse_engine.hpp:79-88);
 * point: out[i] = rank when keys[i] is present, -rank-1 when absent. */
void bwo_csr_point(const uint64_t* ukeys, int64_t m, const uint64_t* q, int64_t n, int64_t* out);
/* CsrBase::range (sparse_engine.hpp:89-97): out[2i] = rank(hi)-rank(lo), out[2i+1] =
 * pre[rank(hi)-1] - pre[rank(lo)-1] (0 when the ranks are equal). */
void bwo_csr_range(const uint64_t* ukeys, const int64_t* pre, int64_t m, const uint64_t* bounds,
                   int64_t n, int64_t* out);

#ifdef __cplusplus
}
#endif
#endif
