/*
 * bw_host.h -- host-side C ABI of the GB300 executor (libbwhost.so).
 *
 * Reference-native front end: a BWBASE02 fixture (common.hpp:57-75) plus the
 * deterministic declared workload (common.hpp:279-374) compiled into the event
 * model consumed by bw_replay_launch (include/bw_gpu.h):
 *
 *  * keys are endpoint classes: class_of(t) = number of declared endpoints <= t
 *    (batch_engine_v7.hpp:559-572);
 *  * state 0 carries the base rows: (0, class_of(t), amount * base_factor(g))
 *    (batch_engine_v7.hpp:1350-1376);
 *  * a row edit at state v removes the row's previous image and adds the new one,
 *    both weighted by the group's factor at v (batch_engine_v7.hpp:884-904);
 *  * a factor edit at v on group g adds (new - old) * mass_g(v, c) at every class c
 *    of the group's merged support (batch_engine_v7.hpp:905-922, 1578-1629);
 *  * query k of state v is (v, class_of(lo), class_of(hi)) in the reference's
 *    answer order v = 1..S-1, k = 0..q-1 (oracle.cpp:17-18, batch_engine_v7.hpp:666-698).
 *
 * Also: SHA-256 / FNV-1a of answer vectors (sha_fast.hpp:27-43, common.hpp:396-400).
 * Functions return 0 on success, 2 on bad arguments, 3 on an unreadable or
 * malformed fixture (the reference worker's exit codes, panel_batch_gpu.cpp:61-80).
 */
#ifndef BW_HOST_H
#define BW_HOST_H
#include <stddef.h>
#include <stdint.h>

#include "bw_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct BwFixture BwFixture;  /* opaque, owns the mapped or copied image */

/* mmap a BWBASE02 file (common.hpp:112-155 checks: magic, n, G, size, factors > 0). */
int bw_fixture_open(const char* path, BwFixture** out);
/* Same checks on an image in memory (copied). */
int bw_fixture_from_memory(const void* image, size_t len, BwFixture** out);
void bw_fixture_close(BwFixture* f);
int64_t bw_fixture_rows(const BwFixture* f);

typedef struct {
  int32_t n_states;       /* kStates of the reference (root + edited states) */
  int32_t topology;       /* 0 chain, 1 bushy, 2 star (common.hpp:219-226) */
  int32_t seed;
  int32_t factor_period;
  int32_t q;              /* queries per state */
  int32_t per_state;      /* 1 = BWH_RANGE_SCOPE=per_state, 0 = one shared set */
  int32_t factor_pct;     /* BWH_FACTOR_PCT, or -1 for the factor-period pattern */
} BwNativeSpec;

typedef struct {          /* host arrays owned by the library */
  int32_t n_states;
  uint32_t n_keys;        /* endpoint classes (distinct endpoints + 1) */
  int64_t n_events;
  int64_t n_queries;      /* (n_states - 1) * q */
  int32_t* parent;        /* n_states */
  BwEvent* events;        /* grouped by state */
  BwQuery* queries;       /* reference answer order */
  int64_t n_factor_events;/* of n_events, expanded from factor edits */
} BwNativeWorkload;

int bw_native_build(const BwFixture* f, const BwNativeSpec* spec, BwNativeWorkload** out);
void bw_native_free(BwNativeWorkload* w);

/* The same declared workload for a chain (topology 0) in the compact form whose
 * factor expansion the device performs (bw_native_expand, include/bw_gpu.h): the
 * expanded event list equals bw_native_build's apart from extra zero-delta events
 * (classes whose mass is zero at the factor edit).  2 for a tree. */
int bw_native_build_compact(const BwFixture* f, const BwNativeSpec* spec, BwNativeCompact** out);
void bw_native_compact_free(BwNativeCompact* c);

/* An explicit declared workload: the reference's Workload (common.hpp:177-212) as a
 * caller fills it directly, e.g. the reference's randomized branching fuzz
 * (fuzz_fullpath.cpp:196-283), instead of drawing it from (topology, seed, factor
 * period).  Row ids: base rows 0..n-1, inserted rows n..n+n_inserted-1 (row n+k is
 * the k-th insert, initially absent at ins_t[k] in group ins_g[k]).  Edit v >= 1:
 * op BW_OP_*; REPLACE sets row id's amount to val (and makes it present), INSERT and
 * MOVE set its (t, g, amount) to (t, g, val), DELETE removes it, FACTOR sets group
 * g's factor to val (any int64, zero and negative included).  Endpoint classes are
 * the sorted distinct declared bounds (batch_engine_v7.hpp:559-572). */
enum { BW_OP_REPLACE = 0, BW_OP_INSERT = 1, BW_OP_DELETE = 2, BW_OP_MOVE = 3, BW_OP_FACTOR = 4 };

typedef struct {
  int32_t n_states;       /* states 0..n_states-1 (state 0 = the fixture, no edit) */
  int32_t q;              /* ranges per state */
  int32_t per_state;      /* 1: qlo/qhi hold n_states*q entries (v*q+k); 0: q shared entries */
  const int32_t* parent;  /* n_states; parent[0] = -1, 0 <= parent[v] < v */
  const uint8_t* op;      /* n_states (index 0 unused) */
  const int32_t* g;       /* n_states: group of INSERT/MOVE/FACTOR */
  const int64_t* id;      /* n_states: row of REPLACE/INSERT/DELETE/MOVE */
  const int64_t* val;     /* n_states: amount or factor */
  const int64_t* t;       /* n_states: timestamp of INSERT/MOVE */
  const int64_t* qlo;     /* declared ranges [qlo, qhi) */
  const int64_t* qhi;
  int64_t n_inserted;
  const int64_t* ins_t;   /* n_inserted */
  const int32_t* ins_g;   /* n_inserted */
} BwDeclared;

/* Same output as bw_native_build for an explicit workload (answer order v = 1..S-1,
 * k = 0..q-1).  Returns 2 for malformed edits (unknown op, row or group out of
 * range, bad parent), 3 for an unusable fixture. */
int bw_native_build_declared(const BwFixture* f, const BwDeclared* w, BwNativeWorkload** out);

/* The reference's v7 chain plan (batch_engine_v7.hpp:576-830) in the argument
 * layout of gpu_v7_launch / gpu_combine_launch, built on the host: node plans,
 * equal state blocks, block-start factor vectors, block-start deviation
 * snapshots, merged per-group supports, endpoint classes of every query, the
 * root leaf and the state -> block map.  Chains only (topology 0), as the
 * reference's block path (batch_engine_v7.hpp:708). */
typedef struct {
  int32_t B, G, Cpfx, ncls, q, n_states, n_active;
  struct GpuV7Node* nodes;   /* n_states */
  int32_t* block_v0;         /* B */
  int32_t* block_v1;         /* B */
  int64_t* fac_start;        /* B*G */
  int32_t* g2row;            /* G */
  int32_t* ms_off;           /* n_active+1 */
  int64_t* ms_cls;           /* ms_off[n_active] */
  int64_t* ms_base;
  int32_t* ms_dev;
  int64_t* devbuf;           /* n_devbuf */
  int64_t n_devbuf;
  int64_t* need_off;         /* B*G */
  int32_t* qlb;              /* n_states*q */
  int32_t* qhb;
  int32_t* bidx;             /* n_states */
  int64_t* vbase;            /* Cpfx, root leaf */
} BwV7Plan;

int bw_v7_plan_build(const BwFixture* f, const BwNativeSpec* spec, int32_t blocks, BwV7Plan** out);
/* The same plan for an explicit chain workload (parent[v] == v-1, else 2). */
int bw_v7_plan_build_declared(const BwFixture* f, const BwDeclared* w, int32_t blocks, BwV7Plan** out);
void bw_v7_plan_free(BwV7Plan* p);

/* BWLEV001 event stream ingest (emit_events.cpp:5-8, 21-27, 62-66): the reference's
 * sequential stream of row deltas, factor sets and queries (16-byte header, 36-byte
 * records) over a fixture's base rows, compiled into a linear-chain event workload:
 * chain state i is the stream before its i-th query, keys are endpoint classes over
 * the stream's distinct query bounds, a factor change expands into one event per
 * class of the group's live mass.  slot[i] is the i-th query's index in the answer
 * vector ((state - 1) * q + k; -1 for state-0 queries), n_answers its length.
 * Returns 2 on bad arguments or allocation failure, 3 on a malformed stream. */
typedef struct BwStreamWorkload {
  BwNativeWorkload chain;
  int64_t* slot;
  int64_t n_answers;
  int32_t q;
} BwStreamWorkload;
int bw_stream_build(const BwFixture* f, const void* data, size_t bytes, BwStreamWorkload** out);
void bw_stream_free(BwStreamWorkload* w);

/* Lowercase hex SHA-256 (64 chars + NUL) and the reference's FNV-1a
   (common.hpp:396-400, sha_fast/sha256.hpp), one-shot and streaming: a digest
   fed the same bytes in any split gives the one-shot value. */
void bw_sha256_hex(const void* data, size_t n, char out_hex[65]);
uint64_t bw_fnv1a(const void* data, size_t n);

typedef struct BwSha256 {
  uint32_t h[8];
  uint64_t bytes;      /* bytes fed so far */
  uint8_t buf[64];     /* pending partial block */
  uint32_t fill;
  void* hw;            /* the platform digest in use (OpenSSL EVP, found at run time), else NULL;
                          bw_sha256_final releases it.  BW_SHA=sw forces the portable code. */
} BwSha256;
void bw_sha256_init(BwSha256* s);
void bw_sha256_update(BwSha256* s, const void* data, size_t n);
void bw_sha256_final(BwSha256* s, char out_hex[65]);

#define BW_FNV1A_BASIS 1469598103934665603ULL
/* FNV-1a continued over more bytes: start from BW_FNV1A_BASIS. */
uint64_t bw_fnv1a_update(uint64_t h, const void* data, size_t n);

#ifdef __cplusplus
}
#endif
#endif
