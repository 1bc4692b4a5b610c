// bw_host.cpp -- host front end of the GB300 executor (include/bw_host.h).
//
// Compiles a reference-native workload (BWBASE02 fixture + declared edits and
// per-state nested ranges) into the event model of bw_replay_launch: class-delta
// events grouped by state and class-interval queries in the reference's answer
// order.  One preorder pass over the version tree with apply/undo keeps each
// row's current image, each group's factor and each group's per-class alive mass,
// so factor edits expand to exactly the deltas the reference's executor adds.
#include "bw_host.h"

#include <dlfcn.h>
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <unordered_map>
#include <vector>

struct BwFixture {
  std::vector<uint8_t> copy;
  void* map = nullptr;
  size_t len = 0;
  const uint8_t* base = nullptr;
  int64_t n = 0;
  int32_t G = 0;
  int64_t t_min = 0, t_max = 0;

  int64_t ld64(size_t off) const { int64_t x; std::memcpy(&x, base + off, 8); return x; }
  int32_t ld32(size_t off) const { int32_t x; std::memcpy(&x, base + off, 4); return x; }
  int64_t row_t(int64_t i) const { return ld64(64 + 24 * (size_t)i); }
  int64_t row_amt(int64_t i) const { return ld64(64 + 24 * (size_t)i + 8); }
  int32_t row_g(int64_t i) const { return ld32(64 + 24 * (size_t)i + 16); }
  int64_t factor(int32_t g) const { return ld64(64 + 24 * (size_t)n + 8 * (size_t)g); }
  ~BwFixture() { if (map) ::munmap(map, len); }
};

namespace {

// Header checks of common.hpp:125-132 and 152-153.
int parse_fixture(BwFixture* f) {
  if (f->len < 64 || std::memcmp(f->base, "BWBASE02", 8) != 0) return 3;
  f->n = f->ld64(8);
  f->G = f->ld32(16);
  if (f->n <= 0 || f->G <= 0 || f->n > ((int64_t)1 << 40) || f->G > (1 << 20)) return 3;
  const size_t need = 64 + 24 * (size_t)f->n + 12 * (size_t)f->G;
  if (need > f->len) return 3;
  f->t_min = f->ld64(40);
  f->t_max = f->ld64(48);
  for (int32_t g = 0; g < f->G; ++g)
    if (f->factor(g) <= 0) return 3;
  return 0;
}

// SplitMix64 generator with the reference's seeding and draws (common.hpp:40-54):
// identical numbers are required to reproduce the declared workload.
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed ? seed : 0x9E3779B97F4A7C15ULL) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  uint32_t bounded(uint32_t n) { return n ? (uint32_t)(next() % n) : 0u; }
  int64_t range(int64_t lo, int64_t hi) { return hi <= lo ? lo : lo + (int64_t)(next() % (uint64_t)(hi - lo)); }
  // Counter property (batch_engine_v7c.hpp:244-249): the k-th draw (0-based) of a
  // generator started at state s0 is mix(s0 + (k + 1) * gamma), independent of the
  // draws before it.
  static uint64_t at(uint64_t s0, uint64_t k) {
    uint64_t z = s0 + (k + 1) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
};

enum : uint8_t { OP_REPLACE = 0, OP_INSERT = 1, OP_DELETE = 2, OP_MOVE = 3, OP_FACTOR = 4 };

struct Edit {
  uint8_t op = 0;
  int32_t g = 0;
  int64_t id = 0, val = 0, t = 0;
};

struct Declared {
  std::vector<int32_t> parent;
  std::vector<Edit> edit;
  std::vector<int64_t> qlo, qhi;  // per state (v*q+k) or shared (k)
  std::vector<int64_t> ins_t;
  std::vector<int32_t> ins_g;
  std::vector<int64_t> endpoints;
  std::vector<uint32_t> clo, chi;  // endpoint classes of qlo / qhi (class_of of each bound)
};

int32_t version_parent(int32_t topology, int32_t v) {
  if (v <= 0) return -1;
  return topology == 0 ? v - 1 : topology == 1 ? (v - 1) / 2 : 0;
}

// Nested ranges of one state (common.hpp:229-246), first q levels.
void nested(Rng& r, int64_t tmin, int64_t tmax, int32_t q, int64_t* lo_out, int64_t* hi_out) {
  int64_t lo = tmin, hi = tmax + 1;
  const int64_t span0 = hi - lo;
  for (int32_t k = 0; k < q; ++k) {
    int64_t span = hi - lo;
    if (span <= 4096) {
      lo = tmin + span0 / 2;
      hi = lo + 2048;
      span = hi - lo;
    }
    const int64_t a = span * (int64_t)(3 + r.bounded(16)) / 100;
    const int64_t b = span * (int64_t)(3 + r.bounded(16)) / 100;
    lo += a;
    hi -= b;
    if (hi - lo < 1024) hi = lo + 1024;
    lo_out[k] = lo;
    hi_out[k] = hi;
  }
}

// Declared workload of common.hpp:279-374 for a runtime state count.
void declare(const BwFixture& f, const BwNativeSpec& sp, Declared& w) {
  const int32_t S = sp.n_states, q = sp.q, G = f.G;
  const int64_t N = f.n, tmin = f.t_min, tmax = f.t_max;
  const uint64_t seed = (uint64_t)(int64_t)sp.seed, topo = (uint64_t)(int64_t)sp.topology,
                 fp = (uint64_t)(int64_t)sp.factor_period;
  if (sp.per_state) {
    w.qlo.assign((size_t)S * q, 0);
    w.qhi.assign((size_t)S * q, 0);
    // every state's ranges come from their own seed: independent, drawn in parallel
#pragma omp parallel for schedule(static)
    for (int32_t v = 1; v < S; ++v) {
      Rng r(seed * 1000000007ULL + topo * 65537ULL + fp * 131ULL + (uint64_t)v * 2654435761ULL + 17ULL);
      nested(r, tmin, tmax, q, &w.qlo[(size_t)v * q], &w.qhi[(size_t)v * q]);
    }
  } else {
    w.qlo.assign(q, 0);
    w.qhi.assign(q, 0);
    Rng r(seed * 1000000007ULL + topo * 65537ULL + fp * 131ULL + 17ULL);
    nested(r, tmin, tmax, q, w.qlo.data(), w.qhi.data());
  }
  Rng rng(seed * 1000003ULL + topo * 7919ULL + fp * 104729ULL + 20261025ULL);
  w.parent.resize(S);
  for (int32_t v = 0; v < S; ++v) w.parent[v] = version_parent(sp.topology, v);
  w.edit.assign(S, Edit{});
  // The edit stream in two phases, bit-identical to drawing it sequentially (the
  // reference's v7c split, batch_engine_v7c.hpp:332-408): a cheap sequential pass
  // decides every state's op, its insert slot and the index of its first draw; the
  // edits are then materialised in parallel from the counter property.
  const uint64_t s0 = rng.s;
  std::vector<uint32_t> draw0((size_t)S, 0), ins_slot((size_t)S, 0);
  std::vector<int64_t> gfactor(G, 1000);
  int32_t next_group = 0, n_ins = 0;
  uint64_t k = 0;
  for (int32_t v = 1; v < S; ++v) {
    Edit& e = w.edit[v];
    const bool factor_step = sp.factor_pct >= 0 ? (uint32_t)(Rng::at(s0, k++) % 100u) < (uint32_t)sp.factor_pct
                                                : (sp.factor_period > 0 && v % sp.factor_period == 0);
    if (factor_step) {
      const int32_t g = next_group++ % G;
      const int64_t cur = gfactor[g];
      const int64_t nf = cur == 950 ? 1000 : (cur == 1000 ? 1050 : 950);
      gfactor[g] = nf;
      e.op = OP_FACTOR; e.g = g; e.val = nf;
      continue;
    }
    const uint32_t roll = (uint32_t)(Rng::at(s0, k++) % 100u);
    draw0[v] = (uint32_t)k;
    if (roll < 55) { e.op = OP_REPLACE; k += 2; }
    else if (roll < 75) { e.op = OP_INSERT; ins_slot[v] = (uint32_t)n_ins++; k += 4; }
    else if (roll < 90) { e.op = OP_DELETE; k += 1; }
    else { e.op = OP_MOVE; k += 4; }
  }
  w.ins_t.assign((size_t)n_ins, 0);
  w.ins_g.assign((size_t)n_ins, 0);
  auto range_at = [&](uint64_t kk, int64_t lo, int64_t hi) {
    return hi <= lo ? lo : lo + (int64_t)(Rng::at(s0, kk) % (uint64_t)(hi - lo));
  };
  auto bounded_at = [&](uint64_t kk, uint32_t n) { return n ? (uint32_t)(Rng::at(s0, kk) % n) : 0u; };
#pragma omp parallel for schedule(static)
  for (int32_t v = 1; v < S; ++v) {
    Edit& e = w.edit[v];
    if (e.op == OP_FACTOR) continue;
    uint64_t kk = draw0[v];
    switch (e.op) {
      case OP_REPLACE:
        e.id = range_at(kk++, 0, N);
        e.val = f.row_amt(e.id) + range_at(kk++, -100000, 100000);
        break;
      case OP_INSERT: {
        e.id = N + (int64_t)ins_slot[v];
        e.t = range_at(kk++, tmin, tmax + 1);
        e.g = (int32_t)bounded_at(kk++, (uint32_t)G);
        const int64_t base_amt = f.row_amt(bounded_at(kk++, (uint32_t)N));
        e.val = base_amt + range_at(kk++, -100000, 100000);
        w.ins_t[ins_slot[v]] = e.t;
        w.ins_g[ins_slot[v]] = e.g;
        break;
      }
      case OP_DELETE:
        e.id = range_at(kk++, 0, N);
        break;
      default:   // move
        e.id = range_at(kk++, 0, N);
        e.t = range_at(kk++, tmin, tmax + 1);
        e.g = (int32_t)bounded_at(kk++, (uint32_t)G);
        e.val = f.row_amt(e.id) + range_at(kk++, -100000, 100000);
        break;
    }
  }
}

// Per-group support: every class a row of the group can occupy (base rows of the
// group, inserted/moved rows landing in it); holds the group's alive mass per class.
struct GroupMass {
  std::vector<int32_t> cls;
  std::vector<uint64_t> mass;
  size_t index(int32_t c) const {
    return (size_t)(std::lower_bound(cls.begin(), cls.end(), c) - cls.begin());
  }
};

struct RowImage {
  uint8_t ex;
  int32_t g, c;
  int64_t amt;
  int32_t si = 0;   // index of class c in group g's support (the compact builder keeps it)
};

}  // namespace

extern "C" int bw_fixture_open(const char* path, BwFixture** out) {
  if (!path || !out) return 2;
  const int fd = ::open(path, O_RDONLY);
  if (fd < 0) return 3;
  struct stat st {};
  if (::fstat(fd, &st) != 0 || st.st_size < 64) { ::close(fd); return 3; }
  void* m = ::mmap(nullptr, (size_t)st.st_size, PROT_READ, MAP_PRIVATE, fd, 0);
  ::close(fd);
  if (m == MAP_FAILED) return 3;
  BwFixture* f = new (std::nothrow) BwFixture();
  if (!f) { ::munmap(m, (size_t)st.st_size); return 3; }
  f->map = m;
  f->len = (size_t)st.st_size;
  f->base = static_cast<const uint8_t*>(m);
  const int rc = parse_fixture(f);
  if (rc) { delete f; return rc; }
  *out = f;
  return 0;
}

extern "C" int bw_fixture_from_memory(const void* image, size_t len, BwFixture** out) {
  if (!image || !out) return 2;
  BwFixture* f = new (std::nothrow) BwFixture();
  if (!f) return 3;
  f->copy.assign(static_cast<const uint8_t*>(image), static_cast<const uint8_t*>(image) + len);
  f->len = len;
  f->base = f->copy.data();
  const int rc = parse_fixture(f);
  if (rc) { delete f; return rc; }
  *out = f;
  return 0;
}

extern "C" void bw_fixture_close(BwFixture* f) { delete f; }
extern "C" int64_t bw_fixture_rows(const BwFixture* f) { return f ? f->n : 0; }

namespace {

// Edits must name existing rows and groups, parents must precede their children
// (the reference aborts on the same conditions, oracle.cpp:268-275, 325-328).
int validate(const BwFixture& f, const Declared& w, int32_t S) {
  const int64_t M = f.n + (int64_t)w.ins_t.size();
  if ((int32_t)w.parent.size() != S || w.parent[0] != -1) return 2;
  for (int32_t v = 1; v < S; ++v) {
    if (w.parent[v] < 0 || w.parent[v] >= v) return 2;
    const Edit& e = w.edit[v];
    if (e.op > OP_FACTOR) return 2;
    if (e.op == OP_FACTOR || e.op == OP_INSERT || e.op == OP_MOVE)
      if (e.g < 0 || e.g >= f.G) return 2;
    if (e.op != OP_FACTOR && (e.id < 0 || e.id >= M)) return 2;
  }
  for (int32_t g : w.ins_g)
    if (g < 0 || g >= f.G) return 2;
  return 0;
}

// Sorted distinct declared bounds (batch_engine_v7.hpp:362-442 dedupe) and the
// endpoint class of every declared bound.  The bounds are sorted with their
// positions by an LSD radix sort over 11-bit digits (passes whose digit is the same
// in every key are skipped); a bound's class, the number of distinct bounds at or
// below it, is then its rank among the distinct values + 1, so no per-query binary
// search is needed.
void collect_endpoints(Declared& w, int32_t S, int32_t q, bool per_state) {
  const size_t nq = per_state ? (size_t)S * q : (size_t)q;
  const size_t lo_q = per_state ? (size_t)q : 0;   // first used slot (state 0 holds none)
  const size_t n = 2 * (nq - lo_q);
  std::vector<uint64_t> key(n), key2(n);
  std::vector<uint32_t> pos(n), pos2(n);
  for (size_t i = lo_q, j = 0; i < nq; ++i, j += 2) {
    key[j] = (uint64_t)w.qlo[i] ^ (1ull << 63);   // order-preserving for int64
    key[j + 1] = (uint64_t)w.qhi[i] ^ (1ull << 63);
    pos[j] = (uint32_t)(2 * i);
    pos[j + 1] = (uint32_t)(2 * i + 1);
  }
  uint64_t all_or = 0, all_and = ~0ull;
  for (uint64_t k : key) {
    all_or |= k;
    all_and &= k;
  }
  // each pass: per-part digit histograms, their exclusive scan in (digit, part)
  // order, then a stable scatter of every part from its own offsets (parts are
  // contiguous key ranges, so the order within a digit is preserved)
  constexpr int kBits = 11, kDigits = 1 << kBits;
  const int parts = n < (1u << 16) ? 1 : 16;
  std::vector<uint32_t> cnt((size_t)parts * kDigits);
  for (int sh = 0; sh < 64; sh += kBits) {
    const uint64_t m = kDigits - 1;
    if ((((all_or ^ all_and) >> sh) & m) == 0) continue;   // constant digit
    std::fill(cnt.begin(), cnt.end(), 0u);
#pragma omp parallel for schedule(static) num_threads(parts)
    for (int t = 0; t < parts; ++t) {
      uint32_t* c = &cnt[(size_t)t * kDigits];
      for (size_t i = n * t / parts; i < n * (t + 1) / parts; ++i) ++c[(key[i] >> sh) & m];
    }
    uint32_t run = 0;
    for (int d = 0; d < kDigits; ++d)
      for (int t = 0; t < parts; ++t) {
        uint32_t& c = cnt[(size_t)t * kDigits + d];
        const uint32_t x = c;
        c = run;
        run += x;
      }
#pragma omp parallel for schedule(static) num_threads(parts)
    for (int t = 0; t < parts; ++t) {
      uint32_t* c = &cnt[(size_t)t * kDigits];
      for (size_t i = n * t / parts; i < n * (t + 1) / parts; ++i) {
        const uint32_t d = c[(key[i] >> sh) & m]++;
        key2[d] = key[i];
        pos2[d] = pos[i];
      }
    }
    key.swap(key2);
    pos.swap(pos2);
  }
  w.endpoints.clear();
  w.clo.assign(nq, 0);
  w.chi.assign(nq, 0);
  for (size_t i = 0; i < n; ++i) {
    if (i == 0 || key[i] != key[i - 1]) w.endpoints.push_back((int64_t)(key[i] ^ (1ull << 63)));
    const uint32_t cls = (uint32_t)w.endpoints.size();   // rank among the distinct bounds + 1
    (pos[i] & 1 ? w.chi : w.clo)[pos[i] >> 1] = cls;
  }
}

// Copy of a caller's explicit workload into the builder's form.
int from_declared(const BwFixture& f, const BwDeclared* d, Declared& w) {
  if (!d || d->n_states < 2 || d->q < 1 || !d->parent || !d->op || !d->g || !d->id || !d->val || !d->t ||
      !d->qlo || !d->qhi || d->n_inserted < 0 || (d->n_inserted && (!d->ins_t || !d->ins_g)))
    return 2;
  const int32_t S = d->n_states, q = d->q;
  w.parent.assign(d->parent, d->parent + S);
  w.edit.assign(S, Edit{});
  for (int32_t v = 1; v < S; ++v) {
    Edit& e = w.edit[v];
    e.op = d->op[v]; e.g = d->g[v]; e.id = d->id[v]; e.val = d->val[v]; e.t = d->t[v];
  }
  const size_t nq = d->per_state ? (size_t)S * q : (size_t)q;
  w.qlo.assign(d->qlo, d->qlo + nq);
  w.qhi.assign(d->qhi, d->qhi + nq);
  w.ins_t.assign(d->ins_t, d->ins_t + d->n_inserted);
  w.ins_g.assign(d->ins_g, d->ins_g + d->n_inserted);
  collect_endpoints(w, S, q, d->per_state != 0);
  return validate(f, w, S);
}

// The event model of a declared workload (see the file comment).
int build_events(const BwFixture& f, const Declared& w, int32_t S, int32_t q, bool per_state,
                 BwNativeWorkload** out) {
  const int32_t G = f.G;
  const int64_t N = f.n, M = N + (int64_t)w.ins_t.size();
  const std::vector<int64_t>& ep = w.endpoints;
  auto class_of = [&](int64_t t) {
    return (int32_t)(std::upper_bound(ep.begin(), ep.end(), t) - ep.begin());
  };

  // row images and group supports
  // endpoint classes of every row and edit time, found in parallel up front (the
  // binary searches over the endpoint array are the walk's main cost otherwise)
  std::vector<int32_t> ecls((size_t)S, 0);
  std::vector<RowImage> row((size_t)M);
#pragma omp parallel for schedule(static)
  for (int32_t v = 1; v < S; ++v)
    if (w.edit[v].op == OP_INSERT || w.edit[v].op == OP_MOVE) ecls[v] = class_of(w.edit[v].t);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i) row[i] = {1, f.row_g(i), class_of(f.row_t(i)), f.row_amt(i)};
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)w.ins_t.size(); ++k) row[N + k] = {0, w.ins_g[k], class_of(w.ins_t[k]), 0};
  std::vector<std::vector<int32_t>> sup(G);
  for (int64_t i = 0; i < N; ++i) {
    if (row[i].g < 0 || row[i].g >= G) return 3;
    sup[row[i].g].push_back(row[i].c);
  }
  for (int32_t v = 1; v < S; ++v) {
    const Edit& e = w.edit[v];
    if (e.op == OP_INSERT || e.op == OP_MOVE) sup[e.g].push_back(ecls[v]);
  }
  std::vector<GroupMass> gm(G);
#pragma omp parallel for schedule(dynamic)
  for (int32_t g = 0; g < G; ++g) {
    std::sort(sup[g].begin(), sup[g].end());
    sup[g].erase(std::unique(sup[g].begin(), sup[g].end()), sup[g].end());
    gm[g].cls.swap(sup[g]);
    gm[g].mass.assign(gm[g].cls.size(), 0);
  }
  std::vector<int64_t> fac(G);
  for (int32_t g = 0; g < G; ++g) fac[g] = f.factor(g);

  // upper bound of the event count: base rows, two per row edit, the group support
  // of every factor edit
  size_t cap = (size_t)N;
  for (int32_t v = 1; v < S; ++v) cap += w.edit[v].op == OP_FACTOR ? gm[w.edit[v].g].cls.size() : 2;
  bool chain = true;
  for (int32_t v = 1; v < S && chain; ++v) chain = w.parent[v] == v - 1;
  // a chain's preorder is state order: its events go straight to the output
  BwEvent* evbuf = new (std::nothrow) BwEvent[cap ? cap : 1];
  if (!evbuf) return 3;
  struct EvSink {
    BwEvent* p;
    size_t n;
    void push_back(const BwEvent& e) { p[n++] = e; }
    size_t size() const { return n; }
  } ev{evbuf, 0};
  int64_t n_factor = 0;
  // state 0: the base relation weighted by the fixture factors
  for (int64_t i = 0; i < N; ++i) {
    const RowImage& r = row[i];
    GroupMass& m = gm[r.g];
    m.mass[m.index(r.c)] += (uint64_t)r.amt;
    const uint64_t d = (uint64_t)r.amt * (uint64_t)fac[r.g];
    if (d) ev.push_back({0u, (uint32_t)r.c, (int64_t)d});
  }

  // preorder apply/undo over the version tree, children ascending
  std::vector<int32_t> cnt((size_t)S + 1, 0);
  for (int32_t v = 1; v < S; ++v) {
    const int32_t p = w.parent[v];
    if (p < 0 || p >= v) return 2;
    ++cnt[p + 1];
  }
  for (int32_t v = 0; v < S; ++v) cnt[v + 1] += cnt[v];
  std::vector<int32_t> kids((size_t)S), cur(cnt.begin(), cnt.end() - 1);
  for (int32_t v = 1; v < S; ++v) kids[cur[w.parent[v]]++] = v;
  std::vector<RowImage> undo_row((size_t)S);
  std::vector<int64_t> undo_fac((size_t)S);
  std::vector<std::pair<int32_t, int32_t>> st;
  st.reserve((size_t)S);
  st.push_back({0, cnt[0]});
  auto add_mass = [&](const RowImage& r, uint64_t sign_amt) {
    GroupMass& m = gm[r.g];
    m.mass[m.index(r.c)] += sign_amt;
  };
  while (!st.empty()) {
    auto& top = st.back();
    const int32_t v = top.first;
    if (top.second < cnt[v + 1]) {
      const int32_t c = kids[top.second++];
      const Edit& e = w.edit[c];
      if (e.op == OP_FACTOR) {
        const uint64_t ds = (uint64_t)e.val - (uint64_t)fac[e.g];
        const GroupMass& m = gm[e.g];
        if (ds)
          for (size_t i = 0; i < m.cls.size(); ++i) {
            const uint64_t d = ds * m.mass[i];
            if (d) { ev.push_back({(uint32_t)c, (uint32_t)m.cls[i], (int64_t)d}); ++n_factor; }
          }
        undo_fac[c] = fac[e.g];
        fac[e.g] = e.val;
      } else {
        RowImage& r = row[(size_t)e.id];
        const RowImage old = r;
        RowImage nw = old;
        switch (e.op) {
          case OP_REPLACE: nw.ex = 1; nw.amt = e.val; break;
          case OP_DELETE: nw.ex = 0; break;
          default: nw.ex = 1; nw.g = e.g; nw.c = ecls[c]; nw.amt = e.val; break;  // insert, move
        }
        if (old.ex && old.amt != 0)
          ev.push_back({(uint32_t)c, (uint32_t)old.c,
                        (int64_t)((uint64_t)0 - (uint64_t)fac[old.g] * (uint64_t)old.amt)});
        if (nw.ex && nw.amt != 0)
          ev.push_back({(uint32_t)c, (uint32_t)nw.c, (int64_t)((uint64_t)fac[nw.g] * (uint64_t)nw.amt)});
        if (old.ex) add_mass(old, (uint64_t)0 - (uint64_t)old.amt);
        if (nw.ex) add_mass(nw, (uint64_t)nw.amt);
        undo_row[c] = old;
        r = nw;
      }
      st.push_back({c, cnt[c]});
    } else {
      if (v > 0) {
        const Edit& e = w.edit[v];
        if (e.op == OP_FACTOR) {
          fac[e.g] = undo_fac[v];
        } else {
          RowImage& r = row[(size_t)e.id];
          if (r.ex) add_mass(r, (uint64_t)0 - (uint64_t)r.amt);
          r = undo_row[v];
          if (r.ex) add_mass(r, (uint64_t)r.amt);
        }
      }
      st.pop_back();
    }
  }

  // group events by state (stable counting sort; a chain's are already in order)
  BwNativeWorkload* o = new (std::nothrow) BwNativeWorkload();
  if (!o) {
    delete[] evbuf;
    return 3;
  }
  o->n_states = S;
  o->n_keys = (uint32_t)ep.size() + 1u;
  o->n_events = (int64_t)ev.size();
  o->n_queries = (int64_t)(S - 1) * q;
  o->n_factor_events = n_factor;
  o->parent = new int32_t[S];
  std::memcpy(o->parent, w.parent.data(), sizeof(int32_t) * S);
  if (chain) {
    o->events = evbuf;
  } else {
    o->events = new BwEvent[ev.size() ? ev.size() : 1];
    std::vector<int64_t> off((size_t)S + 1, 0);
    for (size_t i = 0; i < ev.size(); ++i) ++off[evbuf[i].state + 1];
    for (int32_t v = 0; v < S; ++v) off[v + 1] += off[v];
    for (size_t i = 0; i < ev.size(); ++i) o->events[off[evbuf[i].state]++] = evbuf[i];
    delete[] evbuf;
  }
  o->queries = new BwQuery[o->n_queries ? o->n_queries : 1];
  for (int32_t v = 1; v < S; ++v)
    for (int32_t k = 0; k < q; ++k) {
      const size_t qi = per_state ? (size_t)v * q + k : (size_t)k;
      o->queries[(size_t)(v - 1) * q + k] = {(uint32_t)v, w.clo[qi], w.chi[qi]};
    }
  *out = o;
  return 0;
}

}  // namespace

namespace {
// The compact form of a chain's event model (see bw_native_build_compact): the same
// sequential walk as build_events, with the factor expansion left to the device.
int build_compact(const BwFixture& f, const Declared& w, int32_t S, int32_t q, bool per_state,
                  BwNativeCompact** out) {
  for (int32_t v = 1; v < S; ++v)
    if (w.parent[v] != v - 1) return 2;
  const int32_t G = f.G;
  const int64_t N = f.n, M = N + (int64_t)w.ins_t.size();
  const std::vector<int64_t>& ep = w.endpoints;
  auto class_of = [&](int64_t t) {
    return (int32_t)(std::upper_bound(ep.begin(), ep.end(), t) - ep.begin());
  };
  // endpoint classes of every row and edit time, found in parallel up front (the
  // binary searches over the endpoint array are the walk's main cost otherwise)
  std::vector<int32_t> ecls((size_t)S, 0);
  std::vector<RowImage> row((size_t)M);
#pragma omp parallel for schedule(static)
  for (int32_t v = 1; v < S; ++v)
    if (w.edit[v].op == OP_INSERT || w.edit[v].op == OP_MOVE) ecls[v] = class_of(w.edit[v].t);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i) row[i] = {1, f.row_g(i), class_of(f.row_t(i)), f.row_amt(i)};
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)w.ins_t.size(); ++k) row[N + k] = {0, w.ins_g[k], class_of(w.ins_t[k]), 0};
  std::vector<std::vector<int32_t>> sup(G);
  for (int64_t i = 0; i < N; ++i) {
    if (row[i].g < 0 || row[i].g >= G) return 3;
    sup[row[i].g].push_back(row[i].c);
  }
  for (int32_t v = 1; v < S; ++v) {
    const Edit& e = w.edit[v];
    if (e.op == OP_INSERT || e.op == OP_MOVE) sup[e.g].push_back(ecls[v]);
  }
  std::vector<GroupMass> gm(G);
#pragma omp parallel for schedule(dynamic)
  for (int32_t g = 0; g < G; ++g) {
    std::sort(sup[g].begin(), sup[g].end());
    sup[g].erase(std::unique(sup[g].begin(), sup[g].end()), sup[g].end());
    gm[g].cls.swap(sup[g]);
    gm[g].mass.assign(gm[g].cls.size(), 0);
  }
  // support positions of every row's and every insert/move edit's class, in parallel:
  // the walk below then needs no search
  std::vector<int32_t> esi((size_t)S, 0);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < M; ++i) {
    const std::vector<int32_t>& cl = gm[row[i].g].cls;
    row[i].si = (int32_t)(std::lower_bound(cl.begin(), cl.end(), row[i].c) - cl.begin());
  }
#pragma omp parallel for schedule(static)
  for (int32_t v = 1; v < S; ++v)
    if (w.edit[v].op == OP_INSERT || w.edit[v].op == OP_MOVE) {
      const std::vector<int32_t>& cl = gm[w.edit[v].g].cls;
      esi[v] = (int32_t)(std::lower_bound(cl.begin(), cl.end(), ecls[v]) - cl.begin());
    }
  std::vector<int64_t> fac(G);
  for (int32_t g = 0; g < G; ++g) fac[g] = f.factor(g);
  std::vector<BwEvent> fixed;
  std::vector<int64_t> fixed_pos;
  fixed.reserve((size_t)N + 2 * (size_t)S);
  fixed_pos.reserve((size_t)N + 2 * (size_t)S);
  int64_t pos = 0;
  for (int64_t i = 0; i < N; ++i) {   // state 0: the base rows, weighted by the fixture factors
    const RowImage& r = row[i];
    gm[r.g].mass[r.si] += (uint64_t)r.amt;
    const uint64_t d = (uint64_t)r.amt * (uint64_t)fac[r.g];
    if (d) {
      fixed.push_back({0u, (uint32_t)r.c, (int64_t)d});
      fixed_pos.push_back(pos++);
    }
  }
  // timeline records in walk (state) order with their groups; grouped afterwards
  std::vector<BwTimeline> tlf;
  std::vector<int32_t> tlg;
  tlf.reserve(2 * (size_t)S);
  tlg.reserve(2 * (size_t)S);
  auto tl_push = [&](int32_t g, const BwTimeline& x) {
    tlf.push_back(x);
    tlg.push_back(g);
  };
  for (int32_t v = 1; v < S; ++v) {
    const Edit& e = w.edit[v];
    if (e.op == OP_FACTOR) {
      const uint64_t ds = (uint64_t)e.val - (uint64_t)fac[e.g];
      if (ds && !gm[e.g].cls.empty()) {
        tl_push(e.g, {v, -1, (int64_t)ds, pos});
        pos += (int64_t)gm[e.g].cls.size();
      }
      fac[e.g] = e.val;
      continue;
    }
    RowImage& r = row[(size_t)e.id];
    const RowImage old = r;
    RowImage nw = old;
    switch (e.op) {
      case OP_REPLACE: nw.ex = 1; nw.amt = e.val; break;
      case OP_DELETE: nw.ex = 0; break;
      default: nw.ex = 1; nw.g = e.g; nw.c = ecls[v]; nw.si = esi[v]; nw.amt = e.val; break;  // insert, move
    }
    if (old.ex && old.amt != 0) {
      fixed.push_back({(uint32_t)v, (uint32_t)old.c, (int64_t)((uint64_t)0 - (uint64_t)fac[old.g] * (uint64_t)old.amt)});
      fixed_pos.push_back(pos++);
    }
    if (nw.ex && nw.amt != 0) {
      fixed.push_back({(uint32_t)v, (uint32_t)nw.c, (int64_t)((uint64_t)fac[nw.g] * (uint64_t)nw.amt)});
      fixed_pos.push_back(pos++);
    }
    if (old.ex) tl_push(old.g, {v, old.si, (int64_t)((uint64_t)0 - (uint64_t)old.amt), 0});
    if (nw.ex) tl_push(nw.g, {v, nw.si, nw.amt, 0});
    r = nw;
  }

  BwNativeCompact* o = new (std::nothrow) BwNativeCompact();
  if (!o) return 3;
  o->n_states = S;
  o->n_groups = G;
  o->n_keys = (uint32_t)ep.size() + 1u;
  o->n_events = pos;
  o->n_queries = (int64_t)(S - 1) * q;
  o->n_fixed = (int64_t)fixed.size();
  size_t nsup = 0;
  const size_t ntl = tlf.size();
  for (int32_t g = 0; g < G; ++g) nsup += gm[g].cls.size();
  o->parent = new (std::nothrow) int32_t[S];
  o->queries = new (std::nothrow) BwQuery[o->n_queries ? o->n_queries : 1];
  o->fixed = new (std::nothrow) BwEvent[fixed.size() ? fixed.size() : 1];
  o->fixed_pos = new (std::nothrow) int64_t[fixed.size() ? fixed.size() : 1];
  o->sup_off = new (std::nothrow) int64_t[G + 1];
  o->sup_cls = new (std::nothrow) uint32_t[nsup ? nsup : 1];
  o->base_mass = new (std::nothrow) int64_t[nsup ? nsup : 1];
  o->tl_off = new (std::nothrow) int64_t[G + 1];
  o->tl = new (std::nothrow) BwTimeline[ntl ? ntl : 1];
  if (!o->parent || !o->queries || !o->fixed || !o->fixed_pos || !o->sup_off || !o->sup_cls || !o->base_mass ||
      !o->tl_off || !o->tl) {
    bw_native_compact_free(o);
    return 3;
  }
  std::memcpy(o->parent, w.parent.data(), sizeof(int32_t) * S);
  std::memcpy(o->fixed, fixed.data(), fixed.size() * sizeof(BwEvent));
  std::memcpy(o->fixed_pos, fixed_pos.data(), fixed_pos.size() * 8);
  size_t a = 0;
  for (int32_t g = 0; g < G; ++g) {
    o->sup_off[g] = (int64_t)a;
    for (size_t i = 0; i < gm[g].cls.size(); ++i, ++a) {
      o->sup_cls[a] = (uint32_t)gm[g].cls[i];
      o->base_mass[a] = (int64_t)gm[g].mass[i];   // the walk leaves the state-0 masses as they are
    }
  }
  o->sup_off[G] = (int64_t)a;
  // timelines grouped by group, state order kept (stable counting sort)
  for (int32_t g = 0; g <= G; ++g) o->tl_off[g] = 0;
  for (int32_t g : tlg) ++o->tl_off[g + 1];
  for (int32_t g = 0; g < G; ++g) o->tl_off[g + 1] += o->tl_off[g];
  {
    std::vector<int64_t> at(o->tl_off, o->tl_off + G);
    for (size_t i = 0; i < ntl; ++i) o->tl[at[tlg[i]]++] = tlf[i];
  }
  for (int32_t v = 1; v < S; ++v)
    for (int32_t k = 0; k < q; ++k) {
      const size_t qi = per_state ? (size_t)v * q + k : (size_t)k;
      o->queries[(size_t)(v - 1) * q + k] = {(uint32_t)v, w.clo[qi], w.chi[qi]};
    }
  *out = o;
  return 0;
}
}  // namespace

extern "C" int bw_native_build_compact(const BwFixture* fx, const BwNativeSpec* sp, BwNativeCompact** out) {
  if (!fx || !sp || !out || sp->n_states < 2 || sp->q < 1 || sp->topology < 0 || sp->topology > 2)
    return 2;
  if (sp->topology != 0) return 2;
  Declared w;
  declare(*fx, *sp, w);
  collect_endpoints(w, sp->n_states, sp->q, sp->per_state != 0);
  const int rc = validate(*fx, w, sp->n_states);
  return rc ? rc : build_compact(*fx, w, sp->n_states, sp->q, sp->per_state != 0, out);
}

extern "C" void bw_native_compact_free(BwNativeCompact* c) {
  if (!c) return;
  delete[] c->parent;
  delete[] c->queries;
  delete[] c->fixed;
  delete[] c->fixed_pos;
  delete[] c->sup_off;
  delete[] c->sup_cls;
  delete[] c->base_mass;
  delete[] c->tl_off;
  delete[] c->tl;
  delete c;
}

extern "C" int bw_native_build(const BwFixture* fx, const BwNativeSpec* sp, BwNativeWorkload** out) {
  if (!fx || !sp || !out || sp->n_states < 2 || sp->q < 1 || sp->topology < 0 || sp->topology > 2)
    return 2;
  Declared w;
  declare(*fx, *sp, w);
  collect_endpoints(w, sp->n_states, sp->q, sp->per_state != 0);
  const int rc = validate(*fx, w, sp->n_states);
  return rc ? rc : build_events(*fx, w, sp->n_states, sp->q, sp->per_state != 0, out);
}

extern "C" int bw_native_build_declared(const BwFixture* fx, const BwDeclared* d, BwNativeWorkload** out) {
  if (!fx || !out) return 2;
  Declared w;
  const int rc = from_declared(*fx, d, w);
  return rc ? rc : build_events(*fx, w, d->n_states, d->q, d->per_state != 0, out);
}

extern "C" void bw_native_free(BwNativeWorkload* w) {
  if (!w) return;
  delete[] w->parent;
  delete[] w->events;
  delete[] w->queries;
  delete w;
}

// ------------------------------------------------------------------ BWLEV001 stream
// The reference's sequential event stream (emit_events.cpp:5-8, 21-27, 62-66): the
// header "BWLEV001" + u64 record count, then 36-byte little-endian records
//   kind u32, state u32, qidx u32, g i32, w i32, a i64, b i64
// kind 0 row delta (a = t, b = amount, g = group, w = +1 insert / -1 retract),
// kind 1 factor set (g, a = the group's new factor), kind 2 query (state v, bag
// index k, interval [a, b)).  Its consumers start from the fixture's base rows and
// answer each query from the rows live at that point of the stream: the sum over
// groups of factor x the amounts with t in [lo, hi); the answer vector is ordered
// by (state, k) without state 0 (external/dd_probe/src/main.rs:66-80, 245-262).
//
// As an event-model chain: chain state i is the stream before its i-th query
// (records after query i-1 get state i; query i sits at state i).  Keys are
// endpoint classes over the distinct query bounds (class(t) = bounds <= t), so
// t in [lo, hi) is the key range [class(lo), class(hi)).  A row delta is the event
// (class(t), w * amount * factor(g)); a factor change of group g from m to m' is one
// event (class, (m' - m) * L) per class of the group's live mass L.  Base rows are
// state-0 events.  An interval with hi <= lo answers 0.
namespace {
struct StreamRec {
  uint32_t kind, state, qidx;
  int32_t g, w;
  int64_t a, b;
};
inline StreamRec stream_rec(const uint8_t* p) {
  StreamRec r;
  std::memcpy(&r.kind, p, 4);
  std::memcpy(&r.state, p + 4, 4);
  std::memcpy(&r.qidx, p + 8, 4);
  std::memcpy(&r.g, p + 12, 4);
  std::memcpy(&r.w, p + 16, 4);
  std::memcpy(&r.a, p + 20, 8);
  std::memcpy(&r.b, p + 28, 8);
  return r;
}
}  // namespace

extern "C" int bw_stream_build(const BwFixture* fx, const void* data, size_t bytes, BwStreamWorkload** out) {
  if (!fx || !out || (!data && bytes)) return 2;
  *out = nullptr;
  const uint8_t* p = static_cast<const uint8_t*>(data);
  if (bytes < 16 || std::memcmp(p, "BWLEV001", 8) != 0) return 3;
  uint64_t n = 0;
  std::memcpy(&n, p + 8, 8);
  if (n > (bytes - 16) / 36 || 16 + 36 * n != bytes) return 3;
  const uint8_t* rec = p + 16;
  const int32_t G = fx->G;
  // pass 1: validation, query bounds, answer shape
  std::vector<int64_t> bounds;
  int64_t nq = 0;
  uint32_t max_state = 0, max_k = 0;
  for (uint64_t i = 0; i < n; ++i) {
    const StreamRec r = stream_rec(rec + 36 * i);
    if (r.kind == 2) {
      bounds.push_back(r.a);
      bounds.push_back(r.b);
      ++nq;
      max_state = std::max(max_state, r.state);
      max_k = std::max(max_k, r.qidx);
    } else if (r.kind == 0) {
      if (r.g < 0 || r.g >= G || (r.w != 1 && r.w != -1)) return 3;
    } else if (r.kind == 1) {
      if (r.g < 0 || r.g >= G) return 3;
    } else {
      return 3;
    }
  }
  if (nq >= ((int64_t)1 << 31) - 1 || max_k >= 4096) return 3;
  std::sort(bounds.begin(), bounds.end());
  bounds.erase(std::unique(bounds.begin(), bounds.end()), bounds.end());
  if (bounds.size() >= ((size_t)1 << 32) - 1) return 3;
  auto cls = [&](int64_t t) {
    return (uint32_t)(std::upper_bound(bounds.begin(), bounds.end(), t) - bounds.begin());
  };
  const int32_t q = nq ? (int32_t)max_k + 1 : 0;
  const int64_t n_answers = (int64_t)max_state * q;
  std::vector<int64_t> slot((size_t)nq, -1);
  std::vector<uint8_t> seen((size_t)n_answers, 0);

  // pass 2: events and queries in stream order (states non-decreasing)
  std::vector<BwEvent> ev;
  std::vector<BwQuery> qs;
  ev.reserve((size_t)fx->n + n);
  qs.reserve((size_t)nq);
  std::vector<int64_t> mul(G);
  for (int32_t g = 0; g < G; ++g) mul[g] = fx->factor(g);
  std::unordered_map<uint64_t, int64_t> live;     // (group, class) -> live amount
  std::vector<std::vector<uint32_t>> gcls(G);      // classes each group has touched
  auto add_live = [&](int32_t g, uint32_t c, int64_t amt) {
    const uint64_t key = ((uint64_t)(uint32_t)g << 32) | c;
    auto it = live.find(key);
    if (it == live.end()) {
      live.emplace(key, amt);
      gcls[g].push_back(c);
    } else {
      it->second = (int64_t)((uint64_t)it->second + (uint64_t)amt);
    }
  };
  auto wmul = [](int64_t x, int64_t y) { return (int64_t)((uint64_t)x * (uint64_t)y); };
  for (int64_t i = 0; i < fx->n; ++i) {
    const int32_t g = fx->row_g(i);
    if (g < 0 || g >= G) return 3;
    const uint32_t c = cls(fx->row_t(i));
    add_live(g, c, fx->row_amt(i));
    const int64_t d = wmul(fx->row_amt(i), mul[g]);
    if (d) ev.push_back(BwEvent{0u, c, d});
  }
  uint32_t state = 0;
  for (uint64_t i = 0; i < n; ++i) {
    const StreamRec r = stream_rec(rec + 36 * i);
    if (r.kind == 0) {
      const uint32_t c = cls(r.a);
      const int64_t amt = r.w > 0 ? r.b : (int64_t)(0 - (uint64_t)r.b);
      add_live(r.g, c, amt);
      const int64_t d = wmul(amt, mul[r.g]);
      if (d) ev.push_back(BwEvent{state, c, d});
    } else if (r.kind == 1) {
      const int64_t dm = (int64_t)((uint64_t)r.a - (uint64_t)mul[r.g]);
      if (dm) {
        for (uint32_t c : gcls[r.g]) {
          const int64_t L = live[((uint64_t)(uint32_t)r.g << 32) | c];
          const int64_t d = wmul(dm, L);
          if (d) ev.push_back(BwEvent{state, c, d});
        }
      }
      mul[r.g] = r.a;
    } else {
      const uint32_t lo = cls(r.a), hi = cls(r.b);
      qs.push_back(BwQuery{state, lo, hi < lo ? lo : hi});
      if (r.state > 0) {
        const int64_t s = (int64_t)(r.state - 1) * q + r.qidx;
        if (seen[(size_t)s]) return 3;   // a (state, k) answered twice
        seen[(size_t)s] = 1;
        slot[qs.size() - 1] = s;
      }
      ++state;
    }
  }
  for (uint8_t x : seen)
    if (!x) return 3;   // the answer vector would have a hole

  BwStreamWorkload* o = new (std::nothrow) BwStreamWorkload();
  if (!o) return 2;
  BwNativeWorkload& w = o->chain;
  w.n_states = (int32_t)state + 1;
  w.n_keys = (uint32_t)bounds.size() + 1;
  w.n_events = (int64_t)ev.size();
  w.n_queries = (int64_t)qs.size();
  w.n_factor_events = 0;
  w.parent = new (std::nothrow) int32_t[(size_t)w.n_states];
  w.events = new (std::nothrow) BwEvent[ev.size() ? ev.size() : 1];
  w.queries = new (std::nothrow) BwQuery[qs.size() ? qs.size() : 1];
  o->slot = new (std::nothrow) int64_t[slot.size() ? slot.size() : 1];
  if (!w.parent || !w.events || !w.queries || !o->slot) {
    bw_stream_free(o);
    return 2;
  }
  for (int32_t v = 0; v < w.n_states; ++v) w.parent[v] = v - 1;
  std::memcpy(w.events, ev.data(), ev.size() * sizeof(BwEvent));
  std::memcpy(w.queries, qs.data(), qs.size() * sizeof(BwQuery));
  std::memcpy(o->slot, slot.data(), slot.size() * 8);
  o->n_answers = n_answers;
  o->q = q;
  *out = o;
  return 0;
}

extern "C" void bw_stream_free(BwStreamWorkload* w) {
  if (!w) return;
  delete[] w->chain.parent;
  delete[] w->chain.events;
  delete[] w->chain.queries;
  delete[] w->slot;
  delete w;
}

// ------------------------------------------------------------------ digests
namespace {
// FIPS 180-4 SHA-256; round constants and initial hash derived from the cube and
// square roots of the first primes with exact integer arithmetic.
struct Sha256Consts {
  uint32_t k[64], h0[8];
  static uint64_t iroot(unsigned __int128 x, int n) {
    uint64_t lo = 0, hi = (uint64_t)1 << 40;
    while (lo < hi) {
      const uint64_t mid = lo + (hi - lo + 1) / 2;
      unsigned __int128 p = (unsigned __int128)mid * mid;
      if (n == 3) p *= mid;
      if (p <= x) lo = mid; else hi = mid - 1;
    }
    return lo;
  }
  Sha256Consts() {
    uint32_t primes[64];
    int np = 0;
    for (uint32_t c = 2; np < 64; ++c) {
      bool prime = true;
      for (int i = 0; i < np && primes[i] * primes[i] <= c; ++i)
        if (c % primes[i] == 0) { prime = false; break; }
      if (prime) primes[np++] = c;
    }
    for (int i = 0; i < 64; ++i) k[i] = (uint32_t)iroot((unsigned __int128)primes[i] << 96, 3);
    for (int i = 0; i < 8; ++i) h0[i] = (uint32_t)iroot((unsigned __int128)primes[i] << 64, 2);
  }
};
const Sha256Consts& sha_consts() {
  static const Sha256Consts c;
  return c;
}
inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }
inline uint32_t big_sigma0(uint32_t x) { return rotr(x, 2) ^ rotr(x, 13) ^ rotr(x, 22); }
inline uint32_t big_sigma1(uint32_t x) { return rotr(x, 6) ^ rotr(x, 11) ^ rotr(x, 25); }
inline uint32_t small_sigma0(uint32_t x) { return rotr(x, 7) ^ rotr(x, 18) ^ (x >> 3); }
inline uint32_t small_sigma1(uint32_t x) { return rotr(x, 17) ^ rotr(x, 19) ^ (x >> 10); }
// One FIPS 180-4 round: the working variables are renamed instead of moved (the
// callers rotate the argument order), t1 lands in d and t1 + t2 in h.
#define BW_SHA_ROUND(a, b, c, d, e, f, g, h, i)                                           \
  do {                                                                                    \
    const uint32_t t1 = h + big_sigma1(e) + (g ^ (e & (f ^ g))) + K[i] + w[(i) & 15];    \
    d += t1;                                                                              \
    h = t1 + big_sigma0(a) + ((a & b) | (c & (a | b)));                                   \
  } while (0)
// The message schedule kept as a rolling window of 16 words.
void sha_compress(uint32_t h[8], const uint8_t* p, const uint32_t* K) {
  uint32_t w[16];
  for (int i = 0; i < 16; ++i)
    w[i] = ((uint32_t)p[4 * i] << 24) | ((uint32_t)p[4 * i + 1] << 16) | ((uint32_t)p[4 * i + 2] << 8) | p[4 * i + 3];
  uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], hh = h[7];
  for (int i = 0; i < 64; i += 8) {
    if (i >= 16)
      for (int j = i; j < i + 8; ++j)
        w[j & 15] += small_sigma1(w[(j - 2) & 15]) + w[(j - 7) & 15] + small_sigma0(w[(j - 15) & 15]);
    BW_SHA_ROUND(a, b, c, d, e, f, g, hh, i + 0);
    BW_SHA_ROUND(hh, a, b, c, d, e, f, g, i + 1);
    BW_SHA_ROUND(g, hh, a, b, c, d, e, f, i + 2);
    BW_SHA_ROUND(f, g, hh, a, b, c, d, e, i + 3);
    BW_SHA_ROUND(e, f, g, hh, a, b, c, d, i + 4);
    BW_SHA_ROUND(d, e, f, g, hh, a, b, c, i + 5);
    BW_SHA_ROUND(c, d, e, f, g, hh, a, b, i + 6);
    BW_SHA_ROUND(b, c, d, e, f, g, hh, a, i + 7);
  }
  h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += hh;
}
#undef BW_SHA_ROUND
}  // namespace

// The platform's SHA-256 through OpenSSL's EVP interface, found at run time
// (dlopen, no header or link dependency), as the reference's extract phase uses
// OpenSSL's SHA256 (sha_fast.hpp:1-40); BW_SHA=sw, or no libcrypto, selects the
// portable implementation above.  Both give the same digest.
namespace {
struct Evp {
  void* (*ctx_new)() = nullptr;
  void (*ctx_free)(void*) = nullptr;
  const void* (*sha256)() = nullptr;
  int (*init)(void*, const void*, void*) = nullptr;
  int (*update)(void*, const void*, size_t) = nullptr;
  int (*final_)(void*, unsigned char*, unsigned int*) = nullptr;
  bool ok = false;
};
const Evp& evp() {
  static const Evp e = [] {
    Evp x;
    const char* mode = std::getenv("BW_SHA");
    if (mode && std::strcmp(mode, "sw") == 0) return x;
    void* h = dlopen("libcrypto.so.3", RTLD_NOW | RTLD_LOCAL);
    if (!h) h = dlopen("libcrypto.so", RTLD_NOW | RTLD_LOCAL);
    if (!h) return x;
    x.ctx_new = reinterpret_cast<void* (*)()>(dlsym(h, "EVP_MD_CTX_new"));
    x.ctx_free = reinterpret_cast<void (*)(void*)>(dlsym(h, "EVP_MD_CTX_free"));
    x.sha256 = reinterpret_cast<const void* (*)()>(dlsym(h, "EVP_sha256"));
    x.init = reinterpret_cast<int (*)(void*, const void*, void*)>(dlsym(h, "EVP_DigestInit_ex"));
    x.update = reinterpret_cast<int (*)(void*, const void*, size_t)>(dlsym(h, "EVP_DigestUpdate"));
    x.final_ = reinterpret_cast<int (*)(void*, unsigned char*, unsigned int*)>(dlsym(h, "EVP_DigestFinal_ex"));
    x.ok = x.ctx_new && x.ctx_free && x.sha256 && x.init && x.update && x.final_;
    return x;
  }();
  return e;
}
void sha_hex(const uint32_t h[8], char out_hex[65]) {
  static const char* hx = "0123456789abcdef";
  for (int i = 0; i < 8; ++i)
    for (int j = 0; j < 8; ++j) out_hex[8 * i + j] = hx[(h[i] >> (28 - 4 * j)) & 15];
  out_hex[64] = 0;
}
}  // namespace

extern "C" void bw_sha256_init(BwSha256* s) {
  std::memcpy(s->h, sha_consts().h0, sizeof(s->h));
  s->bytes = 0;
  s->fill = 0;
  s->hw = nullptr;
  const Evp& e = evp();
  if (e.ok) {
    void* ctx = e.ctx_new();
    if (ctx && e.init(ctx, e.sha256(), nullptr) == 1) s->hw = ctx;
    else if (ctx) e.ctx_free(ctx);
  }
}

extern "C" void bw_sha256_update(BwSha256* s, const void* data, size_t n) {
  if (s->hw) {
    s->bytes += n;
    if (n && evp().update(s->hw, data, n) == 1) return;
    if (!n) return;
    // the platform digest failed mid-stream: no way to resume it in software
    evp().ctx_free(s->hw);
    s->hw = nullptr;
    s->fill = 0xffffffffu;   // poisoned: final reports an all-zero digest
    return;
  }
  if (s->fill == 0xffffffffu) return;
  const uint32_t* K = sha_consts().k;
  const uint8_t* p = static_cast<const uint8_t*>(data);
  s->bytes += n;
  if (s->fill) {
    const size_t take = std::min<size_t>(n, 64 - s->fill);
    std::memcpy(s->buf + s->fill, p, take);
    s->fill += (uint32_t)take;
    p += take;
    n -= take;
    if (s->fill < 64) return;
    sha_compress(s->h, s->buf, K);
    s->fill = 0;
  }
  for (; n >= 64; p += 64, n -= 64) sha_compress(s->h, p, K);
  if (n) std::memcpy(s->buf, p, n);
  s->fill = (uint32_t)n;
}

extern "C" void bw_sha256_final(BwSha256* s, char out_hex[65]) {
  if (s->hw) {
    unsigned char md[32];
    unsigned int len = 0;
    const bool ok = evp().final_(s->hw, md, &len) == 1 && len == 32;
    evp().ctx_free(s->hw);
    s->hw = nullptr;
    uint32_t h[8] = {0};
    if (ok)
      for (int i = 0; i < 8; ++i)
        h[i] = ((uint32_t)md[4 * i] << 24) | ((uint32_t)md[4 * i + 1] << 16) | ((uint32_t)md[4 * i + 2] << 8) |
               md[4 * i + 3];
    sha_hex(h, out_hex);
    return;
  }
  if (s->fill == 0xffffffffu) {
    const uint32_t z[8] = {0};
    sha_hex(z, out_hex);
    return;
  }
  const uint32_t* K = sha_consts().k;
  uint8_t tail[128] = {0};
  const size_t rem = s->fill;
  std::memcpy(tail, s->buf, rem);
  tail[rem] = 0x80;
  const size_t tl = rem < 56 ? 64 : 128;
  const uint64_t bits = s->bytes * 8u;
  for (int i = 0; i < 8; ++i) tail[tl - 1 - i] = (uint8_t)(bits >> (8 * i));
  sha_compress(s->h, tail, K);
  if (tl == 128) sha_compress(s->h, tail + 64, K);
  sha_hex(s->h, out_hex);
}

extern "C" void bw_sha256_hex(const void* data, size_t n, char out_hex[65]) {
  BwSha256 s;
  bw_sha256_init(&s);
  bw_sha256_update(&s, data, n);
  bw_sha256_final(&s, out_hex);
}

// FNV-1a with the reference's offset basis 1469598103934665603 (common.hpp:396-400).
extern "C" uint64_t bw_fnv1a_update(uint64_t h, const void* data, size_t n) {
  const uint8_t* p = static_cast<const uint8_t*>(data);
  for (size_t i = 0; i < n; ++i) h = (h ^ p[i]) * 1099511628211ULL;
  return h;
}

extern "C" uint64_t bw_fnv1a(const void* data, size_t n) { return bw_fnv1a_update(BW_FNV1A_BASIS, data, n); }

// ------------------------------------------------------------------ v7 chain plan
// Host-side restatement of the reference's v7 setup for chains in the argument
// layout of gpu_v7_launch: row-edit previous images (batch_engine_v7.hpp:1123-1230),
// touched-class coordinates per group (1234-1308), factor plan (1311-1340), base
// leaf and base mass (1350-1415), merged support (1578-1629), equal state blocks,
// block-start factors and deviation snapshots (707-830).
namespace {
int build_v7(const BwFixture& f, const Declared& w, int32_t S, int32_t q, bool per_state, int32_t blocks,
             BwV7Plan** out) {
  for (int32_t v = 1; v < S; ++v)
    if (w.parent[v] != v - 1) return 2;   // the block path takes chains only (batch_engine_v7.hpp:708)
  const int32_t G = f.G, VS = S - 1;
  const int64_t N = f.n;
  const std::vector<int64_t>& ep = w.endpoints;
  auto class_of = [&](int64_t t) {
    return (int32_t)(std::upper_bound(ep.begin(), ep.end(), t) - ep.begin());
  };
  const int32_t ncls = (int32_t)ep.size() + 1, Cpfx = ncls + 1;
  std::vector<int64_t> s0(G);
  for (int32_t g = 0; g < G; ++g) s0[g] = f.factor(g);

  // node plans: previous image of each edited row = its last image along the chain
  std::vector<GpuV7Node> nodes((size_t)S);
  std::memset(nodes.data(), 0, sizeof(GpuV7Node) * (size_t)S);
  {
    std::vector<RowImage> img((size_t)(N + (int64_t)w.ins_t.size()));
    for (int64_t i = 0; i < N; ++i) img[i] = {1, f.row_g(i), class_of(f.row_t(i)), f.row_amt(i)};
    for (size_t k = 0; k < w.ins_t.size(); ++k) img[N + k] = {0, w.ins_g[k], class_of(w.ins_t[k]), 0};
    std::vector<int64_t> fcur = s0;
    for (int32_t v = 1; v < S; ++v) {
      const Edit& e = w.edit[v];
      GpuV7Node& p = nodes[v];
      if (e.op == OP_FACTOR) {
        p.kind = 2; p.g_old = e.g; p.fac_prev = fcur[e.g]; p.fac_val = e.val;
        fcur[e.g] = e.val;
        continue;
      }
      RowImage& r = img[(size_t)e.id];
      p.kind = 1;
      p.ex_old = r.ex; p.g_old = r.g; p.c_old = r.c; p.amt_old = r.amt;
      switch (e.op) {
        case OP_REPLACE: r.ex = 1; r.amt = e.val; break;
        case OP_DELETE: r.ex = 0; break;
        default: r.ex = 1; r.g = e.g; r.c = class_of(e.t); r.amt = e.val; break;
      }
      p.ex_new = r.ex; p.g_new = r.g; p.c_new = r.c; p.amt_new = r.amt;
    }
  }
  // touched classes per group and the row deviation coordinates
  std::vector<std::vector<int32_t>> tcoord(G);
  for (int32_t v = 1; v < S; ++v) {
    const GpuV7Node& p = nodes[v];
    if (p.kind != 1) continue;
    if (p.ex_old && p.amt_old != 0) tcoord[p.g_old].push_back(p.c_old);
    if (p.ex_new && p.amt_new != 0) tcoord[p.g_new].push_back(p.c_new);
  }
  for (auto& t : tcoord) { std::sort(t.begin(), t.end()); t.erase(std::unique(t.begin(), t.end()), t.end()); }
  auto ti_of = [&](int32_t g, int32_t c) {
    return (int32_t)(std::lower_bound(tcoord[g].begin(), tcoord[g].end(), c) - tcoord[g].begin());
  };
  for (int32_t v = 1; v < S; ++v) {
    GpuV7Node& p = nodes[v];
    if (p.kind != 1) continue;
    if (p.ex_old && p.amt_old != 0) p.ti_old = ti_of(p.g_old, p.c_old);
    if (p.ex_new && p.amt_new != 0) p.ti_new = ti_of(p.g_new, p.c_new);
  }
  // factor-edited groups -> rows
  std::vector<int32_t> g2row(G, -1);
  int32_t n_active = 0;
  {
    std::vector<uint8_t> touched(G, 0);
    for (int32_t v = 1; v < S; ++v) if (nodes[v].kind == 2) touched[nodes[v].g_old] = 1;
    for (int32_t g = 0; g < G; ++g) if (touched[g]) g2row[g] = n_active++;
  }
  // root leaf and base mass per (active group, class)
  std::vector<int64_t> vbase((size_t)Cpfx, 0);
  std::vector<std::vector<std::pair<int32_t, int64_t>>> gb(n_active);
  for (int64_t i = 0; i < N; ++i) {
    const int32_t c = class_of(f.row_t(i)), g = f.row_g(i);
    vbase[(size_t)c + 1] = (int64_t)((uint64_t)vbase[(size_t)c + 1] + (uint64_t)f.row_amt(i) * (uint64_t)s0[g]);
    if (g2row[g] >= 0) gb[g2row[g]].push_back({c, f.row_amt(i)});
  }
  // merged support: union of nonzero base classes and touched classes, class order
  std::vector<int32_t> ms_off((size_t)n_active + 1, 0);
  std::vector<int64_t> ms_cls, ms_base;
  std::vector<int32_t> ms_dev;
  for (int32_t g = 0; g < G; ++g) {
    const int32_t r = g2row[g];
    if (r < 0) continue;
    auto& lst = gb[r];
    std::sort(lst.begin(), lst.end());
    std::vector<std::pair<int32_t, int64_t>> base;  // (class, mass != 0)
    for (size_t i = 0; i < lst.size();) {
      size_t j = i;
      uint64_t m = 0;
      while (j < lst.size() && lst[j].first == lst[i].first) m += (uint64_t)lst[j++].second;
      if (m) base.push_back({lst[i].first, (int64_t)m});
      i = j;
    }
    const auto& tc = tcoord[g];
    size_t bi = 0, di = 0;
    while (bi < base.size() || di < tc.size()) {
      if (di >= tc.size() || (bi < base.size() && base[bi].first < tc[di])) {
        ms_cls.push_back(base[bi].first); ms_base.push_back(base[bi].second); ms_dev.push_back(-1); ++bi;
      } else if (bi >= base.size() || tc[di] < base[bi].first) {
        ms_cls.push_back(tc[di]); ms_base.push_back(0); ms_dev.push_back((int32_t)di); ++di;
      } else {
        ms_cls.push_back(base[bi].first); ms_base.push_back(base[bi].second); ms_dev.push_back((int32_t)di);
        ++bi; ++di;
      }
    }
    ms_off[r + 1] = (int32_t)ms_cls.size();
  }
  // blocks, block-start factors, deviation snapshots of the groups each block edits
  int32_t B = blocks > 0 ? blocks : 1;
  if (B > VS) B = VS;
  std::vector<int32_t> v0(B), v1(B), bidx((size_t)S, 0);
  for (int32_t b = 0; b < B; ++b) {
    v0[b] = 1 + (int32_t)(((int64_t)VS * b) / B);
    v1[b] = 1 + (int32_t)(((int64_t)VS * (b + 1)) / B);
    for (int32_t v = v0[b]; v < v1[b]; ++v) bidx[v] = b;
  }
  std::vector<int64_t> fac_start((size_t)B * G), need_off((size_t)B * G, -1);
  std::vector<std::vector<int32_t>> bgroups(B);
  for (int32_t v = 1; v < S; ++v) if (nodes[v].kind == 2) bgroups[bidx[v]].push_back(nodes[v].g_old);
  int64_t ndev = 0;
  for (int32_t b = 0; b < B; ++b) {
    auto& gs = bgroups[b];
    std::sort(gs.begin(), gs.end());
    gs.erase(std::unique(gs.begin(), gs.end()), gs.end());
    for (int32_t g : gs) { need_off[(size_t)b * G + g] = ndev; ndev += (int64_t)tcoord[g].size(); }
  }
  std::vector<int64_t> devbuf((size_t)(ndev ? ndev : 1), 0);
  {
    std::vector<int64_t> fcur = s0;
    std::vector<std::vector<uint64_t>> dv(G);
    for (int32_t g = 0; g < G; ++g) dv[g].assign(tcoord[g].size(), 0);
    int32_t b = 0;
    for (int32_t v = 1; v < S; ++v) {
      if (v == v0[b]) {
        for (int32_t g = 0; g < G; ++g) fac_start[(size_t)b * G + g] = fcur[g];
        for (int32_t g : bgroups[b])
          for (size_t k = 0; k < tcoord[g].size(); ++k)
            devbuf[(size_t)need_off[(size_t)b * G + g] + k] = (int64_t)dv[g][k];
      }
      const GpuV7Node& p = nodes[v];
      if (p.kind == 2) fcur[p.g_old] = p.fac_val;
      if (p.kind == 1) {
        if (p.ex_old && p.amt_old != 0) dv[p.g_old][p.ti_old] -= (uint64_t)p.amt_old;
        if (p.ex_new && p.amt_new != 0) dv[p.g_new][p.ti_new] += (uint64_t)p.amt_new;
      }
      if (b + 1 < B && v + 1 == v1[b]) ++b;
    }
  }
  std::vector<int32_t> qlb((size_t)S * q, 0), qhb((size_t)S * q, 0);
  for (int32_t v = 1; v < S; ++v)
    for (int32_t k = 0; k < q; ++k) {
      const size_t qi = per_state ? (size_t)v * q + k : (size_t)k;
      qlb[(size_t)v * q + k] = (int32_t)w.clo[qi];
      qhb[(size_t)v * q + k] = (int32_t)w.chi[qi];
    }

  BwV7Plan* o = new (std::nothrow) BwV7Plan();
  if (!o) return 3;
  auto dup = [](const auto& v) {
    using T = typename std::decay_t<decltype(v)>::value_type;
    T* p = new T[v.empty() ? 1 : v.size()];
    if (!v.empty()) std::memcpy(p, v.data(), sizeof(T) * v.size());
    return p;
  };
  o->B = B; o->G = G; o->Cpfx = Cpfx; o->ncls = ncls; o->q = q; o->n_states = S; o->n_active = n_active;
  o->nodes = dup(nodes); o->block_v0 = dup(v0); o->block_v1 = dup(v1); o->fac_start = dup(fac_start);
  o->g2row = dup(g2row); o->ms_off = dup(ms_off); o->ms_cls = dup(ms_cls); o->ms_base = dup(ms_base);
  o->ms_dev = dup(ms_dev); o->devbuf = dup(devbuf); o->n_devbuf = ndev; o->need_off = dup(need_off);
  o->qlb = dup(qlb); o->qhb = dup(qhb); o->bidx = dup(bidx); o->vbase = dup(vbase);
  *out = o;
  return 0;
}
}  // namespace

extern "C" int bw_v7_plan_build(const BwFixture* fx, const BwNativeSpec* sp, int32_t blocks, BwV7Plan** out) {
  if (!fx || !sp || !out || sp->n_states < 3 || sp->q < 1 || sp->topology != 0) return 2;
  Declared w;
  declare(*fx, *sp, w);
  collect_endpoints(w, sp->n_states, sp->q, sp->per_state != 0);
  const int rc = validate(*fx, w, sp->n_states);
  return rc ? rc : build_v7(*fx, w, sp->n_states, sp->q, sp->per_state != 0, blocks, out);
}

extern "C" int bw_v7_plan_build_declared(const BwFixture* fx, const BwDeclared* d, int32_t blocks, BwV7Plan** out) {
  if (!fx || !out || !d || d->n_states < 3) return 2;
  Declared w;
  const int rc = from_declared(*fx, d, w);
  return rc ? rc : build_v7(*fx, w, d->n_states, d->q, d->per_state != 0, blocks, out);
}

extern "C" void bw_v7_plan_free(BwV7Plan* p) {
  if (!p) return;
  delete[] p->nodes; delete[] p->block_v0; delete[] p->block_v1; delete[] p->fac_start; delete[] p->g2row;
  delete[] p->ms_off; delete[] p->ms_cls; delete[] p->ms_base; delete[] p->ms_dev; delete[] p->devbuf;
  delete[] p->need_off; delete[] p->qlb; delete[] p->qhb; delete[] p->bidx; delete[] p->vbase;
  delete p;
}
