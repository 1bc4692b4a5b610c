// ref_fuzz.cpp -- TEST INFRASTRUCTURE ONLY (built by oracle/ref.mk into oracle/_ref/).
//
// Golden vectors for the randomized branching fuzz, taken from the reference's own
// code: this harness compiles the reference's fuzz_fullpath.cpp where it lies (its
// main renamed away), draws each case's parameters the way that file's main does
// (fuzz_fullpath.cpp:362-387: 60 deterministic edge cases = 10 profiles x 3
// topologies x 2 range scopes, then seeded random profiles), builds the case with
// the reference's build_case (fuzz_fullpath.cpp:162-320: fresh tiny fixture, edits,
// declared ranges) and answers it with the reference's rollback-Fenwick arm "rf"
// (fuzz_fullpath.cpp:408-417, the fuzz's oracle).  One JSON line per case: the
// case parameters, the SHA-256 of the fixture file and of the answer vector.
//
//   oracle/_ref/fuzz_ref_33 --cases 600 --fixture /tmp/x.bin > fuzz.jsonl
#define main bw_reference_fuzz_main
#include "fuzz_fullpath.cpp"
#undef main

#include "../oracle/bw_oracle.h"

static std::string file_sha(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return "";
  std::vector<unsigned char> buf;
  unsigned char tmp[65536];
  size_t n;
  while ((n = std::fread(tmp, 1, sizeof(tmp), f)) > 0) buf.insert(buf.end(), tmp, tmp + n);
  std::fclose(f);
  char hex[65];
  bwo_sha256_hex(buf.data(), buf.size(), hex);
  return hex;
}

int main(int argc, char** argv) {
  long long ncases = 600;
  std::string fx = "/tmp/bw_ref_fuzz_fixture.bin";
  for (int i = 1; i + 1 < argc; ++i) {
    if (!std::strcmp(argv[i], "--cases")) ncases = std::atoll(argv[++i]);
    else if (!std::strcmp(argv[i], "--fixture")) fx = argv[++i];
  }
  setenv("BWH_BATCH_FORCE", "1", 1);
  for (long long ci = 0; ci < ncases; ++ci) {
    Case c;
    c.seed = u64(ci) * 0x2545F4914F6CDD1DULL + 12345;
    FRng r(c.seed ^ 0xABCDEFULL);
    i32 prof;
    if (ci < 60) {
      prof = i32(ci % 10);
      c.topology = i32((ci / 10) % 3);
      c.per_state = ((ci / 30) % 2) == 0;
      c.q = 1 + i32((ci / 6) % 3);
    } else {
      prof = r.bounded(10);
      c.topology = r.bounded(3);
      c.q = 1 + r.bounded(3);
      c.per_state = r.chance(55);
    }
    c.N = 12 + r.bounded(40);
    c.G = 2 + r.bounded(3);
    switch (prof) {
      case 0: c.p_factor = 10 + r.bounded(20); break;
      case 1: c.p_factor = 50 + r.bounded(30); break;
      case 2: c.empty_ranges = true; break;
      case 3: c.tmax1_inserts = true; c.p_factor = 20; break;
      case 4: c.neg_amounts = true; c.p_factor = 20; break;
      case 5: c.zero_factor = true; c.p_factor = 60; break;
      case 6: c.neg_factor = true; c.p_factor = 60; break;
      case 7: c.p_factor = 100; break;
      case 8: c.span = 8; c.dense = true; c.p_factor = 30; break;
      default: c.p_factor = 25; break;
    }
    c.profile = prof;
    Fixture f;
    Workload w;
    BatchWorkload bw;
    BatchWorkloadV2 bw2;
    if (!build_case(c, f, w, bw, bw2, fx)) {
      std::fprintf(stderr, "case %lld: fixture build failed\n", ci);
      return 3;
    }
    std::vector<i64> want;
    Arm* a = make_classic_arm("rf", f, w);
    if (!a) return 3;
    a->build();
    run_arm_answers(a, w, c.q, want);
    delete a;
    char hex[65];
    bwo_sha256_hex(want.data(), want.size() * sizeof(i64), hex);
    std::printf("{\"case\": %lld, \"seed\": %llu, \"profile\": %d, \"topology\": %d, \"q\": %d, "
                "\"per_state\": %s, \"N\": %d, \"G\": %d, \"p_factor\": %d, \"states\": %d, "
                "\"fixture_sha256\": \"%s\", \"n_answers\": %zu, \"answers_sha256\": \"%s\"}\n",
                ci, (unsigned long long)c.seed, c.profile, c.topology, c.q, c.per_state ? "true" : "false",
                c.N, c.G, c.p_factor, (int)kStates, file_sha(fx).c_str(), want.size(), hex);
  }
  return 0;
}
