// ref_csr.cpp -- test harness (oracle side, never shipped): answers rank and range
// lookups with the reference's own CsrBase::rank / CsrBase::range
// (sparse_engine.hpp:79-97), compiled from the reference's header, to pin the
// oracle's and the GPU index's lookup semantics.
//
// The CsrBase of one group is filled with the steps of build_csr_base
// (sparse_engine.hpp:287-360): class bitmap, cumulative popcount LUT, support
// amounts accumulated at their rank, cumulative prefix.
//
// stdin:  u32 C, u64 n_rows, u64 n_q, n_rows x {u32 class, i64 amount},
//         n_q x {i64 i, i64 j}
// stdout: n_q x {i32 rank(i), i32 rank(j), i64 range(i, j)}
#include <cstdint>
#include <cstdio>
#include <vector>

#include "sparse_engine.hpp"

template <typename T>
static bool rd(T* p, size_t n) { return std::fread(p, sizeof(T), n, stdin) == n; }

int main() {
  uint32_t C = 0;
  uint64_t nr = 0, nq = 0;
  if (!rd(&C, 1) || !rd(&nr, 1) || !rd(&nq, 1)) return 2;
  std::vector<uint32_t> cls(nr);
  std::vector<int64_t> amt(nr);
  for (uint64_t i = 0; i < nr; ++i)
    if (!rd(&cls[i], 1) || !rd(&amt[i], 1)) return 2;
  std::vector<int64_t> qi(nq), qj(nq);
  for (uint64_t i = 0; i < nq; ++i)
    if (!rd(&qi[i], 1) || !rd(&qj[i], 1)) return 2;

  bwh::CsrBase csr;
  const int32_t wpr = int32_t((int64_t(C) + 63) >> 6);
  csr.wpr = wpr;
  csr.ptr.assign(2, 0);
  std::vector<uint64_t> bits(size_t(wpr), 0);
  for (uint64_t i = 0; i < nr; ++i) bits[cls[i] >> 6] |= uint64_t(1) << (cls[i] & 63);
  csr.rlut.assign(size_t(wpr) + 1, 0);
  uint32_t local = 0;
  for (int32_t b = 0; b < wpr; ++b) {
    local += uint32_t(__builtin_popcountll(bits[size_t(b)]));
    csr.rlut[size_t(b) + 1] = local;
  }
  csr.ptr[1] = local;
  csr.nnz = local;
  csr.bits = bits;
  std::vector<int64_t> sup(local, 0);
  for (uint64_t i = 0; i < nr; ++i) {
    const int32_t r = csr.rank(0, int64_t(cls[i]));
    sup[size_t(r)] = int64_t(uint64_t(sup[size_t(r)]) + uint64_t(amt[i]));
  }
  csr.pre.assign(local, 0);
  uint64_t run = 0;
  for (uint32_t k = 0; k < local; ++k) {
    run += uint64_t(sup[k]);
    csr.pre[k] = int64_t(run);
  }
  for (uint64_t q = 0; q < nq; ++q) {
    const int32_t a = csr.rank(0, qi[q]);
    const int32_t b = csr.rank(0, qj[q]);
    const int64_t s = csr.range(0, qi[q], qj[q]);
    std::fwrite(&a, 4, 1, stdout);
    std::fwrite(&b, 4, 1, stdout);
    std::fwrite(&s, 8, 1, stdout);
  }
  return 0;
}
