// tc_index.cuh -- index arithmetic of the tensor-core pair-form sigma
// (sigma_tc.cu), shared by the kernel and the host-side index check.
//
// Column part: the mirrored orbitals [0, sp), sp <= 16, split into the low
// lo = min(sp, 8) orbitals and the high sp - lo ones.  A column set C with
// elements c_0 < c_1 < ... has colex rank sum_t C(c_t, t + 1); writing
// P = C n [0, lo) (p elements) and Q = C n [lo, sp),
//     colex(C) = c8[P] + G[Q][p],
//     c8[P]    = sum over P's elements of C(c_t, t + 1),
//     G[Q][p]  = sum_t C(lo + q_t, p + t + 1)   (q_t: Q's bits, ascending).
// A row of n columns holds at column c the set of colex n - 1 - c, so the
// own-row position of C u a (a not in C) is
//     a <  lo:  n_own - 1 - G[Q][p + 1] - c8[P | a]
//     a >= lo:  n_own - 1 - c8[P]       - G[Q | a][p]
// (two small shared-memory tables instead of a 16-entry insertion table per
// column).  cset[j][c] lists the column set at column c of a row with j
// column elements.
#pragma once

#include <cstdint>
#include <vector>

namespace doci {
namespace tc {

constexpr int kTablesBytes = 256 + 256 * 10 * 2;  // c8[256] (u8) + G[256][10] (u16)

__host__ __device__ __forceinline__ int gw(int lo) { return lo + 2; }

// own-row position of C u a (a in [0, sp), not in C)
__host__ __device__ __forceinline__ uint32_t own_pos(uint32_t C, int a, uint32_t n_own, int lo, const uint8_t *c8,
                                                     const uint16_t *G) {
  const uint32_t lomask = (1u << lo) - 1u, P = C & lomask, Q = C >> lo;
#ifdef __CUDA_ARCH__
  const int p = __popc(P);
#else
  const int p = __builtin_popcount(P);
#endif
  if (a < lo) return n_own - 1u - G[Q * gw(lo) + p + 1] - c8[P | (1u << a)];
  return n_own - 1u - c8[P] - G[(Q | (1u << (a - lo))) * gw(lo) + p];
}

// The 16-byte aligned global range [a0, a1) (floats) that the bulk copy of
// a hole row's tile segment covers: the row starts at rs, the tile holds the
// sets [c0, c1); the end stays inside the vector's last whole 16-byte chunk
// (elements past it are read directly).
__host__ __device__ __forceinline__ void hole_segment(uint32_t rs, uint32_t c0, uint32_t c1, uint32_t D, uint32_t *a0,
                                                      uint32_t *a1) {
  *a0 = (rs + c0) & ~3u;
  uint32_t e = (rs + c1 + 3u) & ~3u;
  const uint32_t lim = D & ~3u;
  if (e > lim) e = lim;
  if (e < *a0) e = *a0;
  *a1 = e;
}

// host: the tables for a column part of sp orbitals (binomial table B with
// row stride bc)
inline void build_tables(int sp, const uint32_t *B, int bc, std::vector<uint16_t> &cset,
                         std::vector<uint32_t> &cset_off, std::vector<uint8_t> &tables) {
  const int lo = sp < 8 ? sp : 8, hi = sp - lo;
  auto C = [&](int n, int k) -> uint32_t { return (k < 0 || n < 0 || k > n) ? 0u : B[n * bc + k]; };
  auto colex = [&](uint32_t M) {
    uint32_t r = 0;
    int e = 0;
    for (int d = 0; d < sp; ++d)
      if (M >> d & 1u) r += C(d, ++e);
    return r;
  };
  cset.assign(size_t(1) << sp, 0);
  cset_off.assign(sp + 2, 0);
  for (int j = 0; j <= sp; ++j) cset_off[j + 1] = cset_off[j] + C(sp, j);
  for (uint32_t M = 0; M < (1u << sp); ++M) {
    const int j = __builtin_popcount(M);
    cset[cset_off[j] + (C(sp, j) - 1 - colex(M))] = static_cast<uint16_t>(M);
  }
  tables.assign(kTablesBytes, 0);
  for (uint32_t P = 0; P < (1u << lo); ++P) tables[P] = static_cast<uint8_t>(colex(P));
  uint16_t *G = reinterpret_cast<uint16_t *>(tables.data() + 256);
  for (uint32_t Q = 0; Q < (1u << hi); ++Q)
    for (int p = 0; p <= lo + 1; ++p) {
      uint32_t g = 0;
      int e = 0;
      for (int b = 0; b < hi; ++b)
        if (Q >> b & 1u) g += C(lo + b, p + (++e));
      G[Q * gw(lo) + p] = static_cast<uint16_t>(g);
    }
}

// host: ranks of the rows with no column element (row part of N elements):
// one determinant each, of colex sum_t C(sp + a_t, t + 1)
inline std::vector<uint32_t> rows_without_columns(int L, int N, int sp, uint64_t D, const uint32_t *B, int bc) {
  std::vector<uint32_t> v;
  const int na = L - sp;
  if (N > na) return v;
  for (uint32_t m = 0; m < (1u << na); ++m) {
    if (__builtin_popcount(m) != N) continue;
    uint64_t base = 0;
    int t = 0;
    for (int a = 0; a < na; ++a)
      if (m >> a & 1u) base += B[(sp + a) * bc + (++t)];
    v.push_back(static_cast<uint32_t>(D - 1 - base));
  }
  return v;
}

}  // namespace tc
}  // namespace doci
