// Host-side check of the pair-form sigma's index arithmetic
// (doci_gb300/csrc/sigma_pair.cu), compiled by nvcc and run on the CPU.  The
// blocks (row parts R' of the (N-1)-pair sets) are listed by the library's
// rule and the insertion table is the library's (dev::build_cross_tables);
// the kernel's formulas are applied to them (column hole h of the set at
// column c: own row start + (ins >> 8), orbital ins & 255; row-part hole b:
// start of row R' u b + c), and every neighbour rank is recomputed here from
// first principles (lexical rank of the neighbour's bitstring).
// Every set S must visit each orbital outside S exactly once, in range, at the
// rank of S u o; over a whole space (strides 1) every determinant must be
// reached exactly N times (once per pair it holds).
//   usage: pair_check L N split [block_stride] [set_stride]
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../doci_gb300/csrc/addressing.cuh"

constexpr int BC = 35;
static uint64_t binom(unsigned n, unsigned k) {
  if (k > n) return 0;
  uint64_t r = 1;
  for (unsigned d = 1; d <= k; ++d) r = r * (n - k + d) / d;
  return r;
}
static uint64_t direct_rank_mirrored(uint32_t M, int L, int N) {  // M: mirrored set
  uint64_t s = 0;
  int e = 0;
  for (int o = 0; o < L; ++o) {  // original orbital o = mirrored L-1-o
    if (M >> (L - 1 - o) & 1u) {
      s += binom(L - 1 - o, N - e);
      ++e;
    }
  }
  return binom(L, N) - 1 - s;
}

int main(int argc, char **argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: pair_check L N split [block_stride] [set_stride]\n");
    return 2;
  }
  const int L = std::atoi(argv[1]), N = std::atoi(argv[2]), sp = std::atoi(argv[3]);
  const int bstride = argc > 4 ? std::atoi(argv[4]) : 1, sstride = argc > 5 ? std::atoi(argv[5]) : 1;
  const int na = L - sp;
  std::vector<uint32_t> B(33 * BC, 0);
  for (int n = 0; n <= 32; ++n)
    for (int k = 0; k < BC; ++k) B[n * BC + k] = static_cast<uint32_t>(binom(n, k));
  const uint64_t D = binom(L, N);
  auto row_start = [&](uint32_t R) -> uint64_t {  // rank of the row's first determinant
    const int j = N - __builtin_popcount(R);
    const uint32_t n = static_cast<uint32_t>(binom(sp, j));
    const uint32_t Cb = doci::dev::colex_unrank<BC>(n - 1, sp, j, B.data());
    return direct_rank_mirrored(Cb | (R << sp), L, N);
  };
  std::vector<uint32_t> rem, ins, off;
  if (sp <= 16) doci::dev::build_cross_tables(sp, B.data(), BC, rem, ins, off);
  const bool full = bstride == 1 && sstride == 1;
  std::vector<uint8_t> hits(full ? D : 0, 0);
  uint64_t bad = 0, sets = 0, visits = 0;
  int blk = 0;
  for (uint32_t mask = 0; mask < (1u << na); ++mask) {
    const int kp = __builtin_popcount(mask), jp = N - 1 - kp;
    if (jp < 0 || jp > sp) continue;
    if (blk++ % bstride) continue;
    const uint32_t n_s = static_cast<uint32_t>(binom(sp, jp));
    const uint32_t n_own = jp + 1 <= sp ? static_cast<uint32_t>(binom(sp, jp + 1)) : 0u;
    const uint64_t own = n_own ? row_start(mask) : ~0ull;
    // row-part holes in ascending order (the kernel's ballot compaction)
    std::vector<uint64_t> hole_rs;
    std::vector<int> hole_o;
    for (int b = 0; b < na; ++b)
      if (!((mask >> b) & 1u)) {
        hole_rs.push_back(row_start(mask | (1u << b)));
        hole_o.push_back(sp + b);
      }
    const int nch = sp - jp, nhr = na - kp;
    if (static_cast<int>(hole_rs.size()) != nhr || sp + nhr > 32) ++bad;
    for (uint32_t c = 0; c < n_s; c += static_cast<uint32_t>(sstride)) {
      // the set S at column c of a row of n_s columns: colex n_s - 1 - c
      const uint32_t Cm = doci::dev::colex_unrank<BC>(n_s - 1 - c, sp, jp, B.data());
      const uint32_t S = Cm | (mask << sp);
      uint32_t seen = 0;
      ++sets;
      auto check = [&](int o, uint64_t rank, int tile_q) {
        ++visits;
        if (o >= L || (S >> o & 1u) || (seen >> o & 1u) || tile_q < 0 || tile_q >= 32) {
          ++bad;
          return;
        }
        seen |= 1u << o;
        const uint64_t want = direct_rank_mirrored(S | (1u << o), L, N);
        if (rank != want || rank >= D) {
          if (bad < 5)
            std::printf("mismatch S=%x o=%d rank=%llu want=%llu\n", S, o, static_cast<unsigned long long>(rank),
                        static_cast<unsigned long long>(want));
          ++bad;
          return;
        }
        if (full) ++hits[rank];
      };
      for (int h = 0; h < nch; ++h) {
        const uint32_t e = ins[off[jp] + 16u * c + h];
        const uint32_t pos = e >> 8, q = e & 0xffu;
        if (pos >= n_own || q >= static_cast<uint32_t>(sp)) {
          ++bad;
          continue;
        }
        check(static_cast<int>(q), own + pos, static_cast<int>(q));
      }
      for (int h = 0; h < nhr; ++h) check(hole_o[h], hole_rs[h] + c, sp + h);
      const uint32_t outside = doci::dev::low_mask(L) & ~S;
      if (seen != outside) ++bad;
    }
  }
  if (full)
    for (uint64_t t = 0; t < D; ++t)
      if (hits[t] != (N >= 1 ? N : 0)) ++bad;
  std::printf("L=%d N=%d split=%d blocks=%d sets=%llu visits=%llu bad=%llu\n", L, N, sp, blk,
              static_cast<unsigned long long>(sets), static_cast<unsigned long long>(visits),
              static_cast<unsigned long long>(bad));
  return bad ? 1 : 0;
}
