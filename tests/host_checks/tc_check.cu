// Host-side check of the tensor-core pair-form sigma's index arithmetic
// (doci_gb300/csrc/sigma_tc.cu with tc_index.cuh), compiled by nvcc and run
// on the CPU.  The launches (row-part size kp of the sets, largest first),
// units (colex unrank of the row part), own-row positions (tc::own_pos on the
// library's tables), hole rows and bulk-copy segments (tc::hole_segment) are
// taken exactly as the kernel takes them; every neighbour rank is recomputed
// from first principles (lexical rank of the neighbour's set).  Checked:
// every index in range and equal to the direct rank; every segment 16-byte
// aligned, inside the vector and inside its shared-memory slot; over a whole
// space (strides 1) every determinant reached exactly N times (once per pair
// it holds) and its diagonal term written exactly once (own row or the
// no-column rows).
//   usage: tc_check L N split [unit_stride] [set_stride]
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../doci_gb300/csrc/addressing.cuh"
#include "../../doci_gb300/csrc/tc_index.cuh"

constexpr int BC = 35;
constexpr uint32_t kTile = 128, kSlot = 136;
static uint64_t binom(unsigned n, unsigned k) {
  if (k > n) return 0;
  uint64_t r = 1;
  for (unsigned d = 1; d <= k; ++d) r = r * (n - k + d) / d;
  return r;
}
// rank of a mirrored set M (bit d = mirrored orbital d) by the reference's order
static uint64_t direct_rank(uint32_t M, int L, int N) {
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
    std::fprintf(stderr, "usage: tc_check L N split [unit_stride] [set_stride]\n");
    return 2;
  }
  const int L = std::atoi(argv[1]), N = std::atoi(argv[2]), sp = std::atoi(argv[3]);
  const uint32_t ustride = argc > 4 ? std::atoi(argv[4]) : 1, sstride = argc > 5 ? std::atoi(argv[5]) : 1;
  const int na = L - sp, lo = sp < 8 ? sp : 8;
  std::vector<uint32_t> B(33 * BC, 0);
  for (int n = 0; n <= 32; ++n)
    for (int k = 0; k < BC; ++k) B[n * BC + k] = static_cast<uint32_t>(binom(n, k));
  const uint64_t D = binom(L, N);
  std::vector<uint16_t> cset;
  std::vector<uint32_t> coff;
  std::vector<uint8_t> tables;
  doci::tc::build_tables(sp, B.data(), BC, cset, coff, tables);
  const uint8_t *c8 = tables.data();
  const uint16_t *G = reinterpret_cast<const uint16_t *>(tables.data() + 256);
  auto row_start = [&](uint32_t R) -> int64_t {  // as ham_build_rows
    const int k = __builtin_popcount(R), j = N - k;
    if (j < 0 || j > sp) return -1;
    uint64_t base = 0;
    int t = 0;
    for (int a = 0; a < na; ++a)
      if (R >> a & 1u) base += binom(sp + a, j + t + 1), ++t;
    return static_cast<int64_t>(D - base - binom(sp, j));
  };
  const bool full = ustride == 1 && sstride == 1;
  std::vector<uint8_t> hits, diag;
  if (full) {
    hits.assign(D, 0);
    diag.assign(D, 0);
  }
  long bad = 0, checked = 0;
  auto fail = [&](const char *what, long a, long b) {
    if (bad < 10) std::printf("BAD %s: %ld vs %ld\n", what, a, b);
    ++bad;
  };
  for (uint32_t r : doci::tc::rows_without_columns(L, N, sp, D, B.data(), BC)) {
    if (r >= D) fail("rows0 range", r, (long)D);
    else if (full) diag[r]++;
  }
  for (int kp = (na < N - 1 ? na : N - 1); kp >= 0; --kp) {
    const int jp = N - 1 - kp;
    if (jp < 0 || jp > sp) continue;
    const uint32_t n_s = binom(sp, jp), n_own = jp + 1 <= sp ? binom(sp, jp + 1) : 0, n_units = binom(na, kp);
    for (uint32_t u = 0; u < n_units; u += ustride) {
      const uint32_t mask = doci::dev::colex_unrank<BC>(u, na, kp, B.data());
      if (__builtin_popcount(mask) != kp) fail("unit popcount", __builtin_popcount(mask), kp);
      int64_t own = -1;
      if (n_own) {
        own = row_start(mask);
        if (own < 0 || own + n_own > D) { fail("own row", own, n_own); continue; }
        if (full)
          for (uint32_t c = 0; c < n_own; ++c) diag[own + c]++;
      }
      uint32_t hole_rs[16];
      int hole_b[16], nhr = 0;
      for (int b = 0; b < na; ++b)
        if (!(mask >> b & 1u)) {
          const int64_t rs = row_start(mask | (1u << b));
          if (rs < 0) fail("hole row", rs, b);
          hole_rs[nhr] = static_cast<uint32_t>(rs);
          hole_b[nhr++] = b;
        }
      if (nhr != na - kp) fail("holes", nhr, na - kp);
      const uint32_t ntiles = (n_s + kTile - 1) / kTile;
      for (uint32_t t = 0; t < ntiles; ++t) {
        const uint32_t c0 = t * kTile, c1 = c0 + kTile < n_s ? c0 + kTile : n_s;
        for (int h = 0; h < nhr; ++h) {
          uint32_t a0, a1;
          doci::tc::hole_segment(hole_rs[h], c0, c1, static_cast<uint32_t>(D), &a0, &a1);
          if ((a0 & 3u) || (a1 & 3u)) fail("segment alignment", a0, a1);
          if (a1 > D) fail("segment end", a1, (long)D);
          if (a1 - a0 > kSlot) fail("segment slot", a1 - a0, kSlot);
          for (uint32_t cs = c0; cs < c1; ++cs) {
            const uint32_t g = hole_rs[h] + cs;
            if (g < a0) fail("segment start", g, a0);
            if (g < a1 && g - a0 >= kSlot) fail("slot index", g - a0, kSlot);
            // the kernel reads the staged copy below the vector's last whole
            // 16-byte chunk, at slot index ((rs + c0) & 3) + (cs - c0)
            if (g < (static_cast<uint32_t>(D) & ~3u)) {
              if (g >= a1) fail("staged element not copied", g, a1);
              if (((hole_rs[h] + c0) & 3u) + (cs - c0) != g - a0) fail("kernel slot index", g, a0);
            }
            if (g >= D) fail("hole index", g, (long)D);
          }
        }
        for (uint32_t cs = c0; cs < c1; cs += sstride) {
          const uint32_t C = cset[coff[jp] + cs];
          if (__builtin_popcount(C) != jp) fail("cset popcount", __builtin_popcount(C), jp);
          uint32_t cx = 0;
          for (int d = 0, e = 0; d < sp; ++d)
            if (C >> d & 1u) cx += binom(d, ++e);
          if (cx != n_s - 1 - cs) fail("cset colex", cx, n_s - 1 - cs);
          const uint32_t S = C | (mask << sp);
          for (int a = 0; a < sp; ++a) {
            if (C >> a & 1u) continue;
            const uint32_t pos = doci::tc::own_pos(C, a, n_own, lo, c8, G);
            const uint64_t want = direct_rank(S | (1u << a), L, N);
            ++checked;
            if (pos >= n_own) fail("own pos range", pos, n_own);
            else if (static_cast<uint64_t>(own + pos) != want) fail("own pos", own + pos, (long)want);
            else if (full) hits[want]++;
          }
          for (int h = 0; h < nhr; ++h) {
            const uint64_t want = direct_rank(S | (1u << (sp + hole_b[h])), L, N);
            ++checked;
            if (hole_rs[h] + cs != want) fail("hole", hole_rs[h] + cs, (long)want);
            else if (full) hits[want]++;
          }
        }
      }
    }
  }
  if (full) {
    for (uint64_t r = 0; r < D; ++r) {
      if (hits[r] != static_cast<uint8_t>(N)) fail("hits", hits[r], N);
      if (diag[r] != 1) fail("diag writes", diag[r], 1);
    }
  }
  std::printf("L=%d N=%d split=%d checked=%ld bad=%ld\n", L, N, sp, checked, bad);
  return bad ? 1 : 0;
}
