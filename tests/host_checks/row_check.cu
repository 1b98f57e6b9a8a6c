// Host-side check of the row-tiled sigma's index arithmetic
// (doci_gb300/csrc/addressing.cuh, dev::row_column_hops), compiled by nvcc and
// run on the CPU.  Row starts and every neighbour rank are recomputed here
// from first principles (lexical rank of the neighbour's bitstring); each of
// the N(L-N) hops of a determinant must be visited exactly once, in range.
//   usage: row_check L N split [row_stride] [col_stride]
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

struct Ctx {
  int L, N, sp;
  uint64_t D;
  std::vector<uint32_t> B;
};

static bool row_valid(const Ctx &x, uint32_t R) {
  const int j = x.N - __builtin_popcount(R);
  return j >= 0 && j <= x.sp;
}
static uint64_t row_start(const Ctx &x, uint32_t R) {
  const int j = x.N - __builtin_popcount(R);
  const uint32_t n = static_cast<uint32_t>(binom(x.sp, j));
  const uint32_t Mb = doci::dev::colex_unrank<BC>(n - 1, x.sp, j, x.B.data());
  return direct_rank_mirrored(Mb | (R << x.sp), x.L, x.N);
}

struct Check {
  const Ctx &x;
  uint32_t T;  // mirrored set of this determinant
  uint64_t rstart;
  uint32_t n;
  const uint64_t *ab_rs, *ba_rs, *aa_rs;
  const int *aa_m, *aa_q;
  const uint32_t *ab_len, *ba_len;
  long bad = 0, hops = 0;
  std::vector<char> seen = std::vector<char>(64 * 64, 0);
  void visit(int m, int q, uint64_t rank, uint32_t col, uint32_t len) {
    ++hops;
    if (!(T >> m & 1u) || (T >> q & 1u) || col >= len) { ++bad; return; }
    if (seen[m * 64 + q]++) ++bad;
    if (rank != direct_rank_mirrored((T & ~(1u << m)) | (1u << q), x.L, x.N)) ++bad;
  }
  void begin(int) {}
  void inrow(int m, int q, uint32_t c) { visit(m, q, rstart + c, c, n); }
  void up(int t, int m, int q, uint32_t c) { visit(m, q, ab_rs[t] + c, c, ab_len[t]); }
  void down(int t, int m, int q, uint32_t c) { visit(m, q, ba_rs[t] + c, c, ba_len[t]); }
  void across(int t, uint32_t c) { visit(aa_m[t], aa_q[t], aa_rs[t] + c, c, n); }
};

int main(int argc, char **argv) {
  if (argc < 4) return 2;
  Ctx x;
  x.L = std::atoi(argv[1]);
  x.N = std::atoi(argv[2]);
  x.sp = std::atoi(argv[3]);
  const long rstride = argc > 4 ? std::atol(argv[4]) : 1, cstride = argc > 5 ? std::atol(argv[5]) : 1;
  x.D = binom(x.L, x.N);
  x.B.resize(33 * BC);
  for (int a = 0; a < 33; ++a)
    for (int b = 0; b < BC; ++b) x.B[a * BC + b] = static_cast<uint32_t>(binom(a, b));
  const int na = x.L - x.sp;
  long bad = 0, dets = 0, rows = 0;
  std::vector<uint32_t> rem_tab, ins_tab, tab_off;
  doci::dev::build_cross_tables(x.sp, x.B.data(), BC, rem_tab, ins_tab, tab_off);
  uint64_t covered = 0;
  for (uint32_t R = 0; R < (1u << na); ++R) {
    if (!row_valid(x, R)) continue;
    const int k = __builtin_popcount(R), j = x.N - k;
    const uint32_t n = static_cast<uint32_t>(binom(x.sp, j));
    covered += n;
    if (rows++ % rstride) continue;
    // the library's closed form of the row start must agree
    uint64_t base = 0;
    for (int a = 0, t = 0; a < na; ++a)
      if (R >> a & 1u) base += binom(x.sp + a, j + 1 + t++);
    const uint64_t rs = row_start(x, R);
    if (rs != x.D - base - n) ++bad;
    std::vector<uint64_t> ab_rs, ba_rs, aa_rs;
    std::vector<uint32_t> ab_len, ba_len;
    std::vector<int> ab_m, ba_q, aa_m, aa_q;
    for (int a = 0; a < na; ++a) {
      if (R >> a & 1u) {
        ab_m.push_back(x.sp + a);
        const uint32_t R2 = R & ~(1u << a);
        ab_rs.push_back(row_valid(x, R2) ? row_start(x, R2) : ~0ull);
        ab_len.push_back(static_cast<uint32_t>(binom(x.sp, j + 1)));
      } else {
        ba_q.push_back(x.sp + a);
        const uint32_t R2 = R | (1u << a);
        ba_rs.push_back(row_valid(x, R2) ? row_start(x, R2) : ~0ull);
        ba_len.push_back(static_cast<uint32_t>(binom(x.sp, j - 1)));
      }
    }
    for (int e : ab_m)
      for (int h : ba_q) {
        aa_m.push_back(e);
        aa_q.push_back(h);
        aa_rs.push_back(row_start(x, (R & ~(1u << (e - x.sp))) | (1u << (h - x.sp))));
      }
    const int n_ab = j < x.sp ? static_cast<int>(ab_m.size()) : 0;
    const int n_ba = j > 0 ? static_cast<int>(ba_q.size()) : 0;
    for (uint32_t c = 0; c < n; c += static_cast<uint32_t>(cstride)) {
      const uint32_t Mb = doci::dev::colex_unrank<BC>(n - 1 - c, x.sp, j, x.B.data());
      const uint32_t T = Mb | (R << x.sp);
      Check f{x, T, rs, n, ab_rs.data(), ba_rs.data(), aa_rs.data(), aa_m.data(), aa_q.data(), ab_len.data(),
              ba_len.data()};
      if (direct_rank_mirrored(T, x.L, x.N) != rs + c) ++bad;
      doci::dev::row_column_hops<16, BC>(c, n, x.sp, j, x.B.data(), n_ab, ab_m.data(), n_ba, ba_q.data(),
                                         static_cast<int>(aa_rs.size()), f);
      if (f.hops != static_cast<long>(x.N) * (x.L - x.N)) ++bad;
      bad += f.bad;
      // the phase-ordered pass: cross hops through the tables
      {
        long th = 0;
        auto chk = [&](uint64_t rank, uint32_t nb_set) {
          ++th;
          if (rank != direct_rank_mirrored(nb_set, x.L, x.N)) ++bad;
        };
        for (int t = 0; t < n_ba; ++t)
          for (int e = 0; e < j; ++e) {
            const uint32_t v = rem_tab[tab_off[j] + 16 * c + e];
            const int m = static_cast<int>(v & 255u);
            if (!(Mb >> m & 1u) || (v >> 8) >= ba_len[t]) { ++bad; continue; }
            chk(ba_rs[t] + (v >> 8), (T & ~(1u << m)) | (1u << ba_q[t]));
          }
        for (int t = 0; t < n_ab; ++t)
          for (int h = 0; h < x.sp - j; ++h) {
            const uint32_t v = ins_tab[tab_off[j] + 16 * c + h];
            const int q = static_cast<int>(v & 255u);
            if ((Mb >> q & 1u) || q >= x.sp || (v >> 8) >= ab_len[t]) { ++bad; continue; }
            chk(ab_rs[t] + (v >> 8), (T & ~(1u << ab_m[t])) | (1u << q));
          }
        if (th != static_cast<long>(n_ba) * j + static_cast<long>(n_ab) * (x.sp - j)) ++bad;
      }
      ++dets;
    }
  }
  if (covered != x.D) ++bad;
  // Column-panel pass: sector-local row index = C(na,k) - 1 - colex(R); the
  // neighbour machinery on the row part must give the index of R \ m u q,
  // and every row-part hop of R exactly once.
  long col_rows = 0;
  for (uint32_t R = 0; R < (1u << na); R += static_cast<uint32_t>(rstride)) {
    if (!row_valid(x, R)) continue;
    const int k = __builtin_popcount(R);
    const uint32_t nr = static_cast<uint32_t>(binom(na, k));
    uint32_t colex = 0;
    for (int a = 0, t = 0; a < na; ++a)
      if (R >> a & 1u) colex += static_cast<uint32_t>(binom(a, ++t));
    struct ColCheck {
      uint32_t R;
      int na, k;
      uint32_t nr;
      long bad = 0, hops = 0;
      std::vector<char> seen = std::vector<char>(64 * 64, 0);
      void begin(int) {}
      void hop(int m, int q, uint32_t idx) {
        ++hops;
        if (!(R >> m & 1u) || (R >> q & 1u) || idx >= nr || seen[m * 64 + q]++) { ++bad; return; }
        const uint32_t R2 = (R & ~(1u << m)) | (1u << q);
        uint32_t c2 = 0;
        for (int a = 0, t = 0; a < na; ++a)
          if (R2 >> a & 1u) c2 += static_cast<uint32_t>(binom(a, ++t));
        if (idx != nr - 1 - c2) ++bad;
      }
    } f{R, na, k, nr};
    const uint32_t M = doci::dev::colex_unrank<BC>(colex, na, k, x.B.data());
    if (M != R) ++bad;
    // same register bound as the library: 16 row-part holes, else 24
    const int kmin = x.N - x.sp > 0 ? x.N - x.sp : 0;
    if (na - kmin > 16) {
      doci::dev::Neighbours<24, BC> nb;
      nb.precompute(M, colex, na, na - k, x.B.data());
      nb.visit(M, colex, nr - 1, k, na - k, x.B.data(), f);
    } else {
      doci::dev::Neighbours<16, BC> nb;
      nb.precompute(M, colex, na, na - k, x.B.data());
      nb.visit(M, colex, nr - 1, k, na - k, x.B.data(), f);
    }
    if (f.hops != static_cast<long>(k) * (na - k)) ++bad;
    bad += f.bad;
    ++col_rows;
  }
  std::printf("column pass rows checked=%ld\n", col_rows);
  std::printf("L=%d N=%d split=%d rows=%ld dets=%ld bad=%ld\n", x.L, x.N, x.sp, rows, dets, bad);
  return bad ? 1 : 0;
}
