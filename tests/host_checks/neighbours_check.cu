// Host-side check of the sigma kernels' neighbour enumeration
// (doci_gb300/csrc/addressing.cuh, dev::Neighbours), compiled by nvcc and run
// on the CPU: for every determinant r of the sampled ranks, every hop
// i -> a must yield an index < D equal to the directly computed lexical rank
// of T \ i u a, each (occupied, empty) pair exactly once.
//   usage: neighbours_check L N [stride]
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../doci_gb300/csrc/addressing.cuh"

static uint64_t binom(unsigned n, unsigned k) {
  if (k > n) return 0;
  uint64_t r = 1;
  for (unsigned d = 1; d <= k; ++d) r = r * (n - k + d) / d;
  return r;
}

static uint64_t direct_rank(uint32_t bits, int L, int N) {  // D - 1 - sum_e C(L-1-c_e, N-e)
  uint64_t s = 0;
  int e = 0;
  for (int o = 0; o < L; ++o)
    if (bits >> o & 1u) { s += binom(L - 1 - o, N - e); ++e; }
  return binom(L, N) - 1 - s;
}

constexpr int BC = 35;

struct Checker {
  uint32_t bits;  // original orbitals
  int L, N;
  uint64_t D;
  long bad = 0, hops = 0;
  uint64_t seen = 0;  // bitmask of (m,q) pairs seen for this determinant (per m)
  std::vector<uint32_t> pairs;
  void begin(int) {}
  void hop(int m, int q, uint32_t idx) {
    ++hops;
    const int i = L - 1 - m, a = L - 1 - q;
    if (!(bits >> i & 1u) || (bits >> a & 1u)) { ++bad; return; }
    const uint32_t nb = (bits & ~(1u << i)) | (1u << a);
    if (idx >= D || idx != direct_rank(nb, L, N)) ++bad;
    pairs.push_back(static_cast<uint32_t>(m * 64 + q));
  }
};

template <int NH>
static int run(int L, int N, uint64_t stride) {
  std::vector<uint32_t> B(33 * BC);
  for (int n = 0; n < 33; ++n)
    for (int k = 0; k < BC; ++k) B[n * BC + k] = static_cast<uint32_t>(binom(n, k));
  const uint64_t D = binom(L, N);
  const int nh = L - N;
  long bad = 0, hops = 0, dets = 0;
  for (uint64_t r = 0; r < D; r += stride) {
    const uint32_t R = static_cast<uint32_t>(D - 1 - r);
    const uint32_t M = doci::dev::colex_unrank<BC>(R, L, N, B.data());
    if (doci::dev::colex_rank<BC>(M, B.data()) != R) ++bad;
    doci::dev::Neighbours<NH, BC> nbs;
    nbs.precompute(M, R, L, nh, B.data());
    Checker c{doci::dev::mirror_bits(M, L), L, N, D};
    if (__builtin_popcount(c.bits) != N || direct_rank(c.bits, L, N) != r) ++bad;
    nbs.visit(M, R, static_cast<uint32_t>(D - 1), N, nh, B.data(), c);
    if (c.hops != static_cast<long>(N) * nh) ++bad;
    std::vector<char> mark(64 * 64, 0);
    for (uint32_t p : c.pairs) {
      if (mark[p]) ++bad;
      mark[p] = 1;
    }
    bad += c.bad;
    hops += c.hops;
    ++dets;
  }
  std::printf("L=%d N=%d D=%llu dets=%ld hops=%ld bad=%ld\n", L, N, (unsigned long long)D, dets, hops, bad);
  return bad ? 1 : 0;
}

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  const int L = std::atoi(argv[1]), N = std::atoi(argv[2]);
  const uint64_t stride = argc > 3 ? std::strtoull(argv[3], nullptr, 10) : 1;
  const int nh = L - N;
  if (nh <= 4) return run<4>(L, N, stride);
  if (nh <= 8) return run<8>(L, N, stride);
  if (nh <= 12) return run<12>(L, N, stride);
  if (nh <= 16) return run<16>(L, N, stride);
  if (nh <= 20) return run<20>(L, N, stride);
  if (nh <= 24) return run<24>(L, N, stride);
  if (nh <= 28) return run<28>(L, N, stride);
  return run<32>(L, N, stride);
}
