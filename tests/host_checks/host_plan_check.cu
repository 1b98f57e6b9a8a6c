// Host-side check of the host-buffer pair sigma's piece and group schedule
// (doci_gb300/csrc/host_plan.h), compiled by nvcc and run on the CPU.  The
// units are listed by the library's rule (one per row part R' of the
// (N-1)-pair sets, largest first), with the pieces their rows reach computed
// from row starts recomputed here from first principles (lexical rank of the
// row's first determinant).  The library's schedule and launch steps are
// then run through a happens-before simulation of the executor's protocol
// (sigma_pair.cu, run_host_schedule: three streams, events recorded and
// waited as there), which must order
//   * each piece's upload before its diagonal pass and before every group
//     reaching it,
//   * each piece's diagonal pass before every group reaching it,
//   * every group reaching a piece, and its diagonal pass, before its
//     download,
// with one diagonal pass and one download per piece, every unit in exactly
// one group, and the first stream ordered after everything at the end.
// With a fourth argument the check plants a mistake in the steps first (the
// side stream's first upload wait dropped, or every wait of a download for
// the other stream's last group) and must then report it.
//   usage: host_plan_check L N split [drop-up | drop-other]
#include <bitset>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <set>
#include <string>
#include <vector>

#include "../../doci_gb300/csrc/addressing.cuh"
#include "../../doci_gb300/csrc/host_plan.h"

constexpr int BC = 35;
static uint64_t binom(unsigned n, unsigned k) {
  if (k > n) return 0;
  uint64_t r = 1;
  for (unsigned d = 1; d <= k; ++d) r = r * (n - k + d) / d;
  return r;
}
// lexical rank of a determinant (the reference's order) from its mirrored
// orbital set M (bit L-1-o = original orbital o)
static uint64_t direct_rank_mirrored(uint32_t M, int L, int N) {
  uint64_t s = 0;
  int e = 0;
  for (int o = 0; o < L; ++o) {
    if (M >> (L - 1 - o) & 1u) {
      s += binom(L - 1 - o, N - e);
      ++e;
    }
  }
  return binom(L, N) - 1 - s;
}

int main(int argc, char **argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: host_plan_check L N split\n");
    return 2;
  }
  namespace hp = doci::hostplan;
  const int L = std::atoi(argv[1]), N = std::atoi(argv[2]), sp = std::atoi(argv[3]);
  const int na = L - sp;
  std::vector<uint32_t> B(33 * BC, 0);
  for (int n = 0; n <= 32; ++n)
    for (int k = 0; k < BC; ++k) B[n * BC + k] = static_cast<uint32_t>(binom(n, k));
  const uint64_t D = binom(L, N);
  // the lowest rank of a row: its column part's colex-last set (rows hold
  // colex n - 1 - c at column c; ranks grow with c)
  auto row_start = [&](uint32_t R) -> uint64_t {
    const int j = N - __builtin_popcount(R);
    const uint32_t n = static_cast<uint32_t>(binom(sp, j));
    const uint32_t Cb = doci::dev::colex_unrank<BC>(n - 1, sp, j, B.data());
    return direct_rank_mirrored(Cb | (R << sp), L, N);
  };
  uint64_t off[hp::kPieces + 1];
  hp::pieces(D, off);
  uint64_t bad = 0;
  // units in the library's order: by mask, then stably by size, largest first
  std::vector<std::pair<uint64_t, hp::Unit>> bl;
  for (uint32_t mask = 0; mask < (1u << na); ++mask) {
    const int kp = __builtin_popcount(mask), jp = N - 1 - kp;
    if (jp < 0 || jp > sp) continue;
    hp::Unit u{};
    u.own = jp + 1 <= sp ? static_cast<uint32_t>(row_start(mask)) : 0xffffffffu;
    u.word = mask | (static_cast<uint32_t>(kp) << 24);
    u.sets = binom(sp, jp);
    if (u.own != 0xffffffffu) u.touched |= hp::row_pieces(off, u.own, binom(sp, jp + 1));
    for (int b = 0; b < na; ++b)
      if (!(mask >> b & 1u)) u.touched |= hp::row_pieces(off, row_start(mask | (1u << b)), binom(sp, jp));
    bl.push_back({u.sets, u});
  }
  std::stable_sort(bl.begin(), bl.end(), [](const auto &a, const auto &b) { return a.first > b.first; });
  std::vector<hp::Unit> units;
  for (auto &e : bl) units.push_back(e.second);
  std::vector<hp::Group> groups;
  std::vector<uint32_t> flat;
  hp::schedule(units, D, groups, flat);
  std::vector<hp::Step> steps = hp::steps(groups);
  if (steps.size() != groups.size()) ++bad;
  const std::string plant = argc > 4 ? argv[4] : "";
  if (plant == "drop-up" && steps.size() > 1) steps[1].wait_up = -1;
  if (plant == "drop-other")
    for (hp::Step &p : steps)
      for (hp::Down &d : p.down) d.other_group = -1;

  // every unit in exactly one group, inside the group's pieces
  std::map<std::pair<uint32_t, uint32_t>, const hp::Unit *> by_key;
  for (const hp::Unit &u : units) by_key[{u.own, u.word}] = &u;
  std::set<std::pair<uint32_t, uint32_t>> seen;
  size_t covered = 0;
  for (const hp::Group &g : groups) {
    if (g.first != static_cast<int>(covered)) ++bad;
    covered += g.count;
    for (int i = g.first; i < g.first + g.count; ++i) {
      const std::pair<uint32_t, uint32_t> key{flat[2 * i], flat[2 * i + 1]};
      auto it = by_key.find(key);
      if (it == by_key.end() || !seen.insert(key).second) {
        ++bad;
        continue;
      }
      const uint32_t t = it->second->touched;
      if ((t & ~g.touch_mask) || 31 - __builtin_clz(t) > g.need) ++bad;
    }
  }
  if (covered != units.size() || seen.size() != units.size() || flat.size() != 2 * units.size()) ++bad;

  // happens-before simulation of the executor's protocol
  using Set = std::bitset<1024>;
  Set clk[3];  // 0: the handle's stream, 1: the side stream, 2: the copy stream
  std::map<std::string, Set> ev;
  std::vector<Set> before;
  std::vector<std::string> what;
  auto op = [&](int s, const std::string &name) {
    const int id = static_cast<int>(before.size());
    before.push_back(clk[s]);
    what.push_back(name);
    clk[s].set(id);
    return id;
  };
  auto record = [&](int s, const std::string &e) { ev[e] = clk[s]; };
  auto wait = [&](int s, const std::string &e) {
    auto it = ev.find(e);
    if (it == ev.end()) {
      ++bad;  // waiting for an event not yet recorded in this call
      return;
    }
    clk[s] |= it->second;
  };
  const int NC = hp::kPieces;
  std::vector<int> up(NC), init(NC, -1), down(NC, -1), grp(groups.size(), -1);
  record(0, "start");
  wait(2, "start");
  wait(1, "start");
  for (int k = 0; k < NC; ++k) {
    up[k] = op(2, "up" + std::to_string(k));
    record(2, "up" + std::to_string(k));
  }
  for (size_t gi = 0; gi < steps.size(); ++gi) {
    const hp::Step &p = steps[gi];
    const int s = p.stream;
    if (s != 0 && s != 1) ++bad;
    if (p.wait_up >= 0) wait(s, "up" + std::to_string(p.wait_up));
    for (int k = 0; k < NC; ++k)
      if (p.init >> k & 1u) {
        if (init[k] >= 0) ++bad;  // one diagonal pass per piece
        init[k] = op(s, "init" + std::to_string(k));
        record(s, "init" + std::to_string(k));
      }
    for (int k = 0; k < NC; ++k)
      if (p.wait_init >> k & 1u) wait(s, "init" + std::to_string(k));
    grp[gi] = op(s, "group" + std::to_string(gi));
    record(s, "group" + std::to_string(gi));
    for (const hp::Down &d : p.down) {
      wait(2, "group" + std::to_string(gi));
      if (d.other_group >= 0) wait(2, "group" + std::to_string(d.other_group));
      if (d.wait_init) wait(2, "init" + std::to_string(d.piece));
      if (down[d.piece] >= 0) ++bad;  // one download per piece
      down[d.piece] = op(2, "down" + std::to_string(d.piece));
    }
  }
  record(1, "side");
  wait(0, "side");
  record(2, "end");
  wait(0, "end");
  for (int k = 0; k < NC; ++k) {
    if (init[k] < 0 || down[k] < 0) {
      ++bad;
      continue;
    }
    if (!before[init[k]].test(up[k])) ++bad;
    if (!before[down[k]].test(init[k])) ++bad;
  }
  for (size_t gi = 0; gi < groups.size(); ++gi)
    for (int k = 0; k < NC; ++k) {
      if (!(groups[gi].touch_mask >> k & 1u)) continue;
      if (init[k] < 0 || !before[grp[gi]].test(up[k]) || !before[grp[gi]].test(init[k])) ++bad;
      if (down[k] >= 0 && !before[down[k]].test(grp[gi])) ++bad;
    }
  for (size_t id = 0; id < before.size(); ++id)
    if (!clk[0].test(id)) ++bad;
  std::printf("L=%d N=%d split=%d D=%llu units=%zu groups=%zu ops=%zu bad=%llu\n", L, N, sp,
              static_cast<unsigned long long>(D), units.size(), groups.size(), before.size(),
              static_cast<unsigned long long>(bad));
  return bad ? 1 : 0;
}
