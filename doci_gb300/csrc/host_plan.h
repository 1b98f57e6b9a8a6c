// host_plan.h -- the piece and group schedule of the host-buffer pair-form
// sigma (doci_sigma_host on kinds 6 and 9; executed in sigma_pair.cu), host
// code only, shared with the CPU check tests/host_checks/host_plan_check.cpp.
//
// The vector is cut into kPieces contiguous pieces.  x goes up piece by piece
// on a copy stream; the pair units (one per row part R' of the (N-1)-pair
// sets) are grouped by the first and last piece their rows (own row R',
// hole rows R' u b) reach; groups run alternately on two compute streams
// (their sums are atomic adds, so groups may overlap), each after its last
// piece is up, with the diagonal pass of a piece before the first group that
// reaches it; a piece of sigma goes down once every group reaching it is
// done.
#pragma once

#include <algorithm>
#include <cstdint>
#include <map>
#include <random>
#include <utility>
#include <vector>

namespace doci {
namespace hostplan {

constexpr int kPieces = 16;

struct Unit {
  uint32_t own, word;  // as in the pair kernels' block list: own row start or ~0, mask | k' << 24
  uint64_t sets;       // (N-1)-pair sets of the unit
  uint32_t touched;    // pieces its rows reach
};

struct Group {
  int first, count;     // units [first, first + count) of the group-ordered list
  int need;             // last piece its rows reach
  uint32_t touch_mask;  // pieces its rows reach
  uint32_t init_mask;   // pieces whose sigma = diag * x pass runs just before it
  uint32_t down_mask;   // pieces final after it
};

// Piece boundaries: piece k holds elements [off[k], off[k + 1]).
inline void pieces(uint64_t D, uint64_t off[kPieces + 1]) {
  for (int k = 0; k <= kPieces; ++k) off[k] = D * static_cast<uint64_t>(k) / kPieces;
}

inline int piece_of(const uint64_t off[kPieces + 1], uint64_t t) {
  int k = 0;
  while (k + 1 < kPieces && off[k + 1] <= t) ++k;
  return k;
}

// Pieces reached by the rows [rs, rs + len).
inline uint32_t row_pieces(const uint64_t off[kPieces + 1], uint64_t rs, uint64_t len) {
  uint32_t m = 0;
  if (!len) return 0;
  for (int c = piece_of(off, rs); c <= piece_of(off, rs + len - 1); ++c) m |= 1u << c;
  return m;
}

// Group order: minimises a model of the call (GB300 measurements: upload
// 211 GB/s, download 193 GB/s, the FP32 pair kernel 0.061 ns per set) by a
// deterministic local search (random pair swaps from the order by last
// piece).  The order only decides when the work runs: every order gives the
// same sigma.  flat receives the units in group order (own, word pairs).
inline void schedule(const std::vector<Unit> &hu, uint64_t D, std::vector<Group> &groups,
                     std::vector<uint32_t> &flat) {
  constexpr int NC = kPieces;
  struct Cls {
    double sets = 0;
    int first = NC, last = -1;
    uint32_t mask = 0;
    std::vector<const Unit *> units;
  };
  std::map<std::pair<int, int>, Cls> by;
  for (const Unit &u : hu) {
    if (!u.touched) continue;
    const int lo = __builtin_ctz(u.touched), hi = 31 - __builtin_clz(u.touched);
    Cls &c = by[{lo, hi}];
    c.sets += static_cast<double>(u.sets);
    c.first = lo;
    c.last = hi;
    c.mask |= u.touched;
    c.units.push_back(&u);
  }
  std::vector<Cls> cls;
  for (auto &kv : by) cls.push_back(std::move(kv.second));
  const double piece_bytes = static_cast<double>(D) * sizeof(float) / NC;
  const double t_up = piece_bytes / 211e9, t_down = piece_bytes / 193e9, t_set = 0.061e-9;
  auto model = [&](const std::vector<int> &order) {
    double t = 0, ready[NC];
    for (double &r : ready) r = -1;
    for (int i : order) {
      const Cls &c = cls[i];
      t = std::max(t, (c.last + 1) * t_up) + c.sets * t_set;
      for (int k = 0; k < NC; ++k)
        if (c.mask >> k & 1u) ready[k] = t;
    }
    t = std::max(t, NC * t_up);
    for (double &r : ready)
      if (r < 0) r = t;
    std::sort(ready, ready + NC);
    double d = 0;
    for (double r : ready) d = std::max(d, r) + t_down;
    return d;
  };
  std::vector<int> order(cls.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = static_cast<int>(i);
  std::sort(order.begin(), order.end(), [&](int a, int b) {
    return cls[a].last != cls[b].last ? cls[a].last < cls[b].last : cls[a].first < cls[b].first;
  });
  double best = model(order);
  if (order.size() > 1) {
    std::mt19937 rng(12345);
    std::uniform_int_distribution<size_t> pick(0, order.size() - 1);
    for (int it = 0; it < 20000; ++it) {
      std::vector<int> o = order;
      std::swap(o[pick(rng)], o[pick(rng)]);
      const double v = model(o);
      if (v <= best) {
        best = v;
        order.swap(o);
      }
    }
  }
  groups.clear();
  flat.clear();
  uint32_t inited = 0;
  int last_of[NC];
  for (int &l : last_of) l = -1;
  for (size_t g = 0; g < order.size(); ++g)
    for (int k = 0; k < NC; ++k)
      if (cls[order[g]].mask >> k & 1u) last_of[k] = static_cast<int>(g);
  for (size_t g = 0; g < order.size(); ++g) {
    const Cls &c = cls[order[g]];
    Group hg{};
    hg.first = static_cast<int>(flat.size() / 2);
    for (const Unit *u : c.units) {
      flat.push_back(u->own);
      flat.push_back(u->word);
    }
    hg.count = static_cast<int>(c.units.size());
    hg.need = c.last;
    hg.touch_mask = c.mask;
    const uint32_t upto = (c.last + 1 >= 32) ? 0xffffffffu : ((1u << (c.last + 1)) - 1u);
    hg.init_mask = upto & ~inited;
    inited |= hg.init_mask;
    for (int k = 0; k < NC; ++k)
      if (last_of[k] == static_cast<int>(g)) hg.down_mask |= 1u << k;
    groups.push_back(hg);
  }
  // pieces no unit reaches: their diagonal pass and download close the call
  Group tail{};
  tail.first = static_cast<int>(flat.size() / 2);
  tail.need = NC - 1;
  tail.init_mask = ((1u << NC) - 1u) & ~inited;
  for (int k = 0; k < NC; ++k)
    if (last_of[k] < 0) tail.down_mask |= 1u << k;
  if (tail.init_mask || tail.down_mask) groups.push_back(tail);
}

// One piece download after a step: the copy stream waits for the step's
// group event, for other_group's event (the last group on the other compute
// stream reaching the piece, or -1) and, with wait_init, for the piece's
// diagonal pass on the other stream.
struct Down {
  int piece, other_group;
  bool wait_init;
};

// What one call does per group, in order.  The executor's protocol: the
// uploads go first on the copy stream, each followed by its upload event;
// per step on compute stream `stream`: wait for upload event wait_up (if
// >= 0), run the diagonal passes of `init` (each followed by its init event),
// wait for the init events of `wait_init`, run the group's units, record the
// group's event, then the downloads; at the end the first stream waits for
// the second and for the copy stream.
struct Step {
  int stream;
  int wait_up;
  uint32_t init, wait_init;
  std::vector<Down> down;
};

inline std::vector<Step> steps(const std::vector<Group> &groups) {
  constexpr int NC = kPieces;
  std::vector<Step> out;
  int waited[2] = {-1, -1};
  int init_on[NC];        // stream of the piece's diagonal pass; 2 once both are ordered after it
  int last_touch[2][NC];  // per stream: last group reaching the piece
  for (int k = 0; k < NC; ++k) {
    init_on[k] = -1;
    last_touch[0][k] = last_touch[1][k] = -1;
  }
  for (int gi = 0; gi < static_cast<int>(groups.size()); ++gi) {
    const Group &g = groups[gi];
    const int r = gi & 1;
    Step s{};
    s.stream = r;
    s.wait_up = -1;
    if (g.need > waited[r]) {  // pieces go up in order: waiting for the last one covers the rest
      s.wait_up = g.need;
      waited[r] = g.need;
    }
    s.init = g.init_mask;
    for (int k = 0; k < NC; ++k)
      if (g.init_mask >> k & 1u) init_on[k] = r;
    for (int k = 0; k < NC; ++k)
      if ((g.touch_mask >> k & 1u) && init_on[k] == 1 - r) {
        s.wait_init |= 1u << k;
        init_on[k] = 2;
      }
    for (int k = 0; k < NC; ++k)
      if (g.touch_mask >> k & 1u) last_touch[r][k] = gi;
    for (int k = 0; k < NC; ++k)
      if (g.down_mask >> k & 1u) s.down.push_back({k, last_touch[1 - r][k], init_on[k] == 1 - r});
    out.push_back(std::move(s));
  }
  return out;
}

}  // namespace hostplan
}  // namespace doci
