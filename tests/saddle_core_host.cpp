// Host build of the saddle streamline digitizers' parallel form
// (msceer_gb300/csrc/saddle_core.cuh) for the CPU tests: every streamline integrated
// once without labels into per-voxel-step records, then rounds of claims and walks over
// the records until no claim changes -- the loops a kernel per phase would run, here as
// plain loops -- so the scheme's result is checked against the one-thread oracle
// without a GPU.
#include <algorithm>
#include <climits>
#include <cstdint>
#include <vector>

#include "../msceer_gb300/csrc/saddle_core.cuh"

using namespace msc::sl;

namespace {

bool is_greater(const float* f, int64_t a, int64_t b) {
  if (f[a] > f[b]) return true;
  if (f[b] > f[a]) return false;
  return a > b;
}

// Cell2HighestVertex as a vertex index
int64_t highest_vertex(const Grid& G, const float* f, int64_t id) {
  int64_t k[3];
  cell_coords(G, id, k);
  int64_t best = -1;
  for (int s = 0; s < 8; s++) {
    int64_t q[3];
    bool ok = true;
    for (int a = 0; a < 3; a++) {
      const int bit = (s >> a) & 1;
      if (!(k[a] & 1) && bit) ok = false;
      q[a] = (k[a] & 1) ? (bit ? k[a] + 1 : k[a] - 1) : k[a];
    }
    if (!ok) continue;
    const int64_t v = (q[0] >> 1) + (q[1] >> 1) * G.X + (q[2] >> 1) * G.X * G.Y;
    if (best < 0 || is_greater(f, v, best)) best = v;
  }
  return best;
}

// the critical saddles in the one-thread order: sorted by (value, id) (descending
// lines: (-value, id)) and taken from the end
std::vector<int64_t> saddle_order(const float* f, const uint8_t* grad, const Grid& G, int dsc) {
  struct Crit {
    float key;
    int64_t id;
  };
  std::vector<Crit> cr;
  const int64_t nc = G.dX * G.dY * G.dZ;
  const int sdim = dsc ? 1 : 2;
  for (int64_t id = 0; id < nc; id++) {
    int64_t k[3];
    cell_coords(G, id, k);
    if ((int)((k[0] & 1) + (k[1] & 1) + (k[2] & 1)) != sdim || !grad_critical(grad, id)) continue;
    const float v = f[highest_vertex(G, f, id)];
    cr.push_back({dsc ? -1 * v : v, id});
  }
  std::sort(cr.begin(), cr.end(), [](const Crit& a, const Crit& b) {
    if (a.key < b.key) return true;
    if (b.key < a.key) return false;
    return a.id < b.id;
  });
  std::vector<int64_t> order;
  for (size_t i = cr.size(); i-- > 0;) order.push_back(cr[i].id);
  return order;
}

struct Line {
  uint32_t item;
  LineState state;
  std::vector<StepRec> recs;
  int budget;  // voxel steps of the next piece
};

// budget 0: every streamline traced to its end before the rounds; budget b > 0: traced
// b voxel steps at first, and a streamline whose walk runs past its last record traced
// on (twice the previous piece) before the next round.
// stats: [streamlines, recorded steps, kept steps, rounds, pieces traced]
int run_lines(const Field& F, const Params& P, const uint8_t* grad, int dsc, uint8_t target, uint8_t* cells,
              int budget, int64_t* stats) {
  const Grid& G = F.g;
  const std::vector<int64_t> order = saddle_order(F.f, grad, G, dsc);
  std::vector<Line> lines;
  std::vector<std::pair<int64_t, uint32_t>> saddle_writes;
  uint32_t item = 0;
  int64_t pieces = 0;
  auto trace = [&](Line& L) {
    pieces++;
    const int r = trace_more(F, P, dsc, &L.state, L.budget > 0 ? L.budget : INT32_MAX, [&](const StepRec& s) {
      L.recs.push_back(s);
      return true;
    });
    if (L.budget < (1 << 28)) L.budget *= 2;
    return r >= 0;
  };
  for (const int64_t sad : order) {
    int64_t seeds[kMaxSeeds];
    const int ns = saddle_seeds(G, grad, sad, dsc, seeds);
    for (int i = 0; i < ns; i++) {
      int64_t k[3];
      cell_coords(G, seeds[i], k);
      const V3 seed = {(double)k[0] * 0.5, (double)k[1] * 0.5, (double)k[2] * 0.5};
      lines.push_back(Line{item++, line_start(P, seed), {}, budget});
      if (!trace(lines.back())) return -1;
    }
    saddle_writes.push_back({sad, item++});
  }
  const int64_t nc = G.dX * G.dY * G.dZ;
  std::vector<uint64_t> base(nc, kNoClaim);
  for (int64_t c = 0; c < nc; c++)
    if (cells[c] == target) base[c] = 0;
  std::vector<uint64_t> claim = base, next;
  std::vector<Line*> more;
  int64_t rounds = 0, kept = 0;
  for (;;) {
    next = base;
    for (const auto& w : saddle_writes) next[w.first] = std::min(next[w.first], event_key(w.second, 0, 0));
    kept = 0;
    more.clear();
    for (Line& L : lines) {
      bool ran_off = false;
      kept += walk_line(
          F, P, dsc, L.item, [&](int t) -> const StepRec& { return L.recs[t]; }, (int)L.recs.size(),
          [&](int64_t c) { return claim[c]; }, [&](int64_t c, uint64_t key) { next[c] = std::min(next[c], key); },
          &ran_off);
      if (ran_off && !L.state.done) more.push_back(&L);
    }
    rounds++;
    if (next == claim && more.empty()) break;
    claim.swap(next);
    for (Line* L : more)
      if (!trace(*L)) return -1;
  }
  for (int64_t c = 0; c < nc; c++)
    if (claim[c] != kNoClaim) cells[c] = target;
  int64_t recorded = 0;
  for (const Line& L : lines) recorded += (int64_t)L.recs.size();
  stats[0] += (int64_t)lines.size();
  stats[1] += recorded;
  stats[2] += kept;
  stats[3] = std::max(stats[3], rounds);
  stats[4] += pieces;
  return 0;
}

}  // namespace

// which: 1 ascending lines from the 2-saddles (label 4), 2 descending lines from the
// 1-saddles (label 5), 3 both (ascending first); cells updated in place.  budget: 0
// traces every streamline whole before the rounds, b > 0 in pieces of b, 2b, ... voxel
// steps.  stats: [streamlines, recorded steps, kept steps, rounds, pieces traced].
extern "C" int core_saddle_lines_3d(const float* f, const uint8_t* grad, const uint32_t* zeroed, int64_t X,
                                    int64_t Y, int64_t Z, int which, float ethresh, float gthresh, double max_step,
                                    int limit, int budget, uint8_t* cells, int64_t* stats) {
  if (X < 2 || Y < 2 || Z < 2 || limit < 0 || limit >= (1 << 27) || budget < 0) return -1;
  const Field F{f, zeroed, make_grid(X, Y, Z)};
  const Params P{ethresh, gthresh, max_step, limit};
  for (int i = 0; i < 5; i++) stats[i] = 0;
  if ((which & 1) && run_lines(F, P, grad, 0, 4, cells, budget, stats)) return -2;
  if ((which & 2) && run_lines(F, P, grad, 1, 5, cells, budget, stats)) return -2;
  return 0;
}
