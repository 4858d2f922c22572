// The per-streamline core of ondemandaccurate's saddle streamline digitizers (the
// needASC1 / needDSC1 modes: ondemandaccurate.cxx:254-382 ReIntegrateUpFrom2Saddles,
// :383-505 ReIntegrateDownFrom1Saddles, with DigitizingNumericStreamlineIntegrator3dASC /
// 3dDSC, gi_numeric_streamline_integrator.h:525-1080), written once for the device and
// the host.
//
// The reference integrates the streamlines one after another: saddles in value order,
// a breadth-first set of seed cells around each, every streamline labelling the chain
// of cells its voxel segments cross (hex-face-hex ascending, vertex-edge-vertex
// descending) and stopping where an accepted Euler step lands in a cell labelled
// before (by an earlier streamline or by itself); each segment's chain stops at its
// first labelled cell.  Only the ends depend on the labels: the path of a streamline is
// a function of its seed.  The parallel form therefore integrates every streamline
// once without labels, recording per voxel step its start, its iteration budget, the
// cells its accepted Euler steps first enter (the checks) and its end, and then settles
// the ends in rounds over the records: every live write claims its cell with its place
// in the one-thread order (a 64-bit key; the smallest key of a cell wins), and every
// streamline walks its steps again against the claims of the previous round -- it stops
// at its first check of a cell claimed before the check, and cuts each segment at its
// first cell claimed before the write.  Whether an event happens depends only on events
// earlier in the one-thread order, so after r rounds every event of dependency depth
// below r is decided as the one-thread run decides it; the rounds stop when no claim
// changes, at the one-thread result.
//
// Floating point follows the reference operation by operation (doubles, with the
// float products of `Vec3d * float`, gi_vectors.h:250): on the device every double
// operation is an explicitly rounded intrinsic (no contraction into FMAs); the host
// build compiles with -ffp-contract=off.
#pragma once
#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define SL_HD __host__ __device__ __forceinline__
#else
#define SL_HD inline
#endif

namespace msc {
namespace sl {

// events of one voxel advection (AdvectionEvent, gi_advection_events.h)
enum : int {
  kEvOutOfVoxel = 1,
  kEvOverMax = 2,
  kEvLowGradient = 3,
  kEvHit = 5,       // a check found its cell labelled (or the walk's stop_at)
  kEvForced = 6,    // near the boundary: the checkers stop at the first accepted step
  kEvOverflow = 7,  // more distinct cells in one voxel step than a record holds
};

constexpr int kMaxChecks = 9;   // a floor cube meets 8 vertex cells (1 hex), plus the exit
constexpr int kMaxChain = 6;    // three crossings: start, face, next, face, next, face
constexpr int kKeySlots = 16;   // per voxel step: checks 0..8, then the chain 9..14
constexpr uint64_t kNoClaim = ~0ull;

// place of an event in the one-thread order: item (a streamline, or a saddle's own
// write after its streamlines), voxel step, slot in the step
SL_HD uint64_t event_key(uint32_t item, uint32_t step, uint32_t slot) {
  return ((uint64_t)(item + 1u) << 32) | (uint64_t)(step * (uint32_t)kKeySlots + slot);
}

SL_HD double dmul(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
SL_HD double dadd(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
SL_HD double dsub(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
SL_HD double ddiv(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}
SL_HD double dsqrt(double a) {
#if defined(__CUDA_ARCH__)
  return __dsqrt_rn(a);
#else
  return std::sqrt(a);
#endif
}
SL_HD float fmulf(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}

struct V3 {
  double x, y, z;
};

struct Grid {
  int64_t X, Y, Z;     // vertices
  int64_t dX, dY, dZ;  // cells (2n - 1 per axis)
};

SL_HD Grid make_grid(int64_t X, int64_t Y, int64_t Z) { return {X, Y, Z, 2 * X - 1, 2 * Y - 1, 2 * Z - 1}; }

struct Params {
  float ethresh, gthresh;
  double max_step;
  int limit;  // Euler iterations per streamline
};

// The image, its central-difference gradient formed where it is read (the corner
// gradients of ComputeGradFromImage(1), gi_regular_grid_trilinear_function.h:285-341:
// float products summed in double; 0.0 + 0.0f * f on a first or last plane), zero at
// the vertices whose bit `zeroed` sets (the seeds whose gradient the integrations
// before the lines set to zero; null for none).
struct Field {
  const float* f;
  const uint32_t* zeroed;
  Grid g;

  SL_HD double component(int64_t v, int64_t c, int64_t n, int64_t stride) const {
    const float fc = f[v];
    if (c < 1 || c > n - 2) return dadd(0.0, (double)fmulf(0.0f, fc));
    double r = 0.0;
    r = dadd(r, (double)fmulf(-0.5f, f[v - stride]));
    r = dadd(r, (double)fmulf(0.0f, fc));
    r = dadd(r, (double)fmulf(0.5f, f[v + stride]));
    return r;
  }
  SL_HD V3 corner(int64_t x, int64_t y, int64_t z) const {
    const int64_t v = x + g.X * (y + g.Y * z);
    if (zeroed && ((zeroed[v >> 5] >> (v & 31)) & 1u)) return {0.0, 0.0, 0.0};
    return {component(v, x, g.X, 1), component(v, y, g.Y, g.X), component(v, z, g.Z, g.X * g.Y)};
  }
};

SL_HD double clampd(double v, int64_t n) {
  if (v < 0) v = 0;
  if (v >= (double)n) v = (double)n - 1;
  return v;
}

// Lerp (gi_vectors.h:349-351): a * (1 - t) + b * t
SL_HD V3 lerp(V3 a, V3 b, double t) {
  const double u = dsub(1.0, t);
  return {dadd(dmul(a.x, u), dmul(b.x, t)), dadd(dmul(a.y, u), dmul(b.y, t)), dadd(dmul(a.z, u), dmul(b.z, t))};
}
SL_HD double magsq(V3 a) { return dadd(dadd(dmul(a.x, a.x), dmul(a.y, a.y)), dmul(a.z, a.z)); }

// TriLinInterpGrad (gi_regular_grid_trilinear_function.h:211-229); vals in k-j-i order
SL_HD V3 trilin(V3 s, const int64_t b[3], const V3 vals[8]) {
  const double fx = dsub(s.x, (double)b[0]), fy = dsub(s.y, (double)b[1]), fz = dsub(s.z, (double)b[2]);
  const V3 x0 = lerp(vals[0], vals[1], fx), x1 = lerp(vals[2], vals[3], fx);
  const V3 x2 = lerp(vals[4], vals[5], fx), x3 = lerp(vals[6], vals[7], fx);
  return lerp(lerp(x0, x1, fy), lerp(x2, x3, fy), fz);
}

// GatherSurrounding (clamped near the boundary) / ...NoBoundaryCheck
SL_HD void surround(const Field& F, const int64_t b[3], bool clamp, V3 vals[8]) {
  const int64_t ext[3] = {F.g.X, F.g.Y, F.g.Z};
  int64_t vv[3][2];
  for (int a = 0; a < 3; a++) {
    vv[a][0] = b[a];
    vv[a][1] = b[a] + 1;
    if (clamp) {
      if (b[a] < 0) vv[a][0] = 0;
      if (b[a] >= ext[a] - 1) vv[a][0] = vv[a][1] = ext[a] - 1;
    }
  }
  for (int n = 0; n < 8; n++) vals[n] = F.corner(vv[0][n & 1], vv[1][(n >> 1) & 1], vv[2][n >> 2]);
}

// The cell a checker reads for a point: the hex holding it (TerminateNearAssignedHex:
// floor * 2 + 1) ascending, the vertex nearest it (TerminateNearAssignedVert:
// floor(p + 0.5) * 2) descending (gi_advection_checker.h:60-100); -1 outside the grid.
SL_HD int64_t check_cell(const Grid& G, int dsc, V3 p) {
  const double q[3] = {p.x, p.y, p.z};
  const int64_t d[3] = {G.dX, G.dY, G.dZ};
  int64_t k[3];
  for (int a = 0; a < 3; a++) {
    k[a] = dsc ? (int64_t)floor(dadd(q[a], 0.5)) * 2 : (int64_t)floor(q[a]) * 2 + 1;
    if (k[a] < 0 || k[a] >= d[a]) return -1;
  }
  return k[0] + G.dX * (k[1] + G.dY * k[2]);
}

// One voxel advection (AdvectThroughVoxelNoCheck / ...NearBoundary,
// gi_adaptive_euler_advector.h:51-176, 182-305) of a digitizing streamline, without
// labels: the cells its accepted steps enter go to chk (first entries, in order).
// stop_at >= 0 ends the advection where that entry is made (the walk's hit), *cur at
// the step that made it.  Near the boundary the first accepted step ends it (the
// checkers stop there whatever the labels).
SL_HD int voxel_step(const Field& F, const Params& P, int dsc, V3* cur, int* iters, bool nearb, int64_t* chk,
                     int* nchk, int stop_at) {
  const int64_t ext[3] = {F.g.X, F.g.Y, F.g.Z};
  const double p0[3] = {cur->x, cur->y, cur->z};
  int64_t b[3];
  for (int a = 0; a < 3; a++) b[a] = nearb ? (int64_t)clampd(p0[a], ext[a]) : (int64_t)p0[a];
  V3 vals[8];
  surround(F, b, nearb, vals);
  V3 old = *cur;
  V3 g = trilin(*cur, b, vals);
  float gm = (float)dsqrt(magsq(g));
  float step = (float)ddiv(P.max_step, (double)gm);
  const int sgn = dsc ? -1 : 1;  // StepMultiplier: ascending lines climb
  *nchk = 0;
  while ((*iters)-- > 0) {
    if (!(old.x == cur->x && old.y == cur->y && old.z == cur->z)) {
      if ((int)cur->x != (int)old.x || (int)cur->y != (int)old.y || (int)cur->z != (int)old.z) return kEvOutOfVoxel;
      g = trilin(*cur, b, vals);
      gm = (float)dsqrt(magsq(g));
      if ((double)fmulf(gm, step) > P.max_step) step = (float)ddiv(P.max_step, (double)gm);
      old = *cur;
    }
    if (gm < P.gthresh) return kEvLowGradient;
    // the full step in float (Vec3d * float), two half steps in double
    const float sm = fmulf((float)sgn, step);
    const V3 e1 = {(double)fmulf((float)g.x, sm), (double)fmulf((float)g.y, sm), (double)fmulf((float)g.z, sm)};
    const double hs = dmul((double)step, dmul((double)sgn, 0.5));
    const V3 hd = {dmul(g.x, hs), dmul(g.y, hs), dmul(g.z, hs)};
    const V3 hp = {dadd(cur->x, hd.x), dadd(cur->y, hd.y), dadd(cur->z, hd.z)};
    const V3 hg = trilin(hp, b, vals);
    const V3 e2 = {dadd(dmul(hg.x, hs), hd.x), dadd(dmul(hg.y, hs), hd.y), dadd(dmul(hg.z, hs), hd.z)};
    const V3 df = {dsub(e2.x, e1.x), dsub(e2.y, e1.y), dsub(e2.z, e1.z)};
    const float err = (float)magsq(df);
    if (err < P.ethresh) {
      V3 np = {dadd(cur->x, e2.x), dadd(cur->y, e2.y), dadd(cur->z, e2.z)};
      if (nearb) np = {clampd(np.x, ext[0]), clampd(np.y, ext[1]), clampd(np.z, ext[2])};
      *cur = np;
      const float a = (float)dmul((double)step, 1.8), bb = (float)ddiv(P.max_step, (double)gm);
      step = a < bb ? a : bb;
      if (nearb) return kEvForced;
      const int64_t id = check_cell(F.g, dsc, np);
      if (id >= 0) {
        int i = 0;
        while (i < *nchk && chk[i] != id) i++;
        if (i == *nchk) {
          if (i == kMaxChecks) return kEvOverflow;
          chk[(*nchk)++] = id;
          if (i == stop_at) return kEvHit;
        }
      }
    } else {
      step = (float)dmul((double)step, 0.5);
    }
  }
  return kEvOverMax;
}

SL_HD void cell_coords(const Grid& G, int64_t id, int64_t k[3]) {
  k[0] = id % G.dX;
  k[1] = (id / G.dX) % G.dY;
  k[2] = id / (G.dX * G.dY);
}

// facets and cofacets in the iterator orders (+x, -x, +y, -y, +z, -z)
SL_HD int facets(const Grid& G, int64_t id, int64_t out[6]) {
  int64_t k[3];
  cell_coords(G, id, k);
  const int64_t st[3] = {1, G.dX, G.dX * G.dY};
  int n = 0;
  for (int a = 0; a < 3; a++)
    if (k[a] & 1) {
      out[n++] = id + st[a];
      out[n++] = id - st[a];
    }
  return n;
}
SL_HD int cofacets(const Grid& G, int64_t id, int64_t out[6]) {
  int64_t k[3];
  cell_coords(G, id, k);
  const int64_t st[3] = {1, G.dX, G.dX * G.dY}, d[3] = {G.dX, G.dY, G.dZ};
  int n = 0;
  for (int a = 0; a < 3; a++)
    if (!(k[a] & 1)) {
      if (k[a] != d[a] - 1) out[n++] = id + st[a];
      if (k[a] != 0) out[n++] = id - st[a];
    }
  return n;
}

// The chain of cells one voxel segment a -> b labels, in order, before any cut
// (DigitizeSegmentInternal, gi_numeric_streamline_integrator.h:558-713 ascending and
// its vertex-edge form descending): the segment's plane crossings sorted by their
// parameter, and for each crossing whose face (edge) bounds the current hex (vertex)
// the current cell, the face and the cell beyond it.
SL_HD int segment_chain(const Grid& G, V3 a0, V3 b0, int dsc, int64_t out[kMaxChain]) {
  double a[3] = {a0.x, a0.y, a0.z}, b[3] = {b0.x, b0.y, b0.z};
  if (dsc)
    for (int d = 0; d < 3; d++) {
      a[d] = dadd(a[d], 0.5);
      b[d] = dadd(b[d], 0.5);
    }
  const double a2b[3] = {dsub(b[0], a[0]), dsub(b[1], a[1]), dsub(b[2], a[2])};
  int64_t idx[3];
  double tt[3];
  int n = 0;
  for (int d = 0; d < 3; d++) {
    const int va = (int)floor(a[d]), vb = (int)floor(b[d]);
    if (va == vb) continue;
    const int plane = va > vb ? va : vb;
    const double t = ddiv(dsub((double)plane, a[d]), dsub(b[d], a[d]));
    tt[n] = t;
    if (t < 0 || t > 1) return 0;
    int64_t k[3];
    for (int e = 0; e < 3; e++)
      k[e] = (int64_t)floor(dadd(dmul(a2b[e], t), a[e])) * 2 + (e == d ? 0 : 1) - (dsc ? 1 : 0);
    idx[n++] = k[0] + G.dX * (k[1] + G.dY * k[2]);
  }
  // the order of the crossings: this exchange sort (its order of equal parameters
  // included) is the one the one-thread result depends on
  for (int i = 0; i < n; i++)
    for (int j = i; j < n; j++)
      if (tt[i] > tt[j]) {
        const int64_t ti = idx[i];
        idx[i] = idx[j];
        idx[j] = ti;
        const double td = tt[i];
        tt[i] = tt[j];
        tt[j] = td;
      }
  int64_t start;
  {
    int64_t k[3];
    for (int e = 0; e < 3; e++) k[e] = (int64_t)floor(a[e]) * 2 + (dsc ? 0 : 1);
    start = k[0] + G.dX * (k[1] + G.dY * k[2]);
  }
  int m = 0;
  for (int i = 0; i < n; i++) {
    const int64_t face = idx[i];
    int64_t around[6];
    const int na = dsc ? facets(G, face, around) : cofacets(G, face, around);
    bool has_start = false;
    int64_t next = -1;
    for (int j = 0; j < na; j++) {
      if (around[j] == start) has_start = true;
      else next = around[j];
    }
    if (!has_start) continue;
    out[m++] = start;
    out[m++] = face;
    start = next;
  }
  return m;
}

// .grad byte accessors: critical, and the pair (UncompressByteTo6NeighborOffset)
SL_HD bool grad_critical(const uint8_t* grad, int64_t id) { return ((grad[id] >> 2) & 7) == 7; }
SL_HD int64_t grad_pair(const Grid& G, const uint8_t* grad, int64_t id) {
  const unsigned code = (grad[id] >> 2) & 7;
  const int64_t off = (code >> 1) == 0 ? 1 : ((code >> 1) == 1 ? G.dX : G.dX * G.dY);
  return (code & 1) ? id - off : id + off;
}

constexpr int kMaxSeeds = 32;  // five pops of at most six cells each
constexpr int kMaxVisit = 72;

// The seed cells of one saddle, in the order the reference integrates from them
// (ondemandaccurate.cxx:300-356 / :430-480): a breadth-first walk of at most five pops
// from the saddle through its cofacets (facets) and their pairs; the hexes (vertices)
// met, critical or paired, in the order met.
SL_HD int saddle_seeds(const Grid& G, const uint8_t* grad, int64_t sad, int dsc, int64_t seeds[kMaxSeeds]) {
  int64_t result[kMaxSeeds], queue[kMaxSeeds + 1], visited[kMaxVisit];
  int nr = 0, qh = 0, qt = 0, nv = 0;
  auto seen = [&](int64_t id) {
    for (int i = 0; i < nv; i++)
      if (visited[i] == id) return true;
    return false;
  };
  auto visit = [&](int64_t id) {
    if (!seen(id) && nv < kMaxVisit) visited[nv++] = id;
  };
  queue[qt++] = sad;
  for (int counter = 4; qh < qt && counter >= 0; counter--) {
    const int64_t cur = queue[qh++];
    visit(cur);
    int64_t around[6];
    const int m = dsc ? facets(G, cur, around) : cofacets(G, cur, around);
    for (int j = 0; j < m; j++) {
      const int64_t t = around[j];
      if (seen(t)) continue;
      if (nr < kMaxSeeds) result[nr++] = t;
      visit(t);
      if (!grad_critical(grad, t)) {
        const int64_t pr = grad_pair(G, grad, t);
        visit(pr);
        // a pair outside the grid only comes from a damaged .grad: not walked
        if (qt < kMaxSeeds + 1 && (uint64_t)pr < (uint64_t)(G.dX * G.dY * G.dZ)) queue[qt++] = pr;
      }
    }
  }
  const int tdim = dsc ? 0 : 3;
  int ns = 0;
  for (int i = 0; i < nr; i++) {
    int64_t k[3];
    cell_coords(G, result[i], k);
    if ((int)((k[0] & 1) + (k[1] & 1) + (k[2] & 1)) == tdim) seeds[ns++] = result[i];
  }
  return ns;
}

// One voxel step of a streamline's record.
struct StepRec {
  V3 old, end;      // start and label-free end of the voxel advection
  int it0;          // iterations left at its start
  int ev;           // label-free event that ended it
  int nchk;         // checks made (first entries)
  bool nearb;       // advected near the boundary (ends the streamline, writes nothing)
  int64_t chk[kMaxChecks];
};

// Where a label-free streamline stands between voxel steps (to trace it in pieces).
struct LineState {
  V3 cur;
  int iters;
  int64_t x, y, z;  // its nearest vertex
  bool done;        // it has ended
};

SL_HD LineState line_start(const Params& P, V3 seed) {
  return {seed, P.limit, (int64_t)dadd(seed.x, 0.5), (int64_t)dadd(seed.y, 0.5), (int64_t)dadd(seed.z, 0.5), false};
}

// IntegrateStreamline of the digitizing integrators without labels, from *S for at most
// max_steps voxel steps, one record per step (rec(const StepRec&) returns false to stop
// early, e.g. when a record buffer is full).  Returns the number of steps recorded, or
// -1 when a step overflowed its check list.
template <class Rec>
SL_HD int trace_more(const Field& F, const Params& P, int dsc, LineState* S, int max_steps, Rec rec) {
  const int64_t ext[3] = {F.g.X, F.g.Y, F.g.Z};
  int nsteps = 0;
  while (!S->done && nsteps < max_steps) {
    StepRec s;
    s.old = S->cur;
    s.it0 = S->iters;
    const int64_t xyz[3] = {S->x, S->y, S->z};
    int64_t dist = INT64_MAX;
    for (int a = 0; a < 3; a++) {
      const int64_t d = xyz[a] < ext[a] - 1 - xyz[a] ? xyz[a] : ext[a] - 1 - xyz[a];
      if (d < dist) dist = d;
    }
    s.nearb = dist <= 1;
    s.ev = voxel_step(F, P, dsc, &S->cur, &S->iters, s.nearb, s.chk, &s.nchk, -1);
    if (s.ev == kEvOverflow) return -1;
    s.end = S->cur;
    if (!rec(s)) return nsteps;
    nsteps++;
    if (s.nearb || s.ev != kEvOutOfVoxel) S->done = true;
    S->x = (int64_t)dadd(S->cur.x, 0.5);
    S->y = (int64_t)dadd(S->cur.y, 0.5);
    S->z = (int64_t)dadd(S->cur.z, 0.5);
  }
  return nsteps;
}

// The whole label-free streamline from `seed`.
template <class Rec>
SL_HD int trace_line(const Field& F, const Params& P, int dsc, V3 seed, Rec rec) {
  LineState S = line_start(P, seed);
  return trace_more(F, P, dsc, &S, INT32_MAX, rec);
}

// One streamline's walk over its records against the claims of the previous round
// (claim(cell): the smallest key of a live write of the cell, 0 for a cell labelled
// before the lines, kNoClaim for none): emit(cell, key) for each live write, in order.
// Returns the number of steps the streamline keeps; *ran_off (when given) tells whether
// the walk went past the last record of a streamline that goes on (records traced in
// pieces: it needs more).
template <class Steps, class Claim, class Emit>
SL_HD int walk_line(const Field& F, const Params& P, int dsc, uint32_t item, Steps steps, int nsteps, Claim claim,
                    Emit emit, bool* ran_off = nullptr) {
  if (ran_off) *ran_off = false;
  for (int t = 0; t < nsteps; t++) {
    const StepRec& s = steps(t);
    if (s.nearb) return t + 1;
    int hit = -1;
    for (int i = 0; i < s.nchk && hit < 0; i++)
      if (claim(s.chk[i]) < event_key(item, (uint32_t)t, (uint32_t)i)) hit = i;
    V3 end = s.end;
    if (hit >= 0) {  // the step again, to where it entered the labelled cell
      end = s.old;
      int iters = s.it0, n = 0;
      int64_t chk[kMaxChecks];
      voxel_step(F, P, dsc, &end, &iters, false, chk, &n, hit);
    }
    int64_t chain[kMaxChain];
    const int m = segment_chain(F.g, s.old, end, dsc, chain);
    for (int k = 0; k < m; k++) {
      const uint64_t key = event_key(item, (uint32_t)t, (uint32_t)(kMaxChecks + k));
      if (claim(chain[k]) < key) break;
      emit(chain[k], key);
    }
    if (hit >= 0 || s.ev != kEvOutOfVoxel) return t + 1;
  }
  if (ran_off) *ran_off = true;
  return nsteps;
}

}  // namespace sl
}  // namespace msc
