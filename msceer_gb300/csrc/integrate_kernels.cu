// K4: numerical streamline integration to destination labels, and the K5c cleaner.
//
// NumericIntegratorPathCompressingToTerminal::BeginIntegration
// (gi_numeric_integrator_path_compressing.h:75-433) with AdaptiveEulerAdvector3D
// (gi_adaptive_euler_advector.h:51-305):
//   pass 1   every unassigned vertex integrates (FP32) until its nearest vertex is
//            labelled in an earlier level of the reference's spread order, runs out
//            of gradient or of iterations; every vertex it passed takes the
//            destination label (path compression), level by level.
//   fix-up   vertices with a differently labelled 6-neighbour re-integrate until a
//            certain terminal region, in FP32, and those whose FP32 ending is
//            ambiguous again in FP64 with the reference's operation order (explicit
//            _rn intrinsics: no contraction); changed labels reopen their neighbours,
//            in waves to a fixpoint.
// All integration kernels run persistent warps whose lanes each advance their own
// streamline a few iterations per turn and take the next one as soon as it ends; a
// streamline trapped in a tiny orbit ends where the iteration limit would have ended
// it (outside the all-FP64 mode).
// IsolatedCCRegionRemoverNEW::ComputeOutput (gi_isolated_region_remover.h:155-192):
//   same-label 6-connected components by a lock-free union-find whose roots are the
//   components' first vertices in the walk order; every component that does not hold
//   its region's extremum joins the component of its first earlier neighbour from
//   another region; chains resolve by pointer jumping.
#include <cstdio>
#include <cstdlib>

#include "label_common.cuh"

namespace msc {

enum { EV_NONE = 0, EV_OUT_OF_VOXEL, EV_OVER_MAX_ITERATIONS, EV_LOW_GRADIENT, EV_HIT_EXTREMUM, EV_HIT_PREASSIGNED };


__device__ __forceinline__ int64_t vid(const VolDims& V, int64_t x, int64_t y, int64_t z) { return x + V.X * (y + V.Y * z); }

// ---- FP32 advector (pass 1) ------------------------------------------------------------

struct F3 {
  float x, y, z;
};
// clamp into [0, n - 1] given fn = (float)n
__device__ __forceinline__ float clampf_ext(float v, float fn) {
  if (v < 0.f) v = 0.f;
  if (v >= fn) v = fn - 1.f;
  return v;
}

// Streamlines differ in length by orders of magnitude (most end within a few dozen
// iterations, a few run to the iteration limit circling a sink on a boundary face), so
// a warp that integrated 32 fixed streamlines would idle most of its lanes behind the
// longest one.  Instead every lane runs its streamline one iteration per turn of the
// warp's loop and takes the next work item as soon as its own streamline ends; the
// items are handed out by one warp-aggregated atomicAdd per turn.
enum : int { kLaneIdle = 0, kLaneEnter, kLaneStep, kLaneEnd, kLaneDone };

struct Adv32 {
  const float4* G;
  VolDims V;
  IntegParams P;
  const uint8_t* lvl;    // pass-1 stop (when set): nearest vertex labelled in an earlier level
  int level;
  const uint8_t* state;  // fix-up stop (when set): nearest vertex certain terminal
  // Converted once on the host: (float)P.max_step, (float)P.step_mult, the extents
  // (float)V.X .. and (float)(V.X - 2) ..  (a double-to-float or 64-bit integer
  // conversion per iteration would run on the slow FP64 pipe)
  float ms = 0.f, sgn = 0.f;
  float ext[3] = {0.f, 0.f, 0.f}, ext2[3] = {0.f, 0.f, 0.f};
  int64_t XY = 0;    // vertices per z-plane
  bool i32 = false;  // vertex ids fit 32 bits

  static Adv32 make(const float4* G, const VolDims& V, const IntegParams& P, const uint8_t* lvl, int level,
                    const uint8_t* state) {
    Adv32 A{G, V, P, lvl, level, state};
    A.ms = (float)P.max_step;
    A.sgn = (float)P.step_mult;
    const int64_t e[3] = {V.X, V.Y, V.Z};
    for (int a = 0; a < 3; a++) {
      A.ext[a] = (float)e[a];
      A.ext2[a] = (float)(e[a] - 2);
    }
    A.XY = V.X * V.Y;
    A.i32 = V.X * V.Y * V.Z <= (int64_t)0xFFFFFFFF;
    return A;
  }

  // Vertex id of (x, y, z) in 32-bit arithmetic while the grid's ids fit 32 bits
  __device__ __forceinline__ int64_t index(int x, int y, int z) const {
    if (i32) return (int64_t)((uint32_t)x + (uint32_t)V.X * ((uint32_t)y + (uint32_t)V.Y * (uint32_t)z));
    return vid(V, x, y, z);
  }
  // The voxel that holds `cur` (clamped into the grid near its boundary): its base
  // corner as floats and its corner gradients, c[n] for the corners n = x + 2y + 4z,
  // stored for trilin() as c[2k] and c[2k + 1] - c[2k] (the difference along x).  A
  // voxel clamped onto the grid's last plane along an axis repeats that plane's
  // corners there.
  __device__ __forceinline__ void load_voxel(const F3& cur, bool nearb, float bf[3], F3 c[8]) const {
    const float p[3] = {cur.x, cur.y, cur.z};
    int b[3];
    int64_t o[3] = {1, V.X, XY};
    const int E[3] = {(int)V.X, (int)V.Y, (int)V.Z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
      b[a] = nearb ? (int)clampf_ext(p[a], ext[a]) : (int)fminf(fmaxf(p[a], 0.f), ext2[a]);
      b[a] = max(b[a], 0);
      if (nearb && b[a] >= E[a] - 1) o[a] = 0;
      bf[a] = (float)b[a];
    }
    const float4* q = G + index(b[0], b[1], b[2]);
#pragma unroll
    for (int n = 0; n < 8; n++) {
      const float4 v = __ldg(q + ((n & 1) ? o[0] : 0) + ((n & 2) ? o[1] : 0) + ((n & 4) ? o[2] : 0));
      c[n] = {v.x, v.y, v.z};
    }
#pragma unroll
    for (int n = 1; n < 8; n += 2) c[n] = {c[n].x - c[n - 1].x, c[n].y - c[n - 1].y, c[n].z - c[n - 1].z};
  }
  // Trilinear interpolation of the corner gradients at s (bf: the base corner as
  // floats; c as load_voxel() stores it), each linear interpolation as a + t (b - a)
  __device__ __forceinline__ static F3 mix3(F3 a, F3 d, float t) {
    return {fmaf(t, d.x, a.x), fmaf(t, d.y, a.y), fmaf(t, d.z, a.z)};
  }
  __device__ __forceinline__ static F3 sub3(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
  __device__ __forceinline__ static F3 trilin(F3 s, const float bf[3], const F3 c[8]) {
    const float fx = s.x - bf[0], fy = s.y - bf[1], fz = s.z - bf[2];
    const F3 x0 = mix3(c[0], c[1], fx), x1 = mix3(c[2], c[3], fx), x2 = mix3(c[4], c[5], fx), x3 = mix3(c[6], c[7], fx);
    const F3 y0 = mix3(x0, sub3(x1, x0), fy), y1 = mix3(x2, sub3(x3, x2), fy);
    return mix3(y0, sub3(y1, y0), fz);
  }
  // Vec3l(p + 0.5), clamped into the grid (the reference clamps only near the
  // boundary, where its own points can leave it; elsewhere clamping changes nothing)
  __device__ __forceinline__ void nearest3(F3 p, int& ix, int& iy, int& iz) const {
    ix = (int)clampf_ext(p.x + 0.5f, ext[0]);
    iy = (int)clampf_ext(p.y + 0.5f, ext[1]);
    iz = (int)clampf_ext(p.z + 0.5f, ext[2]);
  }
  __device__ __forceinline__ int64_t nearest(F3 p) const {
    int ix, iy, iz;
    nearest3(p, ix, iy, iz);
    return index(ix, iy, iz);
  }
  // The trapped-streamline test (IntegParams::trap_window): compares `cur` with the
  // anchor set trap_window iterations before, moves the anchor, counts the
  // consecutive tight windows in `n`; true once there are two.
  __device__ __forceinline__ bool trapped(const F3& cur, F3& anchor, int& n) const {
    const float d = fmaxf(fabsf(cur.x - anchor.x), fmaxf(fabsf(cur.y - anchor.y), fabsf(cur.z - anchor.z)));
    n = d < P.trap_radius ? n + 1 : 0;
    anchor = cur;
    return n >= 2;
  }
  // One round of a lane's streamline (phase kLaneEnter or kLaneStep): the loop body of
  // AdvectThroughVoxel{NoCheck,NearBoundary}, one `iters` decrement, with the entry
  // into a voxel folded in (x, y, z: the entering lane's nearest vertex).  Written
  // without branches between its outcomes (moved or not, step accepted or rejected):
  // every stepping lane of a warp runs the same instructions, so that the warp issues
  // one iteration's instructions per round rather than one per outcome.  A lane whose
  // last step was rejected evaluates the gradient at its unchanged position again (the
  // same value).  slim caches max_step / |g|.  EV_NONE to go on; gm_end: the gradient
  // magnitude at a low-gradient stop (0 where there was none).
  __device__ __forceinline__ int advance(int& phase, int x, int y, int z, F3& cur, F3& old, int& iters, bool& nb,
                                         float b[3], F3 c[8], F3& g, float& gm, float& step, float& slim,
                                         float& gm_end, int64_t& last_nv, unsigned long long& ntrips) const;
};

// Distance of vertex (x, y, z) to the grid's nearest face, in vertices
__device__ __forceinline__ int dist_to_boundary(const VolDims& V, int x, int y, int z) {
  const int X = (int)V.X, Y = (int)V.Y, Z = (int)V.Z;
  return min(min(min(x, X - 1 - x), min(y, Y - 1 - y)), min(z, Z - 1 - z));
}

__device__ __forceinline__ int Adv32::advance(int& phase, int x, int y, int z, F3& cur, F3& old, int& iters, bool& nb,
                                              float b[3], F3 c[8], F3& g, float& gm, float& step, float& slim,
                                              float& gm_end, int64_t& last_nv, unsigned long long& ntrips) const {
  const bool ent = phase == kLaneEnter;
  if (ent) {
    nb = dist_to_boundary(V, x, y, z) <= 1;
    load_voxel(cur, nb, b, c);
    gm_end = 0.f;
    phase = kLaneStep;
  }
  const bool moved = !ent && !(old.x == cur.x && old.y == cur.y && old.z == cur.z);
  const bool left = moved && ((int)cur.x != (int)old.x || (int)cur.y != (int)old.y || (int)cur.z != (int)old.z);
  const F3 gc = trilin(cur, b, c);
  const float gmc = sqrtf(gc.x * gc.x + gc.y * gc.y + gc.z * gc.z);
  const bool bad = !(gmc > 0.f) || !isfinite(gmc);
  // events before the step, in the reference's order: an entering lane stops on a
  // vanishing gradient before it takes an iteration; a stepping lane checks the
  // iteration count, then whether it left its voxel, then the gradient
  const bool counts = !(ent && bad);
  ntrips += counts;
  const bool spent = counts && !(iters > 0);
  iters -= counts;
  int ev = spent ? EV_OVER_MAX_ITERATIONS : EV_NONE;
  if (ent && bad) ev = EV_LOW_GRADIENT;
  if (!spent && left) ev = EV_OUT_OF_VOXEL;
  if (!spent && !left && moved && bad) ev = EV_LOW_GRADIENT;
  if (ev != EV_NONE) return ev;
  const float sl = ms / gmc;
  if (ent || gmc * step > ms) step = sl;
  g = gc;
  gm = gmc;
  slim = sl;
  old = cur;
  if (gm < P.gthresh) {
    gm_end = gm;
    return EV_LOW_GRADIENT;
  }
  // the adaptive Euler step: a full step and two half steps, accepted (the step grows)
  // when they agree within ethresh, otherwise halved
  const float sm = sgn * step;
  const F3 e1 = {g.x * sm, g.y * sm, g.z * sm};
  const float hs = sm * 0.5f;
  const F3 hd = {g.x * hs, g.y * hs, g.z * hs};
  const F3 hg = trilin({cur.x + hd.x, cur.y + hd.y, cur.z + hd.z}, b, c);
  const F3 e2 = {hg.x * hs + hd.x, hg.y * hs + hd.y, hg.z * hs + hd.z};
  const float dx = e2.x - e1.x, dy = e2.y - e1.y, dz = e2.z - e1.z;
  const bool acc = dx * dx + dy * dy + dz * dz < P.ethresh;
  F3 np = {cur.x + e2.x, cur.y + e2.y, cur.z + e2.z};
  if (nb) {
    np.x = clampf_ext(np.x, ext[0]);
    np.y = clampf_ext(np.y, ext[1]);
    np.z = clampf_ext(np.z, ext[2]);
  }
  step = acc ? fminf(step * 1.8f, sl) : step * 0.5f;
  if (acc) cur = np;
  // the stop test reads memory only when an accepted step changed the nearest vertex:
  // what it reads (certain terminals in the fix-up, earlier levels in the first pass)
  // does not change while the kernel runs, and a vertex it passed once does not stop
  // the streamline later
  const int64_t nv = nearest(np);
  if (acc && nv != last_nv) {
    const uint8_t st = state ? state[nv] : lvl[nv];
    const bool hit = state ? (st == kStSeed || st == kStTerminal) : st < level;
    if (hit) return EV_HIT_PREASSIGNED;
    last_nv = nv;
  }
  return EV_NONE;
}



// Vertex coordinates of index v; 32-bit division while the grid's indices fit 32 bits.
__device__ __forceinline__ void split_index(const VolDims& V, int64_t v, int& x, int& y, int& z) {
  if (V.X * V.Y * V.Z <= (int64_t)0xFFFFFFFF) {
    const uint32_t u = (uint32_t)v, X = (uint32_t)V.X, Y = (uint32_t)V.Y;
    const uint32_t r = u / X;
    x = (int)(u - r * X);
    y = (int)(r % Y);
    z = (int)(r / Y);
  } else {
    x = (int)(v % V.X);
    y = (int)((v / V.X) % V.Y);
    z = (int)(v / (V.X * V.Y));
  }
}

constexpr int kPathCap = 48;
constexpr unsigned kFullMask = 0xffffffffu;

// resident CTAs of 128 threads per SM for the lane-refilling kernels
constexpr int kLaneCtasPerSm = 16;

// Claims a work item for every lane of the warp that asks for one (`want`); returns
// the item of the calling lane (meaningless where it did not ask).
__device__ __forceinline__ unsigned long long claim_item(bool want, unsigned long long* work) {
  const unsigned ask = __ballot_sync(kFullMask, want);
  if (!ask) return 0;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(ask) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(work, (unsigned long long)__popc(ask));
  base = __shfl_sync(kFullMask, base, leader);
  return base + (unsigned long long)__popc(ask & ((1u << lane) - 1u));
}

// Adds the warp's trip counts to *trips (one atomic per warp; every lane calls it).
__device__ __forceinline__ void add_trips(unsigned long long n, unsigned long long* trips) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) n += __shfl_down_sync(kFullMask, n, o);
  if ((threadIdx.x & 31) == 0 && n) atomicAdd(trips, n);
}

// One level of the spread order (or a group of consecutive small levels, [L0, L1),
// which then act as one level: each of those launches would wait for its slowest
// streamline while the GPU idles).  Streamlines of a level see only the labels of
// earlier levels (lvl[v] < level; terminals are level 0, unlabelled vertices 255),
// so a level's outcome does not depend on thread timing; where several streamlines
// of the level pass the same unlabelled vertex, the smallest label wins (unsigned
// atomicMin: a region's id < "reached no region" < unlabelled).  Level by level the
// pass is therefore deterministic.  `work` counts the level's claimed items (zero at
// launch).
// The vertices of levels [L0, L1) not labelled in an earlier level, compacted into
// `items` (their order does not matter: a level's outcome does not depend on it).
// Checking here, before the level runs, skips exactly the vertices the level's
// streamlines would skip: those stamped below `level`.
__global__ void compact_level_kernel(const SpreadOrder S, int L0, int L1, const uint8_t* __restrict__ lvl, int level,
                                     int32_t* __restrict__ items, unsigned long long* __restrict__ n_items) {
  const int64_t count = S.offset[L1] - S.offset[L0];
  const int lane = threadIdx.x & 31;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t - lane < count;
       t += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = -1;
    if (t < count) {
      const int64_t u = S.offset[L0] + t;
      int L = L0;
      while (L + 1 < L1 && S.offset[L + 1] <= u) L++;
      i = S.start[L] + (u - S.offset[L]) * S.stride[L];
      if (lvl[i] < level) i = -1;
    }
    const unsigned m = __ballot_sync(kFullMask, i >= 0);  // (the loop bound is warp-uniform)
    if (!m) continue;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(n_items, (unsigned long long)__popc(m));
    base = __shfl_sync(kFullMask, base, 0);
    if (i >= 0) items[base + __popc(m & ((1u << lane) - 1u))] = (int32_t)i;
  }
}

template <int K>
__global__ void __launch_bounds__(128, 7) integrate_level_kernel(const Adv32 A, const int32_t* __restrict__ items,
                                                              const unsigned long long* __restrict__ n_items,
                                                              int32_t* __restrict__ lab, uint8_t* __restrict__ lvl,
                                                              unsigned long long* __restrict__ work,
                                                              unsigned long long* __restrict__ trips) {
  const VolDims& V = A.V;
  const int level = A.level;
  const unsigned long long count = *n_items;
  int path[kPathCap];
  int np = 0;
  int64_t end = 0;
  int phase = kLaneIdle;
  unsigned long long ntrips = 0;
  int x = 0, y = 0, z = 0;
  F3 cur = {0.f, 0.f, 0.f}, old = cur, g = cur;
  float gm = 0.f, step = 0.f, slim = 0.f, gm_end = 0.f;
  int iters = 0;
  bool nb = false;
  float b[3] = {0.f, 0.f, 0.f};
  F3 c[8];
  F3 anchor = cur;  // trapped-streamline test
  int t_iters = 0, t_n = 0;
  int64_t last_nv = -1;  // nearest vertex the stop test last passed
  while (true) {
    {
      const unsigned long long t = claim_item(phase == kLaneIdle, work);
      if (phase == kLaneIdle) {
        if (t >= count) {
          phase = kLaneDone;
        } else {
          const int64_t i = items[t];
          split_index(V, i, x, y, z);
          cur = {(float)x, (float)y, (float)z};
          iters = A.P.iteration_limit;
          anchor = cur;
          t_iters = iters;
          t_n = 0;
          last_nv = -1;
          np = 0;
          path[np++] = (int)i;
          phase = kLaneEnter;
        }
      }
    }
    if (__all_sync(kFullMask, phase == kLaneDone)) {
      add_trips(ntrips, trips);
      break;
    }
    // K steps; a lane that leaves its voxel enters the next one within the same turn,
    // a lane whose streamline ended waits for the turn's end
    for (int r = 0; r < K; r++) {
      if (phase != kLaneEnter && phase != kLaneStep) continue;
      const int ev = A.advance(phase, x, y, z, cur, old, iters, nb, b, c, g, gm, step, slim, gm_end, last_nv, ntrips);
      if (ev == EV_NONE) continue;
      A.nearest3(cur, x, y, z);
      end = vid(V, x, y, z);
      if (np < kPathCap) path[np++] = (int)end;
      phase = ev == EV_OUT_OF_VOXEL ? kLaneEnter : kLaneEnd;
    }
    {
      if (phase == kLaneStep && A.P.trap_window > 0 && t_iters - iters >= A.P.trap_window) {
        t_iters = iters;
        if (A.trapped(cur, anchor, t_n)) {  // ends where the iteration limit would have
          A.nearest3(cur, x, y, z);
          end = vid(V, x, y, z);
          if (np < kPathCap) path[np++] = (int)end;
          phase = kLaneEnd;
        }
      }
    }
    if (phase == kLaneEnd) {
      const uint8_t le = lvl[end];
      const int32_t lb = lab[end];
      int32_t dest = le < level ? lb : -1;
      if (dest == -1) dest = kLabelNone;  // reached no region: assigned to nothing
      // the path's level bytes are read eight at a time, so that one lane's write-back
      // waits for a memory round trip per eight vertices rather than per vertex
      for (int k0 = 0; k0 < np; k0 += 8) {
        int pk[8];
        uint8_t lk[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
          pk[j] = k0 + j < np ? path[k0 + j] : -1;
          lk[j] = pk[j] >= 0 ? lvl[pk[j]] : 0;
        }
#pragma unroll
        for (int j = 0; j < 8; j++) {
          if (pk[j] < 0 || lk[j] < level) continue;  // labelled in an earlier level: keep
          atomicMin(reinterpret_cast<unsigned int*>(&lab[pk[j]]), (unsigned int)dest);
          lvl[pk[j]] = (uint8_t)level;
        }
      }
      phase = kLaneIdle;
    }
  }
}

__global__ void init_levels_kernel(const int32_t* __restrict__ lab, uint8_t* __restrict__ lvl, int64_t N) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    lvl[i] = lab[i] == -1 ? 255 : 0;
}

// ---- FP64 advector (fix-up), the reference's arithmetic --------------------------------

struct D3 {
  double x, y, z;
};
__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ D3 dlerp(D3 a, D3 b, double t) {
  const double u = ds(1.0, t);
  return {da(dm(a.x, u), dm(b.x, t)), da(dm(a.y, u), dm(b.y, t)), da(dm(a.z, u), dm(b.z, t))};
}
__device__ __forceinline__ double magsq(D3 a) { return da(da(dm(a.x, a.x), dm(a.y, a.y)), dm(a.z, a.z)); }
__device__ __forceinline__ double clampd_ext(double v, int64_t n) {
  if (v < 0) v = 0;
  if (v >= (double)n) v = (double)n - 1;
  return v;
}

struct Adv64 {
  const double* G;  // x,y,z doubles per vertex (ComputeGradFromImage(1), zeroed at the seeds)
  VolDims V;
  IntegParams P;
  const uint8_t* state;  // fix-up stop: certain terminal

  __device__ __forceinline__ D3 corner(int64_t x, int64_t y, int64_t z) const {
    const double* p = G + 3 * vid(V, x, y, z);
    return {p[0], p[1], p[2]};
  }
  __device__ __forceinline__ void surround(const int64_t b[3], bool clamp, D3 c[8]) const {
    int64_t vv[3][2];
    const int64_t ext[3] = {V.X, V.Y, V.Z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
      vv[a][0] = b[a];
      vv[a][1] = b[a] + 1;
      if (clamp) {
        if (b[a] < 0) vv[a][0] = 0;
        if (b[a] >= ext[a] - 1) vv[a][0] = vv[a][1] = ext[a] - 1;
      }
    }
#pragma unroll
    for (int n = 0; n < 8; n++) c[n] = corner(vv[0][n & 1], vv[1][(n >> 1) & 1], vv[2][n >> 2]);
  }
  // bf: the base corner as doubles
  __device__ __forceinline__ static D3 trilin(D3 s, const double bf[3], const D3 c[8]) {
    const double fx = ds(s.x, bf[0]), fy = ds(s.y, bf[1]), fz = ds(s.z, bf[2]);
    const D3 x0 = dlerp(c[0], c[1], fx), x1 = dlerp(c[2], c[3], fx), x2 = dlerp(c[4], c[5], fx), x3 = dlerp(c[6], c[7], fx);
    return dlerp(dlerp(x0, x1, fy), dlerp(x2, x3, fy), fz);
  }
  __device__ __forceinline__ void nearest3(D3 p, int& ix, int& iy, int& iz) const {
    ix = (int)(int64_t)clampd_ext(da(p.x, 0.5), V.X);
    iy = (int)(int64_t)clampd_ext(da(p.y, 0.5), V.Y);
    iz = (int)(int64_t)clampd_ext(da(p.z, 0.5), V.Z);
  }
  __device__ __forceinline__ int64_t nearest(D3 p, bool) const {
    int ix, iy, iz;
    nearest3(p, ix, iy, iz);
    return vid(V, ix, iy, iz);
  }
  // The FP32 advector's trapped-streamline test on FP64 positions.
  __device__ __forceinline__ bool trapped(const D3& cur, D3& anchor, int& n) const {
    const double d = fmax(fabs(cur.x - anchor.x), fmax(fabs(cur.y - anchor.y), fabs(cur.z - anchor.z)));
    n = d < (double)P.trap_radius ? n + 1 : 0;
    anchor = cur;
    return n >= 2;
  }
  // The voxel that holds `cur` and its eight corner gradients (as the FP32 advector's)
  __device__ __forceinline__ void load_voxel(const D3& cur, bool nearb, double bf[3], D3 c[8]) const {
    int64_t b[3];
    if (nearb) {
      b[0] = (int64_t)clampd_ext(cur.x, V.X);
      b[1] = (int64_t)clampd_ext(cur.y, V.Y);
      b[2] = (int64_t)clampd_ext(cur.z, V.Z);
    } else {
      b[0] = (int64_t)fmin(fmax(cur.x, 0.0), (double)(V.X - 2));
      b[1] = (int64_t)fmin(fmax(cur.y, 0.0), (double)(V.Y - 2));
      b[2] = (int64_t)fmin(fmax(cur.z, 0.0), (double)(V.Z - 2));
    }
    surround(b, nearb, c);
    bf[0] = (double)b[0];
    bf[1] = (double)b[1];
    bf[2] = (double)b[2];
  }
  // The FP32 advector's round (Adv32::advance: one uniform iteration for every stepping
  // lane, the voxel entry folded in) in the reference's FP64 arithmetic.
  __device__ __forceinline__ int advance(int& phase, int x, int y, int z, D3& cur, D3& old, int& iters, bool& nb,
                                         double bf[3], D3 c[8], D3& g, float& gm, float& step,
                                         unsigned long long& ntrips) const {
    const bool ent = phase == kLaneEnter;
    if (ent) {
      nb = dist_to_boundary(V, x, y, z) <= 1;
      load_voxel(cur, nb, bf, c);
      phase = kLaneStep;
    }
    const bool moved = !ent && !(old.x == cur.x && old.y == cur.y && old.z == cur.z);
    const bool left = moved && ((int)cur.x != (int)old.x || (int)cur.y != (int)old.y || (int)cur.z != (int)old.z);
    const D3 gc = trilin(cur, bf, c);
    const float gmc = __double2float_rn(__dsqrt_rn(magsq(gc)));
    const bool bad = !(gmc > 0.f) || !isfinite(gmc);  // no direction to follow
    const bool counts = !(ent && bad);
    ntrips += counts;
    const bool spent = counts && !(iters > 0);
    iters -= counts;
    int ev = spent ? EV_OVER_MAX_ITERATIONS : EV_NONE;
    if (ent && bad) ev = EV_LOW_GRADIENT;
    if (!spent && left) ev = EV_OUT_OF_VOXEL;
    if (!spent && !left && moved && bad) ev = EV_LOW_GRADIENT;
    if (ev != EV_NONE) return ev;
    const float sl = __double2float_rn(__ddiv_rn(P.max_step, (double)gmc));
    if (ent || (double)__fmul_rn(gmc, step) > P.max_step) step = sl;
    g = gc;
    gm = gmc;
    old = cur;
    if (gm < P.gthresh) return EV_LOW_GRADIENT;
    // full step: Vec3d * float multiplies in float (gi_vectors.h:250)
    const float sm = __fmul_rn((float)P.step_mult, step);
    const D3 e1 = {(double)__fmul_rn(__double2float_rn(g.x), sm), (double)__fmul_rn(__double2float_rn(g.y), sm),
                   (double)__fmul_rn(__double2float_rn(g.z), sm)};
    const double hs = dm((double)step, (double)P.step_mult * 0.5);
    const D3 hd = {dm(g.x, hs), dm(g.y, hs), dm(g.z, hs)};
    const D3 hg = trilin({da(cur.x, hd.x), da(cur.y, hd.y), da(cur.z, hd.z)}, bf, c);
    const D3 e2 = {da(dm(hg.x, hs), hd.x), da(dm(hg.y, hs), hd.y), da(dm(hg.z, hs), hd.z)};
    const D3 df = {ds(e2.x, e1.x), ds(e2.y, e1.y), ds(e2.z, e1.z)};
    const bool acc = __double2float_rn(magsq(df)) < P.ethresh;
    D3 np = {da(cur.x, e2.x), da(cur.y, e2.y), da(cur.z, e2.z)};
    if (nb) {
      np.x = clampd_ext(np.x, V.X);
      np.y = clampd_ext(np.y, V.Y);
      np.z = clampd_ext(np.z, V.Z);
    }
    const float grown = __double2float_rn(dm((double)step, 1.8));
    step = acc ? (grown < sl ? grown : sl) : __double2float_rn(dm((double)step, 0.5));
    if (acc) {
      cur = np;
      const uint8_t st = state[nearest(cur, nb)];
      if (st == kStSeed || st == kStTerminal) return EV_HIT_PREASSIGNED;
    }
    return EV_NONE;
  }
};

// Vertices assigned in pass 1 with a differently labelled 6-neighbour (:279-307).
__global__ void boundary_set_kernel(const int32_t* __restrict__ lab, const uint8_t* __restrict__ state, const VolDims V,
                                    int64_t* __restrict__ list, int* __restrict__ n, uint32_t* __restrict__ queued) {
  const int64_t N = V.X * V.Y * V.Z;
  const int lane = threadIdx.x & 31;
  // a warp covers 32 consecutive vertices starting at a multiple of 32 (block size and
  // grid stride are multiples of 32), i.e. exactly one word of `queued`
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i - lane < N; i += (int64_t)gridDim.x * blockDim.x) {
    bool diff = false;
    if (i < N && state[i] == kStUnassigned) {
      int x, y, z;
      split_index(V, i, x, y, z);
      const int32_t l = lab[i];
      if (x < V.X - 1) diff |= lab[i + 1] != l;
      if (x > 0) diff |= lab[i - 1] != l;
      if (y < V.Y - 1) diff |= lab[i + V.X] != l;
      if (y > 0) diff |= lab[i - V.X] != l;
      if (z < V.Z - 1) diff |= lab[i + V.X * V.Y] != l;
      if (z > 0) diff |= lab[i - V.X * V.Y] != l;
    }
    const unsigned m = __ballot_sync(kFullMask, diff);  // (the loop bound is warp-uniform)
    if (!m) continue;
    int base = 0;
    if (lane == 0) {
      atomicOr(&queued[i >> 5], m);
      base = atomicAdd(n, __popc(m));
    }
    base = __shfl_sync(kFullMask, base, 0);
    if (diff) list[base + __popc(m & ((1u << lane) - 1u))] = i;
  }
}

// One fix-up wave (:330-415): re-integrate, stopping only at certain terminals.  The
// decided label is read from lab0, the labels as the first pass left them: at a
// certain terminal that is the region's label (never changed), and at any other
// ending (low gradient, iteration limit) it is a value no concurrent re-decision can
// be rewriting, so every wave's outcome is independent of thread timing.
template <int K>
__global__ void __launch_bounds__(32) fixup_kernel(const Adv64 A, int32_t* __restrict__ lab,
                                                    const int32_t* __restrict__ lab0, uint8_t* __restrict__ state,
                                                    const int64_t* __restrict__ list, int n, int64_t* __restrict__ next,
                                                    int* __restrict__ n_next, uint32_t* __restrict__ queued,
                                                    unsigned long long* __restrict__ work,
                                                    unsigned long long* __restrict__ trips) {
  const VolDims& V = A.V;
  int phase = kLaneIdle;
  unsigned long long ntrips = 0;
  int64_t v = 0;
  int x = 0, y = 0, z = 0;
  int32_t init = 0;
  D3 cur = {0.0, 0.0, 0.0}, old = cur, g = cur;
  float gm = 0.f, step = 0.f;
  int iters = 0;
  bool nb = false;
  double b[3] = {0.0, 0.0, 0.0};
  D3 c[8];
  D3 anchor = cur;  // trapped-streamline test (off in the all-FP64 mode)
  int t_iters = 0, t_n = 0;
  while (true) {
    const unsigned long long k = claim_item(phase == kLaneIdle, work);
    if (phase == kLaneIdle) {
      if (k >= (unsigned long long)n) {
        phase = kLaneDone;
      } else {
        v = list[k];
        atomicAnd(&queued[v >> 5], ~(1u << (v & 31)));
        init = lab[v];
        split_index(V, v, x, y, z);
        cur = {(double)x, (double)y, (double)z};
        iters = A.P.iteration_limit;
        anchor = cur;
        t_iters = iters;
        t_n = 0;
        phase = kLaneEnter;
      }
    }
    if (__all_sync(kFullMask, phase == kLaneDone)) {
      add_trips(ntrips, trips);
      break;
    }
    for (int r = 0; r < K; r++) {
      if (phase != kLaneEnter && phase != kLaneStep) continue;
      const int ev = A.advance(phase, x, y, z, cur, old, iters, nb, b, c, g, gm, step, ntrips);
      if (ev == EV_NONE) continue;
      A.nearest3(cur, x, y, z);
      phase = ev == EV_OUT_OF_VOXEL ? kLaneEnter : kLaneEnd;
    }
    if (phase == kLaneStep && A.P.trap_window > 0 && t_iters - iters >= A.P.trap_window) {
      t_iters = iters;
      if (A.trapped(cur, anchor, t_n)) {  // ends where the iteration limit would have
        A.nearest3(cur, x, y, z);
        phase = kLaneEnd;
      }
    }
    if (phase != kLaneEnd) continue;
    phase = kLaneIdle;
    const int64_t end = vid(V, x, y, z);
    int32_t nl = lab0[end];
    if (nl == -1) nl = kLabelNone;
    lab[v] = nl;
    state[v] = kStNonterminal;
    if (nl == init) continue;
    int vx, vy, vz;
    split_index(V, v, vx, vy, vz);
    const int64_t nbr[6] = {vx < V.X - 1 ? v + 1 : -1, vx > 0 ? v - 1 : -1, vy < V.Y - 1 ? v + V.X : -1,
                            vy > 0 ? v - V.X : -1, vz < V.Z - 1 ? v + V.X * V.Y : -1, vz > 0 ? v - V.X * V.Y : -1};
#pragma unroll
    for (int j = 0; j < 6; j++) {
      const int64_t u = nbr[j];
      if (u < 0 || state[u] != kStUnassigned || lab[u] == nl) continue;
      const uint32_t bit = 1u << (u & 31);
      if (atomicOr(&queued[u >> 5], bit) & bit) continue;
      next[atomicAdd(n_next, 1)] = u;
    }
  }
}

// One FP32 fix-up wave.  A streamline whose FP32 ending is ambiguous goes to the FP64
// list instead of being decided here:
//   it stopped at a gradient magnitude within 2^-8 (relative) below the threshold
//   (the FP64 stop test decides), or
//   amb_mode 0: its final point lies within 1/64 voxel of the plane where the
//     nearest vertex changes, and the vertex across that plane belongs to a
//     different certain region (FP32 rounding may have picked the wrong side);
//   amb_mode 2: its final voxel touches two different certain regions (any ending
//     within half a voxel of a basin boundary).
template <int K>
__global__ void __launch_bounds__(128, 7) fixup32_kernel(const Adv32 A, int32_t* __restrict__ lab,
                                                      const int32_t* __restrict__ lab0, uint8_t* __restrict__ state,
                                                      const int64_t* __restrict__ list, int n,
                                                      int64_t* __restrict__ next, int* __restrict__ n_next,
                                                      uint32_t* __restrict__ queued, int64_t* __restrict__ amb,
                                                      int* __restrict__ n_amb, int amb_mode,
                                                      unsigned long long* __restrict__ work,
                                                      unsigned long long* __restrict__ trips) {
  const VolDims& V = A.V;
  int phase = kLaneIdle;
  unsigned long long ntrips = 0;
  int64_t v = 0;
  int x = 0, y = 0, z = 0;
  int32_t init = 0;
  F3 cur = {0.f, 0.f, 0.f}, old = cur, g = cur;
  float gm = 0.f, step = 0.f, slim = 0.f, gm_end = 0.f;
  int iters = 0, ev = EV_NONE;
  bool nb = false;
  float b[3] = {0.f, 0.f, 0.f};
  F3 c[8];
  F3 anchor = cur;  // trapped-streamline test
  int t_iters = 0, t_n = 0;
  int64_t last_nv = -1;  // nearest vertex the stop test last passed
  while (true) {
    const unsigned long long k = claim_item(phase == kLaneIdle, work);
    if (phase == kLaneIdle) {
      if (k >= (unsigned long long)n) {
        phase = kLaneDone;
      } else {
        v = list[k];
        init = lab[v];
        split_index(V, v, x, y, z);
        cur = {(float)x, (float)y, (float)z};
        iters = A.P.iteration_limit;
        anchor = cur;
        t_iters = iters;
        t_n = 0;
        last_nv = -1;
        phase = kLaneEnter;
      }
    }
    if (__all_sync(kFullMask, phase == kLaneDone)) {
      add_trips(ntrips, trips);
      break;
    }
    for (int r = 0; r < K; r++) {
      if (phase != kLaneEnter && phase != kLaneStep) continue;
      ev = A.advance(phase, x, y, z, cur, old, iters, nb, b, c, g, gm, step, slim, gm_end, last_nv, ntrips);
      if (ev == EV_NONE) continue;
      A.nearest3(cur, x, y, z);
      phase = ev == EV_OUT_OF_VOXEL ? kLaneEnter : kLaneEnd;
    }
    {
      if (phase == kLaneStep && A.P.trap_window > 0 && t_iters - iters >= A.P.trap_window) {
        t_iters = iters;
        if (A.trapped(cur, anchor, t_n)) {  // ends where the iteration limit would have
          ev = EV_OVER_MAX_ITERATIONS;
          A.nearest3(cur, x, y, z);
          phase = kLaneEnd;
        }
      }
    }
    if (phase != kLaneEnd) continue;
    phase = kLaneIdle;
    const int64_t end = vid(V, x, y, z);
    const int32_t lend = lab0[end];
    // a low-gradient stop whose FP32 magnitude lies within 2^-8 (relative) of the
    // threshold: FP32 rounding could have taken the other side of the stop test.  A
    // streamline that decelerates into an extremum crosses the threshold well inside
    // that test's FP32 accuracy otherwise, and FP64 would stop it at the same step.
    bool ambiguous = ev == EV_LOW_GRADIENT && gm_end >= A.P.gthresh * (1.f - 1.f / 256.f);
    if (!ambiguous && ev == EV_HIT_PREASSIGNED && amb_mode == 0) {
      const float pc[3] = {cur.x, cur.y, cur.z};
      const int64_t ext[3] = {V.X, V.Y, V.Z};
      const int64_t ev3[3] = {x, y, z};
      const int32_t le = lend;
#pragma unroll
      for (int a = 0; a < 3; a++) {
        const float q = pc[a] + 0.5f;
        const float r = q - floorf(q);
        if (fminf(r, 1.f - r) >= (1.f / 64.f)) continue;
        const int64_t alt_c = ev3[a] + (r < 0.5f ? -1 : 1);
        if (alt_c < 0 || alt_c >= ext[a]) continue;
        int64_t ac[3] = {ev3[0], ev3[1], ev3[2]};
        ac[a] = alt_c;
        const int64_t u = vid(V, ac[0], ac[1], ac[2]);
        const uint8_t st = state[u];
        if ((st == kStSeed || st == kStTerminal) && lab0[u] != le) ambiguous = true;
      }
    } else if (!ambiguous && ev == EV_HIT_PREASSIGNED) {
      const int64_t bb[3] = {(int)fminf(fmaxf(cur.x, 0.f), A.ext2[0]), (int)fminf(fmaxf(cur.y, 0.f), A.ext2[1]),
                             (int)fminf(fmaxf(cur.z, 0.f), A.ext2[2])};
      int32_t seen = kLabelNone;
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int64_t u = vid(V, bb[0] + (q & 1), bb[1] + ((q >> 1) & 1), bb[2] + (q >> 2));
        const uint8_t st = state[u];
        if (st != kStSeed && st != kStTerminal) continue;
        const int32_t l = lab0[u];
        if (seen == kLabelNone) seen = l;
        else if (l != seen) ambiguous = true;
      }
    }
    if (ambiguous) {
      amb[atomicAdd(n_amb, 1)] = v;  // keeps its queued bit until the FP64 wave
      continue;
    }
    atomicAnd(&queued[v >> 5], ~(1u << (v & 31)));
    int32_t nl = lend;
    if (nl == -1) nl = kLabelNone;
    lab[v] = nl;
    state[v] = kStNonterminal;
    if (nl == init) continue;
    int vx, vy, vz;
    split_index(V, v, vx, vy, vz);
    const int64_t nbr[6] = {vx < V.X - 1 ? v + 1 : -1, vx > 0 ? v - 1 : -1, vy < V.Y - 1 ? v + V.X : -1,
                            vy > 0 ? v - V.X : -1, vz < V.Z - 1 ? v + V.X * V.Y : -1, vz > 0 ? v - V.X * V.Y : -1};
    // the six neighbours' bytes and labels are read together (one memory round trip)
    uint8_t su[6];
    int32_t lu[6];
#pragma unroll
    for (int j = 0; j < 6; j++) {
      su[j] = nbr[j] >= 0 ? state[nbr[j]] : (uint8_t)kStNonterminal;
      lu[j] = nbr[j] >= 0 ? lab[nbr[j]] : nl;
    }
#pragma unroll
    for (int j = 0; j < 6; j++) {
      const int64_t u = nbr[j];
      if (su[j] != kStUnassigned || lu[j] == nl) continue;
      const uint32_t bit = 1u << (u & 31);
      if (atomicOr(&queued[u >> 5], bit) & bit) continue;
      next[atomicAdd(n_next, 1)] = u;
    }
  }
}

// ---- K5c: isolated-region cleaner --------------------------------------------------------

__device__ __forceinline__ bool comes_before(const float* f, int dir, int64_t a, int64_t b) {
  return dir < 0 ? vgreater(f, b, a) : vgreater(f, a, b);
}

// Vertex ids are 32-bit here: the labeling takes fewer than 2^31 vertices.
__device__ __forceinline__ int32_t uf_find(int32_t* parent, int32_t v) {
  int32_t p = parent[v];
  while (p != v) {
    const int32_t gp = parent[p];
    if (gp != p) parent[v] = gp;  // path halving
    v = p;
    p = gp;
  }
  return v;
}

__global__ void uf_init_kernel(int32_t* __restrict__ parent, int64_t N) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    parent[i] = (int32_t)i;
}

// MergeWithSameNeighbors + MergeByOrder: the earlier root (walk order) stays root
__global__ void uf_hook_kernel(const int32_t* __restrict__ lab, const float* __restrict__ f, const VolDims V, int dir,
                               int32_t* __restrict__ parent) {
  const int64_t N = V.X * V.Y * V.Z;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N; v += (int64_t)gridDim.x * blockDim.x) {
    int x, y, z;
    split_index(V, v, x, y, z);
    const int64_t nbr[3] = {x < V.X - 1 ? v + 1 : -1, y < V.Y - 1 ? v + V.X : -1, z < V.Z - 1 ? v + V.X * V.Y : -1};
    for (int j = 0; j < 3; j++) {
      const int64_t u = nbr[j];
      if (u < 0 || lab[u] != lab[v]) continue;
      for (int guard = 0; guard < 1 << 20; guard++) {
        const int32_t ru = uf_find(parent, (int32_t)u), rv = uf_find(parent, (int32_t)v);
        if (ru == rv) break;
        const int32_t early = comes_before(f, dir, ru, rv) ? ru : rv;
        const int32_t late = early == ru ? rv : ru;
        if (atomicCAS(&parent[late], late, early) == late) break;
      }
    }
  }
}

// Root of every vertex by a read-only walk up the finished forest (path halving here
// would race with the other threads' walks and could leave a non-root behind).
__global__ void uf_roots_kernel(const int32_t* __restrict__ parent, int32_t* __restrict__ root, int64_t N) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t r = (int32_t)i;
    for (int64_t guard = 0; guard < N && parent[r] != r; guard++) r = parent[r];  // strictly earlier each hop
    root[i] = r;
  }
}

// MergeBoundaryExtrema: a component root joins the component of its first earlier
// neighbour from another region (itself if there is none, i.e. an extremum's component)
__global__ void clean_target_kernel(const int32_t* __restrict__ lab, const float* __restrict__ f, const VolDims V, int dir,
                                    const int32_t* __restrict__ parent, int32_t* __restrict__ target) {
  const int64_t N = V.X * V.Y * V.Z;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
    if (parent[r] != r) {
      target[r] = (int32_t)r;  // only roots are followed; keep the rest defined
      continue;
    }
    int x, y, z;
    split_index(V, r, x, y, z);
    const int64_t nbr[6] = {x < V.X - 1 ? r + 1 : -1, x > 0 ? r - 1 : -1, y < V.Y - 1 ? r + V.X : -1,
                            y > 0 ? r - V.X : -1, z < V.Z - 1 ? r + V.X * V.Y : -1, z > 0 ? r - V.X * V.Y : -1};
    int64_t earliest = r;
    for (int j = 0; j < 6; j++) {
      const int64_t u = nbr[j];
      if (u < 0 || !comes_before(f, dir, u, r) || lab[u] == lab[r]) continue;
      if (comes_before(f, dir, u, earliest)) earliest = u;
    }
    target[r] = parent[earliest];
  }
}

__global__ void clean_resolve_kernel(const int32_t* __restrict__ lab, const VolDims V, const int32_t* __restrict__ parent,
                                     const int32_t* __restrict__ target, int32_t* __restrict__ out) {
  const int64_t N = V.X * V.Y * V.Z;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N; v += (int64_t)gridDim.x * blockDim.x) {
    int32_t r = parent[v];
    for (int64_t guard = 0; guard < N && target[r] != r; guard++) r = target[r];  // strictly earlier each hop
    const int32_t l = lab[v];
    const int32_t lr = lab[r];
    // vertices that reached no region keep "none"; the rest take their final root's region
    int32_t o = (l == kLabelNone) ? -1 : lr;
    if (o == kLabelNone) o = -1;
    out[v] = o;
  }
}

// ---- launchers ---------------------------------------------------------------------------

// Stepping iterations per turn of the lane-refilling loops: more amortise the turn's
// hand-out and voxel-entry work, fewer leave less idle time after a lane's event.
// MSC_TRIPS_PER_TURN (2, 4, 8 or 16) overrides the default for tuning (512^3 k^-3
// labels, both stages alike: 0.44 / 0.43 / 0.42 s for 4 / 8 / 16).
// MSC_TRIPS_PER_TURN_PASS1 sets the first pass's apart from the fix-up's.
static int trips_env(const char* name, int dflt) {
  const char* e = std::getenv(name);
  const int v = e ? std::atoi(e) : dflt;
  return (v == 2 || v == 4 || v == 8 || v == 16) ? v : dflt;
}
int trips_per_turn() {
  static const int k = trips_env("MSC_TRIPS_PER_TURN", 16);
  return k;
}
static int trips_per_turn_pass1() {
  static const int k = trips_env("MSC_TRIPS_PER_TURN_PASS1", trips_per_turn());
  return k;
}

cudaError_t launch_integrate_pass1(const float4* G, const VolDims& V, const IntegParams& P, const SpreadOrder& S,
                                   int32_t* lab, uint8_t* lvl, unsigned long long* work, unsigned long long* trips,
                                   int32_t* items, unsigned long long* n_items, int num_sms, cudaStream_t stream) {
  const int64_t N = V.X * V.Y * V.Z;
  if (cudaError_t e = cudaMemsetAsync(work, 0, sizeof(unsigned long long) * 48, stream)) return e;
  ::msc::count_launch();
  init_levels_kernel<<<num_sms * 8, 256, 0, stream>>>(lab, lvl, N);
  // the levels up to a total of N/512 items form the first group (a fraction of the
  // volume small enough that their mutual path compression does not matter)
  const int64_t small = N / 512;
  int stamp = 0;
  for (int L0 = 0; L0 < S.nlev;) {
    int L1 = L0 + 1;
    while (L1 < S.nlev && S.offset[L1 + 1] - S.offset[L0] <= small) L1++;
    const int64_t count = S.offset[L1] - S.offset[L0];
    const int g0 = L0;
    L0 = L1;
    if (count <= 0) continue;
    const Adv32 A = Adv32::make(G, V, P, lvl, ++stamp, nullptr);
    const int64_t blocks = (count + 127) / 128;
    const int grid = (int)(blocks < num_sms * kLaneCtasPerSm ? blocks : num_sms * kLaneCtasPerSm);
    unsigned long long* w = work + (stamp - 1);
    if (cudaError_t e = cudaMemsetAsync(n_items, 0, sizeof(unsigned long long), stream)) return e;
    ::msc::count_launch();
    compact_level_kernel<<<grid, 128, 0, stream>>>(S, g0, L1, lvl, stamp, items, n_items);
    ::msc::count_launch();
    switch (trips_per_turn_pass1()) {
      case 16:
        integrate_level_kernel<16><<<grid, 128, 0, stream>>>(A, items, n_items, lab, lvl, w, trips);
        break;
      case 2:
        integrate_level_kernel<2><<<grid, 128, 0, stream>>>(A, items, n_items, lab, lvl, w, trips);
        break;
      case 4:
        integrate_level_kernel<4><<<grid, 128, 0, stream>>>(A, items, n_items, lab, lvl, w, trips);
        break;
      default:
        integrate_level_kernel<8><<<grid, 128, 0, stream>>>(A, items, n_items, lab, lvl, w, trips);
    }
    char what[64];
    std::snprintf(what, sizeof(what), "level %d-%d (%lld)", g0, L1 - 1, (long long)count);
    ::msc::label_trace(stream, P.step_mult, what);
  }
  return cudaGetLastError();
}

cudaError_t launch_boundary_set(const int32_t* lab, const uint8_t* state, const VolDims& V, int64_t* list, int* n,
                                uint32_t* queued, int num_sms, cudaStream_t stream) {
  ::msc::count_launch();
  boundary_set_kernel<<<num_sms * 8, 256, 0, stream>>>(lab, state, V, list, n, queued);
  return cudaGetLastError();
}

cudaError_t launch_fixup(const double* G, const VolDims& V, const IntegParams& P, int32_t* lab, const int32_t* lab0,
                         uint8_t* state, const int64_t* list, int n, int64_t* next, int* n_next, uint32_t* queued,
                         unsigned long long* work, unsigned long long* trips, int num_sms, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  Adv64 A{G, V, P, state};
  const int blocks = (n + 31) / 32;
  if (cudaError_t e = cudaMemsetAsync(work, 0, sizeof(unsigned long long), stream)) return e;
  ::msc::count_launch();
  // one-warp CTAs, at most four per SM: the FP64 re-decisions are few (~0.1% of the
  // re-decisions) and bound by each SM's FP64 pipe, which executes every warp
  // instruction in full however few lanes are active -- so a small wave is spread over
  // as many SMs as it has warps, and a large one keeps a few items per lane (512^3
  // labels: 1.10 s with 16 CTAs of 128 per SM, 1.07 s with one)
  // iterations per turn: MSC_TRIPS_PER_TURN_FP64 (2, 4, 8 or 16) overrides the default
  // (512^3 k^-3 labels: the same time for 2, 8 and 16 -- the FP64 waves are as long as
  // their slowest streamline, not bound by the hand-out)
  static const int k = trips_env("MSC_TRIPS_PER_TURN_FP64", 2);
  const int grid = blocks < num_sms * 4 ? blocks : num_sms * 4;
  switch (k) {
    case 4:
      fixup_kernel<4><<<grid, 32, 0, stream>>>(A, lab, lab0, state, list, n, next, n_next, queued, work, trips);
      break;
    case 16:
      fixup_kernel<16><<<grid, 32, 0, stream>>>(A, lab, lab0, state, list, n, next, n_next, queued, work, trips);
      break;
    case 8:
      fixup_kernel<8><<<grid, 32, 0, stream>>>(A, lab, lab0, state, list, n, next, n_next, queued, work, trips);
      break;
    default:
      fixup_kernel<2><<<grid, 32, 0, stream>>>(A, lab, lab0, state, list, n, next, n_next, queued, work, trips);
  }
  return cudaGetLastError();
}

cudaError_t launch_fixup32(const float4* G, const VolDims& V, const IntegParams& P, int32_t* lab, const int32_t* lab0,
                           uint8_t* state, const int64_t* list, int n, int64_t* next, int* n_next, uint32_t* queued,
                           int64_t* amb, int* n_amb, int amb_mode, unsigned long long* work,
                           unsigned long long* trips, int num_sms, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const Adv32 A = Adv32::make(G, V, P, nullptr, 0, state);
  const int blocks = (n + 127) / 128;
  if (cudaError_t e = cudaMemsetAsync(work, 0, sizeof(unsigned long long), stream)) return e;
  ::msc::count_launch();
  const int grid = blocks < num_sms * kLaneCtasPerSm ? blocks : num_sms * kLaneCtasPerSm;
  switch (trips_per_turn()) {
    case 16:
      fixup32_kernel<16><<<grid, 128, 0, stream>>>(A, lab, lab0, state, list, n, next, n_next, queued, amb,
                                                     n_amb, amb_mode, work, trips);
      break;
    case 2:
      fixup32_kernel<2><<<grid, 128, 0, stream>>>(A, lab, lab0, state, list, n, next, n_next, queued, amb,
                                                     n_amb, amb_mode, work, trips);
      break;
    case 4:
      fixup32_kernel<4><<<grid, 128, 0, stream>>>(A, lab, lab0, state, list, n, next, n_next, queued, amb,
                                                     n_amb, amb_mode, work, trips);
      break;
    default:
      fixup32_kernel<8><<<grid, 128, 0, stream>>>(A, lab, lab0, state, list, n, next, n_next, queued, amb,
                                                     n_amb, amb_mode, work, trips);
  }
  return cudaGetLastError();
}

cudaError_t launch_clean(const int32_t* lab, const float* f, const VolDims& V, int dir, int32_t* parent, int32_t* target,
                         int32_t* out, int num_sms, cudaStream_t stream) {
  const int64_t N = V.X * V.Y * V.Z;
  const int grid = num_sms * 8;
  ::msc::count_launch();
  uf_init_kernel<<<grid, 256, 0, stream>>>(parent, N);
  ::msc::count_launch();
  uf_hook_kernel<<<grid, 256, 0, stream>>>(lab, f, V, dir, parent);
  // roots into `target`; from there on `target` holds the roots and `parent` the merge targets
  ::msc::count_launch();
  uf_roots_kernel<<<grid, 256, 0, stream>>>(parent, target, N);
  ::msc::count_launch();
  clean_target_kernel<<<grid, 256, 0, stream>>>(lab, f, V, dir, target, parent);
  ::msc::count_launch();
  clean_resolve_kernel<<<grid, 256, 0, stream>>>(lab, V, target, parent, out);
  return cudaGetLastError();
}

}  // namespace msc
