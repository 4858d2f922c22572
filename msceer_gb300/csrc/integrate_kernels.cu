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

// CTAs of 128 threads per SM launched for the lane-refilling FP32 kernels (their
// registers allow 7 resident per SM); MSC_LANE_CTAS_PER_SM overrides it for tuning.
int lane_ctas_per_sm();

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

// Slots in a list whose length is *n for `cnt` entries of every thread of the block (one
// atomic per block): returns the thread's first slot.  Every thread of the block calls
// it, as often as the others (s_part: kAppendWarps + 1 ints of shared memory; blocks
// of whole warps).  Lists that most vertices enter (the boundary set, a wave's reopened
// neighbours: ~10^8 at 512^3) made millions of atomics on one counter with an append
// per warp, and those serialise in L2.
constexpr int kAppendWarps = 32;  // up to 1024 threads
__device__ __forceinline__ int block_append(int cnt, int* __restrict__ n, int* s_part) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(kFullMask, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) s_part[w] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int j = 0; j < nw; j++) {
      const int t = s_part[j];
      s_part[j] = run;
      run += t;
    }
    s_part[kAppendWarps] = run > 0 ? atomicAdd(n, run) : 0;
  }
  __syncthreads();
  const int slot = s_part[kAppendWarps] + s_part[w] + incl - cnt;
  __syncthreads();  // s_part is reused by the next call
  return slot;
}

// ---- first pass: speculation, then the reference's sequential outcome ------------------
//
// The reference's first pass (:150-240) visits the vertices one at a time in its spread
// order, and every streamline stops at the first vertex any earlier streamline labelled.
// Run a whole batch of that order at once and the streamlines no longer see each
// other's paths: on Gaussian-sum and k^-3 fields that alone moved 0.5-1% of the final
// labels away from the one-thread reference (the FP32 arithmetic moves ~1e-4).  The
// sequential outcome is recovered exactly, in parallel:
//   1. speculate: every streamline of the batch runs, stopping only at vertices
//      labelled before the batch, and records the sequence of vertices its stop test
//      passed (and which of them the reference pushes on its path).  The sequential
//      streamline is a prefix of this one: the advection does not read labels.
//   2. resolve: a path vertex belongs to the first item (in visiting order) whose
//      effective path holds it ("claim"); an item is skipped when an earlier one claims
//      its vertex, and its effective path ends at the first vertex an earlier one
//      claims ("cut").  Item k's outcome depends only on items < k, so recomputing
//      claims and cuts from the previous round's cuts reaches the sequential outcome.
//      After the first round only the claims of vertices between an item's old and new
//      extent can change; they are recomputed from the vertices' holder lists, and only
//      the items that hold such a vertex are looked at again.
//   3. label: a cut item takes the label of the item that claimed its stop vertex
//      (following the chain to an uncut one), an uncut item the label where it stopped;
//      every claimed vertex takes its claimer's label.
// Entry 0 of an item is its own vertex, entry 1 lies in an array of its own, entries
// from 2 on in segments of kSeg words in a pool (a full segment is followed by the word
// offset of the next).  Entries are vertex ids with kRec set on the reference's path
// vertices.

constexpr uint32_t kRec = 0x80000000u;
constexpr int kSeg = 32;
constexpr int kSpecBuf = 48;  // a lane holds <= kSeg entries at a turn's start, + at most K <= 16 in the turn
constexpr uint32_t kNoClaim = 0xFFFFFFFFu;

__device__ __forceinline__ int64_t spread_vertex(const SpreadOrder& S, int64_t u) {
  int L = 0;
  while (L + 1 < S.nlev && S.offset[L + 1] <= u) L++;
  return S.start[L] + (u - S.offset[L]) * S.stride[L];
}

// Ordered compaction of spread positions [u0, u1) whose vertex is not labelled yet:
// block b owns positions u0 + b*kCompactBlock + [0, kCompactBlock), 4 per thread.
constexpr int kCompactThreads = 256;
constexpr int kCompactBlock = 4 * kCompactThreads;

__device__ __forceinline__ int compact_flags(const SpreadOrder& S, int64_t u0, int64_t u1, const uint8_t* lvl,
                                             int stamp, int64_t vx[4]) {
  const int64_t ub = u0 + (int64_t)blockIdx.x * kCompactBlock + 4 * threadIdx.x;
  int n = 0;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    vx[j] = -1;
    const int64_t u = ub + j;
    if (u < u1) {
      const int64_t i = spread_vertex(S, u);
      if (lvl[i] >= stamp) {
        vx[j] = i;
        n++;
      }
    }
  }
  return n;
}

// exclusive block scan of one int per thread (kCompactThreads threads); returns the total
__device__ __forceinline__ int block_excl_scan(int v, int& excl, int* s_warp) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) s_warp[w] = incl;
  __syncthreads();
  if (w == 0) {
    const int nw = kCompactThreads / 32;
    int x = lane < nw ? s_warp[lane] : 0;
    int xi = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, xi, o);
      if (lane >= o) xi += u;
    }
    if (lane < nw) s_warp[lane] = xi - x;
    if (lane == nw - 1) s_warp[32] = xi;
  }
  __syncthreads();
  excl = s_warp[w] + incl - v;
  const int total = s_warp[32];
  __syncthreads();
  return total;
}

__global__ void __launch_bounds__(kCompactThreads) spread_count_kernel(const SpreadOrder S, int64_t u0, int64_t u1,
                                                                      const uint8_t* __restrict__ lvl, int stamp,
                                                                      int* __restrict__ counts) {
  __shared__ int s_warp[33];
  int64_t vx[4];
  const int n = compact_flags(S, u0, u1, lvl, stamp, vx);
  int excl;
  const int total = block_excl_scan(n, excl, s_warp);
  if (threadIdx.x == 0) counts[blockIdx.x] = total;
}

// one block: counts[0, nb) -> exclusive offsets in place, the total to *n_items
__global__ void __launch_bounds__(1024) scan_counts_kernel(int* __restrict__ counts, int64_t nb,
                                                           unsigned long long* __restrict__ n_items) {
  __shared__ long long s_part[1024];
  const int64_t per = (nb + 1023) / 1024;
  const int64_t b0 = threadIdx.x * per, b1 = b0 + per < nb ? b0 + per : nb;
  long long sum = 0;
  for (int64_t b = b0; b < b1; b++) sum += counts[b];
  s_part[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const long long u = threadIdx.x >= o ? s_part[threadIdx.x - o] : 0;
    __syncthreads();
    s_part[threadIdx.x] += u;
    __syncthreads();
  }
  long long run = s_part[threadIdx.x] - sum;
  for (int64_t b = b0; b < b1; b++) {
    const int c = counts[b];
    counts[b] = (int)run;
    run += c;
  }
  if (threadIdx.x == 1023) *n_items = (unsigned long long)s_part[1023];
}

__global__ void __launch_bounds__(kCompactThreads) spread_write_kernel(const SpreadOrder S, int64_t u0, int64_t u1,
                                                                      const uint8_t* __restrict__ lvl, int stamp,
                                                                      const int* __restrict__ offs,
                                                                      int32_t* __restrict__ items) {
  __shared__ int s_warp[33];
  int64_t vx[4];
  const int n = compact_flags(S, u0, u1, lvl, stamp, vx);
  int excl;
  block_excl_scan(n, excl, s_warp);
  int64_t o = (int64_t)offs[blockIdx.x] + excl;
#pragma unroll
  for (int j = 0; j < 4; j++)
    if (vx[j] >= 0) items[o++] = (int32_t)vx[j];
}

// Walks an item's entries in order.
struct SeqWalk {
  const SpecSet& Q;
  int64_t k;
  uint32_t seg = 0;
  int i = 0;
  __device__ __forceinline__ SeqWalk(const SpecSet& q, int64_t item) : Q(q), k(item) {}
  __device__ __forceinline__ uint32_t next() {
    const int j = i++;
    if (j == 0) return (uint32_t)Q.vtx[k] | kRec;
    if (j == 1) return Q.e1[k];
    const int p = j - 2;
    if (p == 0) seg = Q.head[k];
    else if ((p & (kSeg - 1)) == 0) seg = Q.pool[seg + kSeg];
    return Q.pool[seg + (p & (kSeg - 1))];
  }
};

// Speculative streamlines of items [k0, k1) of the ordered list: they stop only at
// vertices labelled before this batch (lvl < A.level), record their entries with a
// holder node per entry, and make the first round's claims (every item alive, its
// whole path effective).
template <int K>
__global__ void __launch_bounds__(128, 7) speculate_kernel(const Adv32 A, const SpecSet Q, int64_t k0, int64_t k1,
                                                           const int32_t* __restrict__ lab,
                                                           uint32_t* __restrict__ claim,
                                                           unsigned long long* __restrict__ work,
                                                           unsigned long long* __restrict__ trips) {
  const VolDims& V = A.V;
  const int level = A.level;
  const int lane = threadIdx.x & 31;
  uint32_t buf[kSpecBuf];  // entries from 2 on, not yet in the pool
  int nb = 0;
  int cnt = 0;             // entries so far
  uint32_t e1 = 0;         // entry 1
  int64_t k = -1;          // the lane's item
  int flushed = 0;         // pool entries written
  uint32_t link = 0;       // word offset of the last full segment's link slot
  int phase = kLaneIdle;
  unsigned long long ntrips = 0;
  int x = 0, y = 0, z = 0;
  F3 cur = {0.f, 0.f, 0.f}, old = cur, g = cur;
  float gm = 0.f, step = 0.f, slim = 0.f, gm_end = 0.f;
  int iters = 0;
  bool nb_near = false;
  float b[3] = {0.f, 0.f, 0.f};
  F3 c[8];
  F3 anchor = cur;
  int t_iters = 0, t_n = 0;
  int64_t last_nv = -1;
  int32_t endlab = kLabelNone;
  auto mark_rec = [&]() {  // the reference pushes its nearest vertex: the last one passed
    if (cnt == 2) e1 |= kRec;
    else if (cnt > 2) buf[nb - 1] |= kRec;
  };
  while (true) {
    {
      const unsigned long long t = claim_item(phase == kLaneIdle, work);
      if (phase == kLaneIdle) {
        k = k0 + (int64_t)t;
        if (k >= k1 || *(volatile int*)Q.overflow) {
          phase = kLaneDone;
        } else {
          const int64_t i = Q.vtx[k];
          if (A.lvl[i] < level) {  // labelled by an earlier batch of this group
            Q.alive[k] = 0;
            Q.len[k] = 0;
          } else {
            split_index(V, i, x, y, z);
            cur = {(float)x, (float)y, (float)z};
            iters = A.P.iteration_limit;
            anchor = cur;
            t_iters = iters;
            t_n = 0;
            last_nv = i;
            nb = 0;
            cnt = 1;
            e1 = 0;
            flushed = 0;
            endlab = kLabelNone;
            phase = kLaneEnter;
          }
        }
      }
    }
    if (__all_sync(kFullMask, phase == kLaneDone)) {
      add_trips(ntrips, trips);
      break;
    }
    for (int r = 0; r < K; r++) {
      if (phase != kLaneEnter && phase != kLaneStep) continue;
      const int64_t seen = last_nv;
      const int ev = A.advance(phase, x, y, z, cur, old, iters, nb_near, b, c, g, gm, step, slim, gm_end, last_nv,
                               ntrips);
      if (last_nv != seen) {  // the stop test passed a new vertex
        if (cnt == 1) e1 = (uint32_t)last_nv;
        else buf[nb++] = (uint32_t)last_nv;
        cnt++;
      }
      if (ev == EV_NONE) continue;
      A.nearest3(cur, x, y, z);
      if (ev == EV_HIT_PREASSIGNED) {
        // stopped by a vertex labelled before the batch: its label is the streamline's
        // (the vertex itself is not recorded, so every entry is a vertex unlabelled
        // before the batch)
        const int32_t l = lab[vid(V, x, y, z)];
        endlab = l == -1 ? kLabelNone : l;
      } else {
        mark_rec();
      }
      phase = ev == EV_OUT_OF_VOXEL ? kLaneEnter : kLaneEnd;
    }
    if (phase == kLaneStep && A.P.trap_window > 0 && t_iters - iters >= A.P.trap_window) {
      t_iters = iters;
      if (A.trapped(cur, anchor, t_n)) {  // ends where the iteration limit would have
        mark_rec();
        phase = kLaneEnd;
      }
    }
    // flush: an ended streamline writes the rest of its entries, a long one a full
    // segment (+ its link word); one pool and one holder-node allocation per warp and
    // turn.  A segment is flushed early only with an entry to spare (an ending marks the
    // last entry).
    const bool ending = phase == kLaneEnd;
    const int words = ending ? nb + (nb > kSeg ? 1 : 0) : (nb > kSeg ? kSeg + 1 : 0);
    const int nodes = ending ? nb + (cnt >= 2 ? 2 : 1) : (nb > kSeg ? kSeg : 0);  // entries flushed now
    int incl = words, nincl = nodes;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(kFullMask, incl, o);
      const int un = __shfl_up_sync(kFullMask, nincl, o);
      if (lane >= o) {
        incl += u;
        nincl += un;
      }
    }
    const int total = __shfl_sync(kFullMask, incl, 31), ntotal = __shfl_sync(kFullMask, nincl, 31);
    unsigned long long base = 0, nbase = 0;
    if (ntotal > 0) {
      if (lane == 31) {
        base = total > 0 ? atomicAdd(Q.cursor, (unsigned long long)total) : 0ull;
        nbase = atomicAdd(Q.ncursor, (unsigned long long)ntotal);
      }
      base = __shfl_sync(kFullMask, base, 31);
      nbase = __shfl_sync(kFullMask, nbase, 31);
      if (base + (unsigned long long)total > Q.pool_words || nbase + (unsigned long long)ntotal > Q.node_cap) {
        if (lane == 0) atomicExch(Q.overflow, 1);
        phase = kLaneDone;  // the batch is redone smaller; its results are discarded
        continue;
      }
    }
    // a recorded entry: its holder node (and, for a path vertex, the first round's claim)
    int32_t node = (int32_t)(nbase + (unsigned long long)(nincl - nodes));
    auto hold = [&](uint32_t u, int idx) {
      const uint32_t v = u & ~kRec;
      Q.hitem[node] = (int32_t)k;
      Q.hidx[node] = (uint32_t)idx | (u & kRec);
      Q.hnext[node] = atomicExch(&Q.hhead[v], node);
      node++;
      if (u & kRec) atomicMin(&claim[v], (uint32_t)k);
    };
    if (words > 0) {
      const uint32_t off = (uint32_t)(base + (unsigned long long)(incl - words));
      if (flushed == 0) Q.head[k] = off;
      else Q.pool[link] = off;
      const int seg = nb > kSeg ? kSeg : nb;  // entries of the segment written now
      for (int e = 0; e < seg; e++) {
        Q.pool[off + e] = buf[e];
        hold(buf[e], 2 + flushed + e);
      }
      if (ending) {
        if (nb > kSeg) {  // the rest follows the full segment's link word
          Q.pool[off + kSeg] = off + kSeg + 1;
          for (int e = kSeg; e < nb; e++) {
            Q.pool[off + 1 + e] = buf[e];
            hold(buf[e], 2 + flushed + e);
          }
        }
      } else {
        link = off + kSeg;
        flushed += kSeg;
        for (int e = kSeg; e < nb; e++) buf[e - kSeg] = buf[e];
        nb -= kSeg;
      }
    }
    if (ending) {
      hold((uint32_t)Q.vtx[k] | kRec, 0);
      if (cnt >= 2) hold(e1, 1);
      Q.e1[k] = e1;
      Q.len[k] = cnt;
      Q.endlab[k] = endlab;
      Q.alive[k] = 1;
      Q.cut[k] = -1;
      nb = 0;
      phase = kLaneIdle;
    }
  }
}

// After a pool overflow: the discarded batch's claims (on vertices not labelled yet) go.
__global__ void spec_unclaim_all_kernel(const uint8_t* __restrict__ lvl, int level, uint32_t* __restrict__ claim,
                                        int64_t N) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    if (lvl[i] >= level) claim[i] = kNoClaim;
}

// Effective extent (entries) of an item's path: none if skipped, up to its cut, or all.
__device__ __forceinline__ int spec_extent(uint8_t alive, int cut, int len) {
  return alive ? (cut >= 0 ? cut : len) : 0;
}

// Marks v dirty (bitmap + list, the list appends aggregated per warp); every lane of the
// warp calls it with its own `want`.
__device__ __forceinline__ void mark_dirty(bool want, uint32_t v, uint32_t* __restrict__ bits,
                                           uint32_t* __restrict__ list, unsigned long long* __restrict__ n_list) {
  bool add = false;
  if (want) {
    const uint32_t bit = 1u << (v & 31);
    add = !(atomicOr(&bits[v >> 5], bit) & bit);
  }
  const unsigned m = __ballot_sync(kFullMask, add);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  unsigned long long base = 0;
  if (lane == __ffs(m) - 1) base = atomicAdd(n_list, (unsigned long long)__popc(m));
  base = __shfl_sync(kFullMask, base, __ffs(m) - 1);
  if (add) list[base + __popc(m & ((1u << lane) - 1u))] = v;
}

// New alive / cut of item t of the batch (t < 0: none; every lane of the warp calls it)
// from the claims.  A changed item marks the path vertices between its old and new
// extent in nxt: their claims are recomputed next round.
__device__ __forceinline__ void check_item(const SpecSet& Q, int64_t k0, int64_t t, const uint32_t* __restrict__ claim,
                                           uint32_t* __restrict__ nxt, uint32_t* __restrict__ nxt_list,
                                           unsigned long long* __restrict__ n_nxt) {
  const int64_t k = k0 + (t >= 0 ? t : 0);
  const int n = t >= 0 ? Q.len[k] : 0;
  const bool look = n > 0;
  uint8_t oa = 0, na = 0;
  int oc = -1, nc = -1;
  bool changed = false;
  if (look) {
    const uint32_t kk = (uint32_t)k;
    oa = Q.alive[k];
    oc = Q.cut[k];
    na = claim[Q.vtx[k]] < kk ? 0 : 1;
    SeqWalk w(Q, k);
    w.next();
    for (int e = 1; e < n; e++) {
      const uint32_t v = w.next() & ~kRec;
      if (claim[v] < kk) {
        nc = e;
        break;
      }
    }
    changed = na != oa || nc != oc;
    if (changed) {
      Q.alive[k] = na;
      Q.cut[k] = nc;
    }
  }
  // the path vertices between the old and the new extent
  const int xo = changed ? spec_extent(oa, oc, n) : 0, xn = changed ? spec_extent(na, nc, n) : 0;
  const int lo = xo < xn ? xo : xn, hi = xo < xn ? xn : xo;
  int trips = hi;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) trips = max(trips, __shfl_xor_sync(kFullMask, trips, o));
  SeqWalk w(Q, k);
  for (int e = 0; e < trips; e++) {
    uint32_t u = 0;
    if (e < hi) u = w.next();
    mark_dirty(e >= lo && e < hi && (u & kRec), u & ~kRec, nxt, nxt_list, n_nxt);
  }
}

// A resolution round's items: every one of the batch (ibits == nullptr: the first
// round), or those whose bit is set in ibits (a bit per item from k0, ibits_words
// words), each bit cleared as it is taken so that the bitmap is clear again after the
// round.
__global__ void spec_check_kernel(const SpecSet Q, int64_t k0, int64_t k1, const uint32_t* __restrict__ claim,
                                  uint32_t* __restrict__ ibits, int64_t ibits_words, uint32_t* __restrict__ nxt,
                                  uint32_t* __restrict__ nxt_list, unsigned long long* __restrict__ n_nxt) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // every lane of a warp runs the same number of check_item calls (mark_dirty is warp-wide)
  if (!ibits) {
    const int64_t span = k1 - k0;
    for (int64_t t0 = blockIdx.x * (int64_t)blockDim.x; t0 < span; t0 += stride) {
      const int64_t t = t0 + threadIdx.x;
      check_item(Q, k0, t < span ? t : -1, claim, nxt, nxt_list, n_nxt);
    }
    return;
  }
  for (int64_t w0 = blockIdx.x * (int64_t)blockDim.x; w0 < ibits_words; w0 += stride) {
    const int64_t wd = w0 + threadIdx.x;
    uint32_t m = 0;
    if (wd < ibits_words) {
      m = ibits[wd];
      if (m) ibits[wd] = 0;
    }
    while (__any_sync(kFullMask, m != 0)) {
      int64_t t = -1;
      if (m) {
        t = wd * 32 + (__ffs(m) - 1);
        m &= m - 1;
      }
      check_item(Q, k0, t, claim, nxt, nxt_list, n_nxt);
    }
  }
}

// The claims of a round's dirty vertices from their holders' current extents, the
// holders marked in ibits for the round's check, and the vertices' dirty bits cleared
// (the bitmap takes the next-but-one round's marks).
__global__ void spec_reclaim_kernel(const SpecSet Q, int64_t k0, const uint32_t* __restrict__ list,
                                    const unsigned long long* __restrict__ n_list, uint32_t* __restrict__ bits,
                                    uint32_t* __restrict__ claim, uint32_t* __restrict__ ibits) {
  const unsigned long long n = *n_list;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const uint32_t v = list[i];
    atomicAnd(&bits[v >> 5], ~(1u << (v & 31)));
    uint32_t m = kNoClaim;
    for (int32_t h = Q.hhead[v]; h >= 0; h = Q.hnext[h]) {
      const int32_t k = Q.hitem[h];
      const int64_t t = k - k0;
      atomicOr(&ibits[t >> 5], 1u << (t & 31));
      const uint32_t ix = Q.hidx[h];
      if (!(ix & kRec)) continue;
      if ((int)(ix & ~kRec) < spec_extent(Q.alive[k], Q.cut[k], Q.len[k]) && (uint32_t)k < m) m = (uint32_t)k;
    }
    claim[v] = m;
  }
}

// ptr: the item whose label a cut item takes (the claimer of its stop vertex), or itself
__global__ void spec_ptr_kernel(const SpecSet Q, int64_t k0, int64_t k1, const uint32_t* __restrict__ claim) {
  for (int64_t k = k0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < k1; k += (int64_t)gridDim.x * blockDim.x) {
    if (!Q.alive[k]) continue;
    const int ct = Q.cut[k];
    int32_t p = (int32_t)k;
    if (ct >= 0) {
      SeqWalk w(Q, k);
      uint32_t u = 0;
      for (int e = 0; e <= ct; e++) u = w.next();
      p = (int32_t)claim[u & ~kRec];
    }
    Q.ptr[k] = p;
  }
}

__global__ void spec_jump_kernel(const SpecSet Q, int64_t k0, int64_t k1) {
  for (int64_t k = k0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < k1; k += (int64_t)gridDim.x * blockDim.x)
    if (Q.alive[k]) Q.ptr[k] = Q.ptr[Q.ptr[k]];
}

// Every claimed vertex takes its claimer's label (the label where the chain of cut
// items through ptr ends); the batch's vertices are stamped.  A chain longer than
// kChainSteps is left to pointer jumping: the item reports it in *long_chain and writes
// nothing.
constexpr int kChainSteps = 64;
__global__ void spec_write_kernel(const SpecSet Q, int64_t k0, int64_t k1, uint8_t* __restrict__ lvl, int level,
                                  const uint32_t* __restrict__ claim, int32_t* __restrict__ lab,
                                  int* __restrict__ long_chain) {
  for (int64_t k = k0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < k1; k += (int64_t)gridDim.x * blockDim.x) {
    if (!Q.alive[k]) continue;
    int32_t p = Q.ptr[k];
    for (int s = 0; s < kChainSteps; s++) {
      const int32_t q = Q.ptr[p];
      if (q == p) break;
      p = q;
    }
    if (Q.ptr[p] != p) {
      atomicExch(long_chain, 1);
      continue;
    }
    const int32_t d = Q.endlab[p];
    const int n = Q.cut[k] >= 0 ? Q.cut[k] : Q.len[k];
    SeqWalk w(Q, k);
    for (int e = 0; e < n; e++) {
      const uint32_t u = w.next();
      if (!(u & kRec)) continue;
      const uint32_t v = u & ~kRec;
      if (claim[v] == (uint32_t)k) {
        lab[v] = d;
        lvl[v] = (uint8_t)level;
      }
    }
  }
}

__global__ void init_levels_kernel(const int32_t* __restrict__ lab, uint8_t* __restrict__ lvl, int64_t N) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    lvl[i] = lab[i] == -1 ? 255 : 0;
}

// The vertices not labelled yet (lvl 255): 16 bytes a thread, one atomic per warp.
__global__ void count_unlabelled_kernel(const uint8_t* __restrict__ lvl, int64_t N,
                                        unsigned long long* __restrict__ n) {
  unsigned long long cnt = 0;
  const int64_t n16 = N / 16;
  const uint4* l4 = reinterpret_cast<const uint4*>(lvl);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += (int64_t)gridDim.x * blockDim.x) {
    const uint4 q = l4[i];
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int j = 0; j < 4; j++) {
      // bytes equal to 0xFF: all bits set
      uint32_t m = w[j] & (w[j] >> 1);
      m &= m >> 2;
      m &= m >> 4;
      cnt += __popc(m & 0x01010101u);
    }
  }
  for (int64_t i = n16 * 16 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x)
    cnt += lvl[i] == 255;
  add_trips(cnt, n);
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
  // The corner gradients are formed from the image where a voxel is entered, as
  // ComputeGradFromImage(1) forms them (gi_regular_grid_trilinear_function.h:285-341;
  // central_diff_kernel's f64 variant, the same operations), and are zero at the
  // vertices whose bit `zeroed` sets (SetGradExplicit at the seeds): the few FP64
  // streamlines do not need the gradient of every vertex stored in FP64.
  const float* f;
  const uint32_t* zeroed;
  VolDims V;
  IntegParams P;
  const uint8_t* state;  // fix-up stop: certain terminal

  __device__ __forceinline__ D3 corner(int64_t x, int64_t y, int64_t z) const {
    const int64_t v = vid(V, x, y, z);
    if ((zeroed[v >> 5] >> (v & 31)) & 1u) return {0.0, 0.0, 0.0};
    const float c = __ldg(f + v);
    // 0 + (-0.5f * f[-1]) + (0.0f * f[0]) + (0.5f * f[+1]), each product a float, summed
    // in double; 0 + (0.0f * f[0]) on a first or last plane
    auto comp = [&](bool inside, int64_t s) -> double {
      if (!inside) return 0.0 + (double)(0.0f * c);
      const float a = __ldg(f + v - s), b = __ldg(f + v + s);
      double r = 0.0;
      r += (double)(-0.5f * a);
      r += (double)(0.0f * c);
      r += (double)(0.5f * b);
      return r;
    };
    return {comp(x > 0 && x < V.X - 1, 1), comp(y > 0 && y < V.Y - 1, V.X), comp(z > 0 && z < V.Z - 1, V.X * V.Y)};
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
  __shared__ int s_part[kAppendWarps + 1];
  const int64_t N = V.X * V.Y * V.Z;
  const int lane = threadIdx.x & 31;
  // a warp covers 32 consecutive vertices starting at a multiple of 32 (block size and
  // grid stride are multiples of 32), i.e. exactly one word of `queued`; every thread of
  // a block makes the same number of trips (block_append)
  for (int64_t b0 = blockIdx.x * (int64_t)blockDim.x; b0 < N; b0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = b0 + threadIdx.x;
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
    const unsigned m = __ballot_sync(kFullMask, diff);
    if (lane == 0 && m) atomicOr(&queued[i >> 5], m);
    const int slot = block_append(diff ? 1 : 0, n, s_part);
    if (diff) list[slot] = i;
  }
}

// Fix-up streamlines (:340-392) in the reference's FP64 arithmetic: from each listed
// vertex, integrate until a certain terminal region (or a low gradient / the iteration
// limit); the streamline's final nearest vertex goes to endv.  The integration reads no
// labels, so where a vertex's streamline ends does not depend on the wave order.
template <int K>
__global__ void __launch_bounds__(32) fixup_end64_kernel(const Adv64 A, const int64_t* __restrict__ list, int n,
                                                         const int* __restrict__ n_dev, int32_t* __restrict__ endv,
                                                         unsigned long long* __restrict__ work,
                                                         unsigned long long* __restrict__ trips) {
  const VolDims& V = A.V;
  if (n_dev) n = *n_dev;  // a list whose length the stream wrote before this launch
  int phase = kLaneIdle;
  unsigned long long ntrips = 0;
  int64_t v = 0;
  int x = 0, y = 0, z = 0;
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
    endv[v] = (int32_t)vid(V, x, y, z);
  }
}

// Fix-up streamlines in FP32 (as fixup_end64_kernel).  A streamline whose FP32 ending
// is ambiguous goes to the FP64 list instead:
//   it stopped at a gradient magnitude within 2^-8 (relative) below the threshold
//   (the FP64 stop test decides), or
//   amb_mode 0: its final point lies within 1/64 voxel of the plane where the
//     nearest vertex changes, and the vertex across that plane belongs to a
//     different certain region (FP32 rounding may have picked the wrong side);
//   amb_mode 2: its final voxel touches two different certain regions (any ending
//     within half a voxel of a basin boundary).
template <int K>
__global__ void __launch_bounds__(128, 7) fixup_end32_kernel(const Adv32 A, const int32_t* __restrict__ lab,
                                                          const uint8_t* __restrict__ state,
                                                          const int64_t* __restrict__ list, int n,
                                                          const int* __restrict__ n_dev,
                                                          int32_t* __restrict__ endv, int64_t* __restrict__ amb,
                                                          int* __restrict__ n_amb, int amb_mode,
                                                          unsigned long long* __restrict__ work,
                                                          unsigned long long* __restrict__ trips) {
  const VolDims& V = A.V;
  if (n_dev) n = *n_dev;  // a list whose length the stream wrote before this launch
  int phase = kLaneIdle;
  unsigned long long ntrips = 0;
  int64_t v = 0;
  int x = 0, y = 0, z = 0;
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
    // a low-gradient stop whose FP32 magnitude lies within 2^-8 (relative) of the
    // threshold: FP32 rounding could have taken the other side of the stop test.  A
    // streamline that decelerates into an extremum crosses the threshold well inside
    // that test's FP32 accuracy otherwise, and FP64 would stop it at the same step.
    bool ambiguous = ev == EV_LOW_GRADIENT && gm_end >= A.P.gthresh * (1.f - 1.f / 256.f);
    if (!ambiguous && ev == EV_HIT_PREASSIGNED && amb_mode == 0) {
      const float pc[3] = {cur.x, cur.y, cur.z};
      const int64_t ext[3] = {V.X, V.Y, V.Z};
      const int64_t ev3[3] = {x, y, z};
      // the end is a certain terminal here, whose label no pass changes (the ends can
      // run beside the first pass, which writes the labels of uncertain vertices only)
      const int32_t le = lab[end];
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
        if ((st == kStSeed || st == kStTerminal) && lab[u] != le) ambiguous = true;
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
        const int32_t l = lab[u];
        if (seen == kLabelNone) seen = l;
        else if (l != seen) ambiguous = true;
      }
    }
    if (ambiguous) {
      amb[atomicAdd(n_amb, 1)] = v;
      continue;
    }
    endv[v] = (int32_t)end;
  }
}

// Every vertex that is not a certain terminal (seed or terminal region): the vertices a
// fix-up wave can hold, whose streamline ends are computed ahead of the waves.
__global__ void uncertain_list_kernel(const uint8_t* __restrict__ state, int64_t N, int64_t* __restrict__ list,
                                      int* __restrict__ n) {
  __shared__ int s_part[kAppendWarps + 1];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v0 = blockIdx.x * (int64_t)blockDim.x; v0 < N; v0 += stride) {
    const int64_t v = v0 + threadIdx.x;
    const bool want = v < N && state[v] != kStSeed && state[v] != kStTerminal;
    const int slot = block_append(want ? 1 : 0, n, s_part);
    if (want) list[slot] = v;
  }
}

// ---- fix-up waves (:316-415) ---------------------------------------------------------------
// The reference decides a wave's vertices one at a time in increasing id, each taking
// the label its streamline's final vertex carries at that moment: a certain terminal's
// region, or -- after a low-gradient stop or the iteration limit -- the current label of
// an ordinary vertex, which an earlier decision of the same wave may have changed.  The
// kernels below reproduce that order: a decision whose end vertex e is decided earlier
// in the same wave (e < v) takes e's new label (the chain of such ends followed), any
// other takes the label at the wave's start; a changed vertex reopens its neighbours
// that were undecided at its moment (never decided before the wave, and not earlier in
// it) and carry another label.

// A slot in a list whose length is *n for every lane of the warp that wants one (one
// atomic per warp); every lane must call it.  Returns -1 where `want` is false.
__device__ __forceinline__ int warp_append(bool want, int* n) {
  const unsigned m = __ballot_sync(kFullMask, want);
  if (!m) return -1;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(n, __popc(m));
  base = __shfl_sync(kFullMask, base, leader);
  return want ? base + __popc(m & ((1u << lane) - 1u)) : -1;
}

// wave w's members: stamp, clear their queued bit, list the ones without an end yet
__global__ void wave_mark_kernel(const int64_t* __restrict__ list, int n, int w, int32_t* __restrict__ inw,
                                 uint32_t* __restrict__ queued, const int32_t* __restrict__ endv,
                                 int64_t* __restrict__ todo, int* __restrict__ n_todo) {
  for (int k0 = blockIdx.x * blockDim.x; k0 < n; k0 += gridDim.x * blockDim.x) {  // warp-uniform trips
    const int k = k0 + threadIdx.x;
    int64_t v = -1;
    if (k < n) {
      v = list[k];
      inw[v] = w;
      atomicAnd(&queued[v >> 5], ~(1u << (v & 31)));
    }
    const int slot = warp_append(v >= 0 && endv[v] < 0, n_todo);
    if (slot >= 0) todo[slot] = v;
  }
}

__global__ void wave_root_kernel(const int64_t* __restrict__ list, int n, int w, const int32_t* __restrict__ endv,
                                 const int32_t* __restrict__ inw, const int32_t* __restrict__ lab,
                                 const uint8_t* __restrict__ state, int32_t* __restrict__ rptr,
                                 int32_t* __restrict__ rval) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int32_t v = (int32_t)list[k];
    const int32_t e = endv[v];
    const uint8_t st = state[e];
    if (st != kStSeed && st != kStTerminal && inw[e] == w && e < v) {
      rptr[v] = e;
    } else {
      rptr[v] = v;
      const int32_t l = lab[e];
      rval[v] = l == -1 ? kLabelNone : l;
    }
  }
}

__global__ void wave_jump_kernel(const int64_t* __restrict__ list, int n, int32_t* __restrict__ rptr) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int64_t v = list[k];
    rptr[v] = rptr[rptr[v]];
  }
}

// Each member's new label: the value where its chain of same-wave ends stops.  A chain
// longer than kChainSteps is left to pointer jumping (*long_chain is set).
constexpr int kWaveChainSteps = 64;
__global__ void wave_resolve_kernel(const int64_t* __restrict__ list, int n, const int32_t* __restrict__ rptr,
                                    const int32_t* __restrict__ rval, int32_t* __restrict__ rfin,
                                    int* __restrict__ long_chain) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int64_t v = list[k];
    int32_t p = rptr[v];
    for (int s = 0; s < kWaveChainSteps; s++) {
      const int32_t q = rptr[p];
      if (q == p) break;
      p = q;
    }
    if (rptr[p] != p) {
      atomicExch(long_chain, 1);
      continue;
    }
    rfin[v] = rval[p];
  }
}

__global__ void wave_enqueue_kernel(const int64_t* __restrict__ list, int n, int w, const VolDims V,
                                    const int32_t* __restrict__ rfin,
                                    const int32_t* __restrict__ lab, const uint8_t* __restrict__ state,
                                    const int32_t* __restrict__ inw, uint32_t* __restrict__ queued,
                                    int64_t* __restrict__ next, int* __restrict__ n_next) {
  __shared__ int s_part[kAppendWarps + 1];
  for (int k0 = blockIdx.x * blockDim.x; k0 < n; k0 += gridDim.x * blockDim.x) {  // block-uniform trips
    const int k = k0 + threadIdx.x;
    int64_t v = -1;
    int32_t nl = 0;
    if (k < n) {
      v = list[k];
      nl = rfin[v];
      if (nl == lab[v]) v = -1;  // unchanged: reopens nothing
    }
    int64_t nbr[6] = {-1, -1, -1, -1, -1, -1};
    if (v >= 0) {
      int vx, vy, vz;
      split_index(V, v, vx, vy, vz);
      nbr[0] = vx < V.X - 1 ? v + 1 : -1;
      nbr[1] = vx > 0 ? v - 1 : -1;
      nbr[2] = vy < V.Y - 1 ? v + V.X : -1;
      nbr[3] = vy > 0 ? v - V.X : -1;
      nbr[4] = vz < V.Z - 1 ? v + V.X * V.Y : -1;
      nbr[5] = vz > 0 ? v - V.X * V.Y : -1;
    }
    int cnt = 0;
#pragma unroll
    for (int j = 0; j < 6; j++) {
      const int64_t u = nbr[j];
      // (the inw test: u was decided before v in this wave)
      bool add = u >= 0 && state[u] == kStUnassigned && lab[u] != nl && !(inw[u] == w && u < v);
      if (add) {
        const uint32_t bit = 1u << (u & 31);
        add = !(atomicOr(&queued[u >> 5], bit) & bit);
      }
      if (!add) nbr[j] = -1;
      cnt += add;
    }
    int slot = block_append(cnt, n_next, s_part);
#pragma unroll
    for (int j = 0; j < 6; j++)
      if (nbr[j] >= 0) next[slot++] = nbr[j];
  }
}

__global__ void wave_apply_kernel(const int64_t* __restrict__ list, int n, const int32_t* __restrict__ rfin,
                                  int32_t* __restrict__ lab, uint8_t* __restrict__ state) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int64_t v = list[k];
    lab[v] = rfin[v];
    state[v] = kStNonterminal;
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

// MergeBoundaryExtrema (:108-145, the loop of :168-176): the reference visits the
// component roots in vertex order; a root with an earlier neighbour (in the comparer's
// order) lies in a component without its region's extremum, and joins -- in the union-
// find as it stands at that moment -- the current component of its earliest neighbour
// whose current component carries another label.  `first` holds every vertex's root
// of the same-label forest; md[r] the root r joined (r itself if none).  Only roots
// with an earlier neighbour decide anything; they are listed in `roots`.
__global__ void clean_roots_kernel(const int32_t* __restrict__ lab, const float* __restrict__ f, const VolDims V, int dir,
                                   const int32_t* __restrict__ first, int32_t* __restrict__ md,
                                   int32_t* __restrict__ roots, int* __restrict__ n_roots) {
  __shared__ int s_part[kAppendWarps + 1];
  const int64_t N = V.X * V.Y * V.Z;
  for (int64_t b0 = blockIdx.x * (int64_t)blockDim.x; b0 < N; b0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = b0 + threadIdx.x;  // (block-uniform trips: block_append)
    bool any = false;
    if (r < N) {
      md[r] = (int32_t)r;
      if (first[r] == r) {
        int x, y, z;
        split_index(V, r, x, y, z);
        const int64_t nbr[6] = {x < V.X - 1 ? r + 1 : -1, x > 0 ? r - 1 : -1, y < V.Y - 1 ? r + V.X : -1,
                                y > 0 ? r - V.X : -1, z < V.Z - 1 ? r + V.X * V.Y : -1,
                                z > 0 ? r - V.X * V.Y : -1};
        for (int j = 0; j < 6; j++) any |= nbr[j] >= 0 && comes_before(f, dir, nbr[j], r);
      }
    }
    const int slot = block_append(any ? 1 : 0, n_roots, s_part);
    if (any) roots[slot] = (int32_t)r;
  }
}

// The current root of x's component at root r's turn: joins made by roots visited
// before r (smaller ids) are followed.
__device__ __forceinline__ int32_t clean_current(const int32_t* md, int32_t x, int32_t r) {
  for (int guard = 0; guard < (1 << 20) && x < r; guard++) {
    const int32_t y = md[x];
    if (y == x) break;
    x = y;
  }
  return x;
}

// One relaxation sweep of the roots' decisions (each depends only on the decisions of
// smaller roots, so the sweeps reach the reference's sequential outcome; *changed
// counts the decisions that moved).
__global__ void clean_sweep_kernel(const int32_t* __restrict__ lab, const float* __restrict__ f, const VolDims V, int dir,
                                   const int32_t* __restrict__ first, int32_t* __restrict__ md,
                                   const int32_t* __restrict__ roots, const int* __restrict__ n_roots,
                                   int* __restrict__ changed) {
  const int n = *n_roots;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int32_t r = roots[k];
    int x, y, z;
    split_index(V, r, x, y, z);
    const int64_t nbr[6] = {x < V.X - 1 ? r + 1 : -1, x > 0 ? r - 1 : -1, y < V.Y - 1 ? r + V.X : -1,
                            y > 0 ? r - V.X : -1, z < V.Z - 1 ? r + V.X * V.Y : -1, z > 0 ? r - V.X * V.Y : -1};
    const int32_t reg = lab[r];
    int64_t earliest = r;
    for (int j = 0; j < 6; j++) {
      const int64_t u = nbr[j];
      if (u < 0 || !comes_before(f, dir, u, r)) continue;
      if (lab[clean_current(md, first[u], r)] == reg) continue;
      if (comes_before(f, dir, u, earliest)) earliest = u;
    }
    const int32_t t = earliest == r ? r : clean_current(md, first[earliest], r);
    if (md[r] != t) {
      md[r] = t;
      atomicAdd(changed, 1);
    }
  }
}

__global__ void clean_resolve_kernel(const int32_t* __restrict__ lab, const VolDims V, const int32_t* __restrict__ first,
                                     const int32_t* __restrict__ md, int32_t* __restrict__ out) {
  const int64_t N = V.X * V.Y * V.Z;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N; v += (int64_t)gridDim.x * blockDim.x) {
    int32_t r = first[v];
    for (int64_t guard = 0; guard < N && md[r] != r; guard++) r = md[r];
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
int lane_ctas_per_sm() {
  static const int k = [] {
    const char* e = std::getenv("MSC_LANE_CTAS_PER_SM");
    const int v = e ? std::atoi(e) : 0;
    return v >= 1 && v <= 32 ? v : 16;
  }();
  return k;
}
int trips_per_turn() {
  static const int k = trips_env("MSC_TRIPS_PER_TURN", 16);
  return k;
}
namespace {
int grid_for(int64_t n, int num_sms) {
  const int64_t blocks = (n + 255) / 256;
  return (int)(blocks < (int64_t)num_sms * 8 ? (blocks > 0 ? blocks : 1) : (int64_t)num_sms * 8);
}
}  // namespace

static int trips_per_turn_pass1() {
  static const int k = trips_env("MSC_TRIPS_PER_TURN_PASS1", trips_per_turn());
  return k;
}

cudaError_t launch_count_unlabelled(const uint8_t* lvl, int64_t N, unsigned long long* n, int num_sms,
                                    cudaStream_t stream) {
  if (cudaError_t e = cudaMemsetAsync(n, 0, sizeof(unsigned long long), stream)) return e;
  ::msc::count_launch();
  count_unlabelled_kernel<<<num_sms * 4, 256, 0, stream>>>(lvl, N, n);
  return cudaGetLastError();
}

cudaError_t launch_init_levels(const int32_t* lab, uint8_t* lvl, int64_t N, int num_sms, cudaStream_t stream) {
  ::msc::count_launch();
  init_levels_kernel<<<num_sms * 8, 256, 0, stream>>>(lab, lvl, N);
  return cudaGetLastError();
}

cudaError_t launch_spread_compact(const SpreadOrder& S, int64_t u0, int64_t u1, const uint8_t* lvl, int stamp,
                                  int* counts, int32_t* items, unsigned long long* n_items, cudaStream_t stream) {
  const int64_t nb = (u1 - u0 + kCompactBlock - 1) / kCompactBlock;
  if (nb <= 0 || nb > 0x7FFFFFFF) return cudaErrorInvalidValue;
  ::msc::count_launch();
  spread_count_kernel<<<(unsigned)nb, kCompactThreads, 0, stream>>>(S, u0, u1, lvl, stamp, counts);
  ::msc::count_launch();
  scan_counts_kernel<<<1, 1024, 0, stream>>>(counts, nb, n_items);
  ::msc::count_launch();
  spread_write_kernel<<<(unsigned)nb, kCompactThreads, 0, stream>>>(S, u0, u1, lvl, stamp, counts, items);
  return cudaGetLastError();
}

cudaError_t launch_speculate(const float4* G, const VolDims& V, const IntegParams& P, const SpecSet& Q, int64_t k0,
                             int64_t k1, const int32_t* lab, const uint8_t* lvl, int stamp, uint32_t* claim,
                             unsigned long long* work, unsigned long long* trips, int num_sms, cudaStream_t stream) {
  if (k1 <= k0) return cudaSuccess;
  const Adv32 A = Adv32::make(G, V, P, lvl, stamp, nullptr);
  const int64_t blocks = (k1 - k0 + 127) / 128;
  const int cap = num_sms * lane_ctas_per_sm();
  const int grid = (int)(blocks < cap ? blocks : cap);
  ::msc::count_launch();
  switch (trips_per_turn_pass1()) {
    case 2:
      speculate_kernel<2><<<grid, 128, 0, stream>>>(A, Q, k0, k1, lab, claim, work, trips);
      break;
    case 4:
      speculate_kernel<4><<<grid, 128, 0, stream>>>(A, Q, k0, k1, lab, claim, work, trips);
      break;
    case 8:
      speculate_kernel<8><<<grid, 128, 0, stream>>>(A, Q, k0, k1, lab, claim, work, trips);
      break;
    default:
      speculate_kernel<16><<<grid, 128, 0, stream>>>(A, Q, k0, k1, lab, claim, work, trips);
  }
  return cudaGetLastError();
}

cudaError_t launch_spec_round(const SpecSet& Q, int64_t k0, int64_t k1, uint32_t* claim, const SpecDirty* cur,
                              const SpecDirty& nxt, uint32_t* ibits, int64_t ibits_words, int num_sms,
                              cudaStream_t stream) {
  if (cudaError_t e = cudaMemsetAsync(nxt.n, 0, sizeof(unsigned long long), stream)) return e;
  // the first round's claims were made by the speculation, and it looks at every item
  if (!cur) {
    ::msc::count_launch();
    spec_check_kernel<<<grid_for(k1 - k0, num_sms), 256, 0, stream>>>(Q, k0, k1, claim, nullptr, 0, nxt.bits,
                                                                      nxt.list, nxt.n);
    return cudaGetLastError();
  }
  ::msc::count_launch();
  spec_reclaim_kernel<<<num_sms * 8, 256, 0, stream>>>(Q, k0, cur->list, cur->n, cur->bits, claim, ibits);
  ::msc::count_launch();
  spec_check_kernel<<<grid_for(ibits_words, num_sms), 256, 0, stream>>>(Q, k0, k1, claim, ibits, ibits_words,
                                                                        nxt.bits, nxt.list, nxt.n);
  return cudaGetLastError();
}

cudaError_t launch_spec_unclaim_all(const uint8_t* lvl, int stamp, uint32_t* claim, int64_t N, int num_sms,
                                    cudaStream_t stream) {
  ::msc::count_launch();
  spec_unclaim_all_kernel<<<num_sms * 8, 256, 0, stream>>>(lvl, stamp, claim, N);
  return cudaGetLastError();
}

cudaError_t launch_spec_ptr(const SpecSet& Q, int64_t k0, int64_t k1, const uint32_t* claim, int num_sms,
                            cudaStream_t stream) {
  ::msc::count_launch();
  spec_ptr_kernel<<<grid_for(k1 - k0, num_sms), 256, 0, stream>>>(Q, k0, k1, claim);
  return cudaGetLastError();
}

cudaError_t launch_spec_jumps(const SpecSet& Q, int64_t k0, int64_t k1, int num_sms, cudaStream_t stream) {
  // every chain of cut items ends at an uncut one within log2 steps
  int jumps = 1;
  for (int64_t n = k1 - k0; n > 1; n >>= 1) jumps++;
  for (int j = 0; j < jumps; j++) {
    ::msc::count_launch();
    spec_jump_kernel<<<grid_for(k1 - k0, num_sms), 256, 0, stream>>>(Q, k0, k1);
  }
  return cudaGetLastError();
}

cudaError_t launch_spec_write(const SpecSet& Q, int64_t k0, int64_t k1, uint8_t* lvl, int stamp, const uint32_t* claim,
                              int32_t* lab, int* long_chain, int num_sms, cudaStream_t stream) {
  ::msc::count_launch();
  spec_write_kernel<<<grid_for(k1 - k0, num_sms), 256, 0, stream>>>(Q, k0, k1, lvl, stamp, claim, lab, long_chain);
  return cudaGetLastError();
}

cudaError_t launch_boundary_set(const int32_t* lab, const uint8_t* state, const VolDims& V, int64_t* list, int* n,
                                uint32_t* queued, int num_sms, cudaStream_t stream) {
  ::msc::count_launch();
  boundary_set_kernel<<<num_sms * 8, 256, 0, stream>>>(lab, state, V, list, n, queued);
  return cudaGetLastError();
}

cudaError_t launch_fixup_end64(const float* f, const uint32_t* zeroed, const VolDims& V, const IntegParams& P,
                               const uint8_t* state,
                               const int64_t* list, int n, int32_t* endv, unsigned long long* work,
                               unsigned long long* trips, int num_sms, cudaStream_t stream, const int* n_dev) {
  if (n <= 0) return cudaSuccess;
  Adv64 A{f, zeroed, V, P, state};
  const int blocks = (n + 31) / 32;
  if (cudaError_t e = cudaMemsetAsync(work, 0, sizeof(unsigned long long), stream)) return e;
  ::msc::count_launch();
  // one-warp CTAs, at most four per SM: the FP64 re-decisions are few (~0.1% of the
  // re-decisions) and bound by each SM's FP64 pipe, which executes every warp
  // instruction in full however few lanes are active -- so a small wave is spread over
  // as many SMs as it has warps, and a large one keeps a few items per lane
  // iterations per turn: MSC_TRIPS_PER_TURN_FP64 (2, 4, 8 or 16) overrides the default
  static const int k = trips_env("MSC_TRIPS_PER_TURN_FP64", 2);
  const int grid = (blocks < num_sms * 4 && !n_dev) ? blocks : num_sms * 4;
  switch (k) {
    case 4:
      fixup_end64_kernel<4><<<grid, 32, 0, stream>>>(A, list, n, n_dev, endv, work, trips);
      break;
    case 16:
      fixup_end64_kernel<16><<<grid, 32, 0, stream>>>(A, list, n, n_dev, endv, work, trips);
      break;
    case 8:
      fixup_end64_kernel<8><<<grid, 32, 0, stream>>>(A, list, n, n_dev, endv, work, trips);
      break;
    default:
      fixup_end64_kernel<2><<<grid, 32, 0, stream>>>(A, list, n, n_dev, endv, work, trips);
  }
  return cudaGetLastError();
}

cudaError_t launch_uncertain_list(const uint8_t* state, int64_t N, int64_t* list, int* n, int num_sms,
                                  cudaStream_t stream) {
  ::msc::count_launch();
  uncertain_list_kernel<<<grid_for(N, num_sms), 256, 0, stream>>>(state, N, list, n);
  return cudaGetLastError();
}

cudaError_t launch_fixup_end32(const float4* G, const VolDims& V, const IntegParams& P, const int32_t* lab,
                               const uint8_t* state, const int64_t* list, int n, int32_t* endv, int64_t* amb,
                               int* n_amb, int amb_mode, unsigned long long* work, unsigned long long* trips,
                               int num_sms, cudaStream_t stream, const int* n_dev) {
  if (n <= 0) return cudaSuccess;
  const Adv32 A = Adv32::make(G, V, P, nullptr, 0, state);
  const int blocks = (n + 127) / 128;
  if (cudaError_t e = cudaMemsetAsync(work, 0, sizeof(unsigned long long), stream)) return e;
  ::msc::count_launch();
  // the ends computed beside the first pass leave it most CTA slots (MSC_EARLY_ENDS_CTAS
  // per SM, 1-16): at 512^3 both directions' labels took 486 / 500 / 526 / 524 ms with
  // 2 / 4 / 8 / 16, and 549 ms with the ends integrated per wave
  static const int early_ctas = [] {
    const char* e = std::getenv("MSC_EARLY_ENDS_CTAS");
    const int v = e ? std::atoi(e) : 2;
    return v >= 1 && v <= 16 ? v : 2;
  }();
  const int cap = num_sms * (n_dev ? early_ctas : lane_ctas_per_sm());
  const int grid = blocks < cap ? blocks : cap;
  switch (trips_per_turn()) {
    case 16:
      fixup_end32_kernel<16><<<grid, 128, 0, stream>>>(A, lab, state, list, n, n_dev, endv, amb, n_amb, amb_mode, work,
                                                          trips);
      break;
    case 2:
      fixup_end32_kernel<2><<<grid, 128, 0, stream>>>(A, lab, state, list, n, n_dev, endv, amb, n_amb, amb_mode, work,
                                                          trips);
      break;
    case 4:
      fixup_end32_kernel<4><<<grid, 128, 0, stream>>>(A, lab, state, list, n, n_dev, endv, amb, n_amb, amb_mode, work,
                                                          trips);
      break;
    default:
      fixup_end32_kernel<8><<<grid, 128, 0, stream>>>(A, lab, state, list, n, n_dev, endv, amb, n_amb, amb_mode, work,
                                                          trips);
  }
  return cudaGetLastError();
}

cudaError_t launch_wave_mark(const int64_t* list, int n, int w, int32_t* inw, uint32_t* queued, const int32_t* endv,
                             int64_t* todo, int* n_todo, int num_sms, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  ::msc::count_launch();
  wave_mark_kernel<<<grid_for(n, num_sms), 256, 0, stream>>>(list, n, w, inw, queued, endv, todo, n_todo);
  return cudaGetLastError();
}

cudaError_t launch_wave_resolve(const int64_t* list, int n, int w, const int32_t* endv, const int32_t* inw,
                                const int32_t* lab, const uint8_t* state, int32_t* rptr, int32_t* rval, int32_t* rfin,
                                int* long_chain, bool jump, int num_sms, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int grid = grid_for(n, num_sms);
  if (cudaError_t e = cudaMemsetAsync(long_chain, 0, sizeof(int), stream)) return e;
  if (!jump) {
    ::msc::count_launch();
    wave_root_kernel<<<grid, 256, 0, stream>>>(list, n, w, endv, inw, lab, state, rptr, rval);
  } else {
    int jumps = 1;
    for (int m = n; m > 1; m >>= 1) jumps++;
    for (int j = 0; j < jumps; j++) {
      ::msc::count_launch();
      wave_jump_kernel<<<grid, 256, 0, stream>>>(list, n, rptr);
    }
  }
  ::msc::count_launch();
  wave_resolve_kernel<<<grid, 256, 0, stream>>>(list, n, rptr, rval, rfin, long_chain);
  return cudaGetLastError();
}

cudaError_t launch_wave_finish(const int64_t* list, int n, int w, const VolDims& V, const int32_t* rfin,
                               const int32_t* inw, int32_t* lab, uint8_t* state, uint32_t* queued, int64_t* next,
                               int* n_next, int num_sms, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int grid = grid_for(n, num_sms);
  ::msc::count_launch();
  wave_enqueue_kernel<<<grid, 256, 0, stream>>>(list, n, w, V, rfin, lab, state, inw, queued, next, n_next);
  ::msc::count_launch();
  wave_apply_kernel<<<grid, 256, 0, stream>>>(list, n, rfin, lab, state);
  return cudaGetLastError();
}

cudaError_t launch_clean(const int32_t* lab, const float* f, const VolDims& V, int dir, int32_t* parent, int32_t* first,
                         int32_t* md, int32_t* roots, int* counters, int* pinned, int32_t* out, int num_sms,
                         cudaStream_t stream, int* sweeps_out) {
  const int64_t N = V.X * V.Y * V.Z;
  const int grid = num_sms * 8;
  ::msc::count_launch();
  uf_init_kernel<<<grid, 256, 0, stream>>>(parent, N);
  ::msc::count_launch();
  uf_hook_kernel<<<grid, 256, 0, stream>>>(lab, f, V, dir, parent);
  ::msc::count_launch();
  uf_roots_kernel<<<grid, 256, 0, stream>>>(parent, first, N);
  if (cudaError_t e = cudaMemsetAsync(counters, 0, 2 * sizeof(int), stream)) return e;
  ::msc::count_launch();
  clean_roots_kernel<<<grid, 256, 0, stream>>>(lab, f, V, dir, first, md, roots, counters);
  // sweeps until no decision moves (after sweep s the s smallest deciding roots are
  // final; in practice a few sweeps), the count read through `pinned`
  int sweeps = 0;
  for (;;) {
    if (cudaError_t e = cudaMemsetAsync(counters + 1, 0, sizeof(int), stream)) return e;
    ::msc::count_launch();
    clean_sweep_kernel<<<num_sms * 4, 256, 0, stream>>>(lab, f, V, dir, first, md, roots, counters, counters + 1);
    if (cudaError_t e = cudaMemcpyAsync(pinned, counters + 1, sizeof(int), cudaMemcpyDeviceToHost, stream)) return e;
    if (cudaError_t e = cudaStreamSynchronize(stream)) return e;
    sweeps++;
    if (*pinned == 0) break;
    if (sweeps > N + 1) return cudaErrorUnknown;
  }
  if (sweeps_out) *sweeps_out = sweeps;
  ::msc::count_launch();
  clean_resolve_kernel<<<grid, 256, 0, stream>>>(lab, V, first, md, out);
  return cudaGetLastError();
}

}  // namespace msc
