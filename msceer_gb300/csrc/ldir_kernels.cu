// K2: ascending-manifold dimension (the ldir bits of the .grad byte), sm_103a.
//
// Replaces TopologicalGradientUsingAlgorithms::setAscendingManifoldDimensions
// (gi_topological_gradient_using_algorithms.h:430-478) and its per-root queue walk
// rec_man_trace_up_marking (:395-425).  The reference marks, from every critical
// 1-cell, value 2 on everything reachable through "cofacet t, not critical, pair(t)
// != current, continue at pair(t)"; then value 1 from every critical 2-cell; then 0
// on critical 3-cells.  Items of the value-2 walk are edges (and hexes, which end
// it); the cells it marks as cofacets are quads, so the walk is a plain monotone
// reachability closure, independent of visiting order -- the reference's own
// output is thread-count invariant for the same reason.  Likewise for value 1
// (items quads, cofacets hexes).  K1 already wrote the roots (critical 1-cells = 2,
// critical 2-cells = 1, critical 3-cells = 0, everything else 3).
//
// GPU form: a tile kernel.  A CTA stages a tile of .grad bytes plus a 2-cell halo in
// shared memory (every rule reaches at most 2 cells), seeds a shared-memory queue
// with the marked items, runs the value-2 walk to its local fixpoint, then the
// value-1 walk, and writes back the tile.  Marks in the halo stay local.  Two ways
// finish the closure across tile borders:
//   single pass (default)  one tile pass saves the halo cells every tile lowered; a
//       check kernel lowers those cells in global memory where the owner holds them
//       higher and queues the lowered items; a walk kernel finishes their walks in
//       global memory.
//   multi pass (fallback, and the allocation-free entry)  repeated tile passes; later
//       passes revisit only tiles whose halo changed (a neighbour wrote a cell within
//       2 cells of the shared border) and seed only from the halo, because everything
//       reachable from the interior was already walked.  The closure is complete when
//       a pass changes no cell near any tile border.
#include "msc_device.cuh"

namespace msc {

template <int ND, int TX, int TY, int TZ>
struct LdirTile {
  static constexpr int H = 2;
  static constexpr int LX = TX + 2 * H;
  static constexpr int LY = TY + 2 * H;
  static constexpr int LZ = (ND == 3) ? TZ + 2 * H : 1;
  static constexpr int NL = LX * LY * LZ;
  static constexpr int ls(int a) { return a == 0 ? 1 : (a == 1 ? LX : LX * LY); }
  static constexpr int NW = (NL + 31) / 32;
  // dynamic shared memory of the pass kernel: queue (u16) | bytes | visited bits | changed bits
  static constexpr size_t smem_bytes() { return (size_t)NL * 2 + ((NL + 3) / 4) * 4 + (size_t)NW * 8; }
};

// local index -> local coords
template <class T>
__device__ __forceinline__ void lcoords(int i, int& lx, int& ly, int& lz) {
  lx = i % T::LX;
  ly = (i / T::LX) % T::LY;
  lz = i / (T::LX * T::LY);
}

// Queue append for the lanes of a warp that are converged here: one shared-memory
// atomic per warp instead of one per pushed item.
__device__ __forceinline__ void warp_push(uint16_t* sq, int* qtail, int cap, int* err, bool want, int item) {
  const unsigned act = __activemask();
  const unsigned m = __ballot_sync(act, want);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(qtail, __popc(m));
  base = __shfl_sync(act, base, leader);
  if (want) {
    const int slot = base + __popc(m & ((1u << lane) - 1u));
    if (slot < cap) sq[slot] = (uint16_t)item; else atomicOr(err, kErrLocalQueue);
  }
}

// Walk one item: visit its cofacets (CofacetsIterator order), mark them, follow their
// partners and queue the newly reached items.  All coordinates are local to the
// staged box, whose origin is even on every axis, so local parity is the cell's
// dimension parity.
template <class T, int ND>
struct LdirWalk {
  uint8_t* sg;
  uint16_t* sq;
  uint32_t* vis;
  uint32_t* dirty;
  int* qtail;
  int* err;
  int lmin[3], lmax[3];  // in-complex local range per axis
  uint32_t dec_map;

  __device__ __forceinline__ void touch(int c) {
    if (dirty) atomicOr(&dirty[c >> 5], 1u << (c & 31));
  }

  // returns the item to queue, or -1
  __device__ __forceinline__ int visit(int i, int l[3], int a, int sgn, int phase) {
    const unsigned value = phase == 0 ? 2u : 1u;
    constexpr int LE[3] = {T::LX, T::LY, T::LZ};
    const int la = l[a] + sgn;
    if (la < lmin[a] || la >= lmax[a]) return -1;
    const int t = i + sgn * T::ls(a);
    const uint8_t bt = sg[t];
    const unsigned code = (bt >> 2) & 7u;
    if (!(bt & 1u) || code == 7u) return -1;  // unassigned or critical
    if (phase == 0) {
      if ((bt >> 5) == 3u) { sg[t] = (uint8_t)((bt & 0x1Fu) | (2u << 5)); touch(t); }
    } else {
      if ((bt >> 5) != 1u) { sg[t] = (uint8_t)((bt & 0x1Fu) | (1u << 5)); touch(t); }
    }
    const int pc = map3(dec_map, (int)code);
    const int pa = pc >> 1, psg = (pc & 1) ? -1 : 1;
    int lp[3] = {l[0], l[1], l[2]};
    lp[a] += sgn;
    lp[pa] += psg;
    if (lp[pa] < 0 || lp[pa] >= LE[pa]) return -1;  // partner outside the box
    const int tp = t + psg * T::ls(pa);
    if (tp == i) return -1;
    const uint8_t bp = sg[tp];
    if (phase == 0) {
      if ((bp >> 5) != 3u) return -1;  // already marked: seeded or queued
      const int pdim = (lp[0] & 1) + (lp[1] & 1) + (ND == 3 ? (lp[2] & 1) : 0);
      if (pdim != 1) {  // a hex: the path ends here
        sg[tp] = (uint8_t)((bp & 0x1Fu) | (2u << 5));
        touch(tp);
        return -1;
      }
    } else {
      if ((bp >> 5) == 1u) return -1;
    }
    const uint32_t bit = 1u << (tp & 31);
    if (atomicOr(&vis[tp >> 5], bit) & bit) return -1;
    sg[tp] = (uint8_t)((bp & 0x1Fu) | (value << 5));
    touch(tp);
    return tp;
  }

  __device__ __forceinline__ void step(int i, int phase) {
    int l[3];
    lcoords<T>(i, l[0], l[1], l[2]);
#pragma unroll
    for (int a = 0; a < ND; a++) {
#pragma unroll
      for (int s = 0; s < 2; s++) {
        // cofacets only along even axes, +axis first
        const int nx = (l[a] & 1) ? -1 : visit(i, l, a, s == 0 ? 1 : -1, phase);
        warp_push(sq, qtail, T::NL, err, nx >= 0, nx);
      }
    }
  }
};

template <int ND, int TX, int TY, int TZ, int BS>
__global__ void __launch_bounds__(BS) ldir_pass_kernel(uint8_t* __restrict__ g, const GradDims D,
                                                       const uint8_t* __restrict__ dirty_in,
                                                       uint8_t* __restrict__ dirty_out,
                                                       int* __restrict__ changed, int* __restrict__ err) {
  using T = LdirTile<ND, TX, TY, TZ>;
  constexpr int NL = T::NL;
  static_assert(NL < 65536, "local ids are 16-bit");
  static_assert(TX % 2 == 0 && TY % 2 == 0 && (ND == 2 || TZ % 2 == 0) && T::H % 2 == 0, "box origins must be even");
  extern __shared__ __align__(16) unsigned char s_dyn[];
  uint16_t* sq = reinterpret_cast<uint16_t*>(s_dyn);
  uint8_t* sg = s_dyn + (size_t)NL * 2;
  uint32_t* s_vis = reinterpret_cast<uint32_t*>(s_dyn + (size_t)NL * 2 + ((NL + 3) / 4) * 4);
  uint32_t* s_dirty = s_vis + T::NW;
  __shared__ int s_qtail, s_qseed, s_border;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NWARPS = BS / 32;
  const int64_t dX = D.d[0], dY = D.d[1], dZ = D.d[2];
  const int64_t ntx = (dX + TX - 1) / TX, nty = (dY + TY - 1) / TY;
  const int64_t ntz = (ND == 3) ? (dZ + TZ - 1) / TZ : 1;
  const int64_t ntiles = ntx * nty * ntz;
  const bool first = (dirty_in == nullptr);

  LdirWalk<T, ND> W;
  W.sg = sg;
  W.sq = sq;
  W.vis = s_vis;
  W.dirty = s_dirty;
  W.qtail = &s_qtail;
  W.err = err;
  W.dec_map = D.dec_map;

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    if (!first && !dirty_in[tile]) continue;
    const int64_t tx = tile % ntx, ty = (tile / ntx) % nty, tz = (ND == 3) ? tile / (ntx * nty) : 0;
    const int64_t o[3] = {tx * TX - T::H, ty * TY - T::H, (ND == 3) ? tz * TZ - T::H : 0};
    const int64_t dd[3] = {dX, dY, dZ};
    constexpr int LE[3] = {T::LX, T::LY, T::LZ};
#pragma unroll
    for (int a = 0; a < 3; a++) {
      W.lmin[a] = (int)(o[a] < 0 ? -o[a] : 0);
      const int64_t hi = dd[a] - o[a];
      W.lmax[a] = (int)(hi < LE[a] ? hi : LE[a]);
    }
    if (tid == 0) {
      s_qtail = 0;
      s_qseed = NL;
      s_border = 0;
    }
    for (int w = tid; w < T::NW; w += BS) {
      s_vis[w] = 0;
      s_dirty[w] = 0;
    }
    __syncthreads();

    // stage the box row by row (cells outside the complex read as 0 = unassigned)
    // and collect the seeds: marked items of both walks (first pass), or of the
    // halo only (later passes: the interior was walked already).  Seeds need no
    // visited bit: being marked already stops a walk from queueing them again.
    constexpr int RPW = 4;  // rows per warp in flight
    for (int row0 = warp * RPW; row0 < T::LY * T::LZ; row0 += NWARPS * RPW) {
      uint8_t b[RPW][(T::LX + 31) / 32];
#pragma unroll
      for (int r = 0; r < RPW; r++) {
        const int row = row0 + r;
        const int ly = row % T::LY, lz = row / T::LY;
        const bool rin = row < T::LY * T::LZ && ly >= W.lmin[1] && ly < W.lmax[1] && lz >= W.lmin[2] && lz < W.lmax[2];
        const uint8_t* grow = g + ((o[1] + ly) * D.cs[1] + (o[2] + lz) * D.cs[2] + o[0]);
#pragma unroll
        for (int c = 0; c < (T::LX + 31) / 32; c++) {
          const int lx = lane + 32 * c;
          b[r][c] = (rin && lx < T::LX && lx >= W.lmin[0] && lx < W.lmax[0]) ? grow[lx] : (uint8_t)0;
        }
      }
#pragma unroll
      for (int r = 0; r < RPW; r++) {
        const int row = row0 + r;
        if (row >= T::LY * T::LZ) break;
        const int ly = row % T::LY, lz = row / T::LY;
        const bool row_halo = ly < T::H || ly >= T::H + TY || (ND == 3 && (lz < T::H || lz >= T::H + TZ));
#pragma unroll
        for (int c = 0; c < (T::LX + 31) / 32; c++) {
          const int lx = lane + 32 * c;
          const int i = lx + T::LX * row;
          const uint8_t v = b[r][c];
          if (lx < T::LX) sg[i] = v;
          const unsigned ld = v >> 5;
          const int dim = (lx & 1) + (ly & 1) + (ND == 3 ? (lz & 1) : 0);
          const bool keep = lx < T::LX && (v & 1u) && (first || row_halo || lx < T::H || lx >= T::H + TX);
          const bool s0 = keep && dim == 1 && ld == 2u;
          const bool s1 = keep && dim == 2 && ld == 1u;
          warp_push(sq, &s_qtail, NL, err, s0, i);
          // value-1 seeds grow down from the top of the queue
          const unsigned m1 = __ballot_sync(0xffffffffu, s1);
          if (m1) {
            int base = 0;
            if (lane == 0) base = atomicSub(&s_qseed, __popc(m1));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (s1) sq[base - 1 - __popc(m1 & ((1u << lane) - 1u))] = (uint16_t)i;
          }
        }
      }
    }
    __syncthreads();

    // value-2 walk, then value-1 walk, level by level
#pragma unroll 1
    for (int phase = 0; phase < 2; phase++) {
      int lo = phase == 0 ? 0 : s_qseed;
      int hi = phase == 0 ? s_qtail : NL;
      if (phase == 1) {
        __syncthreads();
        for (int w = tid; w < T::NW; w += BS) s_vis[w] = 0;
        if (tid == 0) s_qtail = 0;
        __syncthreads();
      }
#pragma unroll 1
      while (lo < hi) {
        for (int k0 = lo; k0 < hi; k0 += BS) {
          const int k = k0 + tid;
          if (k < hi) W.step(sq[k], phase);
        }
        __syncthreads();
        // the first value-1 level came from the seed region; later levels from 0
        const int nlo = (phase == 1 && hi == NL) ? 0 : hi;
        const int nhi = s_qtail;
        __syncthreads();
        lo = nlo;
        hi = nhi;
      }
    }
    __syncthreads();

    // write back the changed interior cells
    for (int w = tid; w < T::NW; w += BS) {
      uint32_t m = s_dirty[w];
      while (m) {
        const int i = w * 32 + __ffs(m) - 1;
        m &= m - 1;
        int lx, ly, lz;
        lcoords<T>(i, lx, ly, lz);
        if (lx < T::H || lx >= T::H + TX || ly < T::H || ly >= T::H + TY) continue;
        if (ND == 3 && (lz < T::H || lz >= T::H + TZ)) continue;
        g[(o[0] + lx) + (o[1] + ly) * D.cs[1] + (o[2] + lz) * D.cs[2]] = sg[i];
        // a change within reach (2 cells) of a neighbour's halo reopens that neighbour
        if (lx < 2 * T::H || lx >= TX || ly < 2 * T::H || ly >= TY || (ND == 3 && (lz < 2 * T::H || lz >= TZ)))
          s_border = 1;
      }
    }
    __syncthreads();
    if (s_border) {
      const int nn = (ND == 3) ? 27 : 9;
      for (int k = tid; k < nn; k += BS) {
        const int64_t nx = tx + (k % 3) - 1, ny = ty + (k / 3) % 3 - 1, nz = (ND == 3) ? tz + k / 9 - 1 : 0;
        if (k == nn / 2 || nx < 0 || nx >= ntx || ny < 0 || ny >= nty || nz < 0 || nz >= ntz) continue;
        dirty_out[nx + ny * ntx + nz * ntx * nty] = 1;
      }
      if (tid == 0) atomicOr(changed, 1);
    }
    __syncthreads();
  }
}

// ---- single-pass form: one bit-row tile pass, a halo check, a global frontier walk -----------
//
// A tile's walk is complete for every item of its interior (all of an item's rule
// reaches lies within 2 cells), so after one pass over all tiles the only missing
// marks are those a tile made in its halo that the halo's owner did not make itself.
// The pass records, per tile, the halo cells its closure holds lower than the .grad
// held them; the check kernel lowers every such cell that its owner still holds
// higher and queues the lowered items, whose walks may continue beyond that tile's
// box; the walk kernel finishes those walks in global memory.  Concurrent lowering of
// a byte uses a compare-and-swap on its aligned 32-bit word (the low five bits never
// change, so the ldir field only ever decreases); bytes whose word is not wholly
// inside the .grad array go through a bounded spin lock instead.

struct GradView {
  uint8_t* g;
  uintptr_t lo, hi;  // [first, last) byte address of the array
  int* lock;
  int* err;
};

// ldir(c) = min(ldir(c), val); true if this call lowered it
__device__ __forceinline__ bool lower_ldir(const GradView& G, int64_t c, unsigned val) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(G.g + c);
  const uintptr_t wa = a & ~uintptr_t(3);
  if (wa >= G.lo && wa + 4 <= G.hi) {
    uint32_t* w = reinterpret_cast<uint32_t*>(wa);
    const int sh = (int)(a & 3u) * 8;
    uint32_t cur = *reinterpret_cast<volatile uint32_t*>(w);
    for (int guard = 0; guard < 64; guard++) {
      const uint32_t b = (cur >> sh) & 0xFFu;
      if ((b >> 5) <= val) return false;
      const uint32_t nb = (b & 0x1Fu) | (val << 5);
      const uint32_t nw = (cur & ~(0xFFu << sh)) | (nb << sh);
      const uint32_t prev = atomicCAS(w, cur, nw);
      if (prev == cur) return true;
      cur = prev;
    }
    atomicOr(G.err, kErrPassLimit);
    return false;
  }
  // a word that reaches outside the array: serialise on the lock
  bool got = false;
  for (int guard = 0; guard < (1 << 20) && !got; guard++) got = atomicCAS(G.lock, 0, 1) == 0;
  if (!got) {
    atomicOr(G.err, kErrPassLimit);
    return false;
  }
  __threadfence();
  volatile uint8_t* p = G.g + c;
  const uint8_t b = *p;
  const bool lowered = (unsigned)(b >> 5) > val;
  if (lowered) *p = (uint8_t)((b & 0x1Fu) | (val << 5));
  __threadfence();
  atomicExch(G.lock, 0);
  return lowered;
}

__device__ __forceinline__ int batch_volume(const LdirBatch& B, int64_t flat_tile) {
  int lo = 0, hi = B.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (B.v[mid].tile0 <= flat_tile) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// The tile pass works on bit rows.  A box is 32 cells along x (28 owned plus the
// 2-cell halo on each side) by LY x LZ rows, and every per-cell property the walks
// need is one 32-bit word per row (bit = x offset in the box).  Both closures advance
// one BFS level at a time over every row at once:
//   T = NC & cof(F)     cofacets of the frontier along its even axes: bit shifts within
//                       a row for x, the neighbour rows for y and z
//   P = partner(T)      for each pair direction, T & PC[direction] moved one cell
//   value 2 marks the quads of T, the hexes of P and the new edges of P
//   value 1 marks the hexes of T and the new quads of P
// The frontier F is the new edges (value-2 items) and quads (value-1 items): the two
// walks' items, cofacets and partners never share a dimension, so one frontier and
// one partner step serve both.  Visiting order does not change a monotone closure, so
// the marks equal those of the item-by-item walk.  The closures of rough fields are
// shallow (14 levels for value 2, 12 for value 1 over a whole 128^3 k^-3 volume), so
// a tile costs a few dozen passes over its rows.
constexpr int kBitLX = 32;
template <int ND, int LY, int LZ>
struct BitTile {
  static constexpr int TX = kBitLX - 4, TY = LY - 4, TZ = ND == 3 ? LZ - 4 : 1;
  static constexpr int R = LY * LZ;  // rows of the box
  // halo rows (every cell in the halo) and inner rows (halo cells at x = 0, 1, 30, 31)
  static constexpr int NHR = ND == 3 ? 4 * LY + 4 * (LZ - 4) : 4;
  static constexpr int NIR = ND == 3 ? (LY - 4) * (LZ - 4) : LY - 4;
  // a tile's record: the {value 2, value 1} masks of each halo row's lowered cells,
  // then one byte per inner row (bits 0-3: value 2 at x = 0, 1, 30, 31; 4-7: value 1)
  static constexpr int64_t REC = ((int64_t)NHR * 8 + NIR + 15) / 16 * 16;
  // shared memory word planes: NC, PC[6] (partner at +x, -x, +y, -y, +z, -z), F, T, M2, M1
  static constexpr size_t smem_bytes() { return (size_t)11 * R * 4; }
  static_assert(ND == 3 || LZ == 1, "2D boxes have one z row");
  static_assert(LY % 2 == 0 && LZ % 2 == (ND == 3 ? 0 : 1), "tile origins must be even");
};

// record slot of halo row (ly, lz); -1 for an inner row
template <int ND, int LY, int LZ>
__device__ __forceinline__ int halo_row_slot(int ly, int lz) {
  if (ND == 3) {
    if (lz < 2) return lz * LY + ly;
    if (lz >= LZ - 2) return (lz - (LZ - 4)) * LY + ly;
  }
  const int base = ND == 3 ? 4 * LY + (lz - 2) * 4 : 0;
  if (ly < 2) return base + ly;
  if (ly >= LY - 2) return base + ly - (LY - 4);
  return -1;
}

template <int ND, int LY, int LZ>
__device__ __forceinline__ void halo_row_of(int h, int& ly, int& lz) {
  if (ND == 3 && h < 4 * LY) {
    const int s = h / LY;
    lz = s < 2 ? s : LZ - 4 + s;
    ly = h % LY;
    return;
  }
  const int k = ND == 3 ? h - 4 * LY : h;
  const int q = k & 3;
  lz = ND == 3 ? 2 + (k >> 2) : 0;
  ly = q < 2 ? q : LY - 4 + q;
}

template <int ND, int LY, int LZ, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) ldir_tile_kernel(const LdirBatch B, uint8_t* __restrict__ rec,
                                                       int* __restrict__ err) {
  using T = BitTile<ND, LY, LZ>;
  constexpr int R = T::R;
  constexpr int NWARP = BS / 32;
  constexpr int RPT = (R + BS - 1) / BS;  // rows per thread in a level
  constexpr int KR = 4;                   // rows per warp with loads in flight
  constexpr uint32_t EVENX = 0x55555555u, ODDX = 0xAAAAAAAAu;
  extern __shared__ __align__(16) uint32_t s_plane[];
  uint32_t* sNC = s_plane;
  uint32_t* sPC = s_plane + R;
  uint32_t* sF = s_plane + 7 * R;
  uint32_t* sT = s_plane + 8 * R;
  uint32_t* sM2 = s_plane + 9 * R;
  uint32_t* sM1 = s_plane + 10 * R;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  for (int64_t flat = blockIdx.x; flat < B.total_tiles; flat += gridDim.x) {
    const LdirVol& vol = B.v[batch_volume(B, flat)];
    uint8_t* __restrict__ g = vol.g;
    const GradDims& D = vol.D;
    const int64_t dX = D.d[0], dY = D.d[1], dZ = D.d[2];
    const int64_t ntx = (dX + T::TX - 1) / T::TX, nty = (dY + T::TY - 1) / T::TY;
    const int64_t tile = flat - vol.tile0;
    const int64_t tx = tile % ntx, ty = (tile / ntx) % nty, tz = ND == 3 ? tile / (ntx * nty) : 0;
    const int64_t o1 = ty * T::TY - 2, o2 = ND == 3 ? tz * T::TZ - 2 : 0;
    const int64_t gx = tx * T::TX - 2 + lane;
    const bool xin = gx >= 0 && gx < dX;

    // stage: a warp per row, a lane per cell; each property becomes a bit row.  Cells
    // outside the complex read as 0 (unassigned).  Marked items seed the frontier.  A
    // warp keeps KR rows' loads in flight before it folds them.
    for (int r0 = warp; r0 < R; r0 += NWARP * KR) {
      uint8_t bk[KR];
#pragma unroll
      for (int k = 0; k < KR; k++) {
        const int r = r0 + k * NWARP;
        const int ly = r % LY, lz = r / LY;
        const int64_t gy = o1 + ly, gz = o2 + lz;
        bk[k] = 0;
        if (r < R && xin && gy >= 0 && gy < dY && gz >= 0 && gz < dZ) bk[k] = g[gx + gy * D.cs[1] + gz * D.cs[2]];
      }
#pragma unroll
      for (int k = 0; k < KR; k++) {
        const int r = r0 + k * NWARP;
        if (r >= R) break;
        const int ly = r % LY, lz = r / LY;
        const uint8_t b = bk[k];
        const unsigned code = (b >> 2) & 7u, ld = b >> 5;
        const bool asg = b & 1u;
        const bool nc = asg && code != 7u;
        const int pc = nc ? map3(D.dec_map, (int)code) : 7;
        const int dim = (lane & 1) + (ly & 1) + (lz & 1);
        const uint32_t mnc = __ballot_sync(~0u, nc);
        const uint32_t m2 = __ballot_sync(~0u, asg && dim == 1 && ld == 2u);
        const uint32_t m1 = __ballot_sync(~0u, asg && dim == 2 && ld == 1u);
        uint32_t pcm[6];
#pragma unroll
        for (int c = 0; c < 6; c++) pcm[c] = __ballot_sync(~0u, pc == c);
        if (lane == 0) {
          sNC[r] = mnc;
#pragma unroll
          for (int c = 0; c < 6; c++) sPC[c * R + r] = pcm[c];
          sF[r] = m2 | m1;
          sM2[r] = m2;
          sM1[r] = m1;
        }
      }
    }
    __syncthreads();

    // BFS levels until no row gains an item; every level adds an item, so the bound
    // is never reached by a valid gradient
    for (int level = 0;; level++) {
#pragma unroll 1
      for (int k = 0; k < RPT; k++) {
        const int r = tid + k * BS;
        if (r < R) {
          const int ly = r % LY, lz = r / LY;
          const uint32_t f = sF[r] & EVENX;
          uint32_t c = (f << 1) | (f >> 1);
          if (ly & 1) c |= sF[r - 1] | (ly + 1 < LY ? sF[r + 1] : 0u);
          if (ND == 3 && (lz & 1)) c |= sF[r - LY] | (lz + 1 < LZ ? sF[r + LY] : 0u);
          sT[r] = c & sNC[r];
        }
      }
      __syncthreads();
      int grew = 0;
#pragma unroll 1
      for (int k = 0; k < RPT; k++) {
        const int r = tid + k * BS;
        if (r < R) {
          const int ly = r % LY, lz = r / LY;
          const uint32_t t = sT[r];
          uint32_t p = ((t & sPC[r]) << 1) | ((t & sPC[R + r]) >> 1);
          if (ly > 0) p |= sT[r - 1] & sPC[2 * R + r - 1];
          if (ly + 1 < LY) p |= sT[r + 1] & sPC[3 * R + r + 1];
          if (ND == 3) {
            if (lz > 0) p |= sT[r - LY] & sPC[4 * R + r - LY];
            if (lz + 1 < LZ) p |= sT[r + LY] & sPC[5 * R + r + LY];
          }
          const int odd = (ly & 1) + (lz & 1);
          const uint32_t edges = odd == 0 ? ODDX : (odd == 1 ? EVENX : 0u);
          const uint32_t quads = odd == 0 ? 0u : (odd == 1 ? ODDX : EVENX);
          const uint32_t hexes = odd == 2 ? ODDX : 0u;
          const uint32_t m2 = sM2[r], m1 = sM1[r];
          const uint32_t e2 = p & edges & ~m2, e1 = p & quads & ~m1;
          sM2[r] = m2 | (t & quads) | (p & hexes) | e2;
          sM1[r] = m1 | (t & hexes) | e1;
          sF[r] = e2 | e1;
          grew |= (e2 | e1) != 0u;
        }
      }
      if (!__syncthreads_or(grew)) break;
      if (level > 64 * R) {
        if (tid == 0) atomicOr(err, kErrPassLimit);
        break;
      }
    }

    // write back the owned cells this tile lowered and record the halo cells it holds
    // lower than the .grad does (their owners may hold them lower by now: the check
    // compares again)
    uint8_t* trec = rec + flat * T::REC;
    for (int r0 = warp; r0 < R; r0 += NWARP * KR) {
      uint8_t bk[KR];
      bool m2k[KR], m1k[KR];
#pragma unroll
      for (int k = 0; k < KR; k++) {
        const int r = r0 + k * NWARP;
        const int ly = r % LY, lz = r / LY;
        const int64_t gy = o1 + ly, gz = o2 + lz;
        m2k[k] = r < R && ((sM2[r] >> lane) & 1u);
        m1k[k] = r < R && ((sM1[r] >> lane) & 1u);
        bk[k] = 0;
        if ((m2k[k] || m1k[k]) && xin && gy >= 0 && gy < dY && gz >= 0 && gz < dZ)
          bk[k] = g[gx + gy * D.cs[1] + gz * D.cs[2]];
      }
#pragma unroll
      for (int k = 0; k < KR; k++) {
        const int r = r0 + k * NWARP;
        if (r >= R) break;
        const int ly = r % LY, lz = r / LY;
        const int64_t gy = o1 + ly, gz = o2 + lz;
        const uint8_t b = bk[k];  // 0 (unassigned) outside the complex
        const bool low2 = m2k[k] && (b & 1u) && (b >> 5) > 2u;
        const bool low1 = m1k[k] && (b & 1u) && (b >> 5) > 1u;
        const int slot = halo_row_slot<ND, LY, LZ>(ly, lz);
        if (slot >= 0) {
          const uint32_t w2 = __ballot_sync(~0u, low2), w1 = __ballot_sync(~0u, low1);
          if (lane < 2) reinterpret_cast<uint32_t*>(trec)[2 * slot + lane] = lane == 0 ? w2 : w1;
        } else {
          const bool own = lane >= 2 && lane < kBitLX - 2;
          if (own && (low2 || low1))
            g[gx + gy * D.cs[1] + gz * D.cs[2]] = (uint8_t)((b & 0x1Fu) | ((low1 ? 1u : 2u) << 5));
          const uint32_t w2 = __ballot_sync(~0u, low2 && !own), w1 = __ballot_sync(~0u, low1 && !own);
          if (lane == 0) {
            const int i = ND == 3 ? (lz - 2) * (LY - 4) + (ly - 2) : ly - 2;
            const uint32_t q2 = (w2 & 3u) | ((w2 >> 28) & 0xCu), q1 = (w1 & 3u) | ((w1 >> 28) & 0xCu);
            trec[T::NHR * 8 + i] = (uint8_t)(q2 | (q1 << 4));
          }
        }
      }
    }
    __syncthreads();
  }
}

__device__ __forceinline__ void push_item(int64_t* q, int* n, int cap, int* err, int64_t c) {
  const int slot = atomicAdd(n, 1);
  if (slot < cap) q[slot] = c; else atomicOr(err, kErrLocalQueue);
}

// frontier entries carry their volume above the cell id (bits 57-62, so entries stay
// non-negative for every volume index below kMaxBatch = 64)
constexpr int kVolShift = 57;
constexpr int64_t kCellMask = ((int64_t)1 << kVolShift) - 1;
static_assert(kMaxBatch <= 64, "six volume bits");
__device__ __forceinline__ int entry_volume(int64_t e) { return (int)((uint64_t)e >> kVolShift); }

__device__ __forceinline__ GradView volume_view(const LdirVol& v, int* lock, int* err) {
  return GradView{v.g, reinterpret_cast<uintptr_t>(v.g), reinterpret_cast<uintptr_t>(v.g + v.D.ncells), lock, err};
}

// A tile's box origin and volume, found once per record unit by the whole warp.
struct TileAt {
  int vi;
  int64_t o[3];
};
template <int ND, int LY, int LZ>
__device__ __forceinline__ TileAt tile_at(const LdirBatch& B, int64_t flat) {
  using T = BitTile<ND, LY, LZ>;
  TileAt t;
  t.vi = batch_volume(B, flat);
  const LdirVol& vol = B.v[t.vi];
  const int64_t ntx = (vol.D.d[0] + T::TX - 1) / T::TX, nty = (vol.D.d[1] + T::TY - 1) / T::TY;
  const int64_t tile = flat - vol.tile0;
  int64_t tx, ty, tz;
  if (tile < ((int64_t)1 << 32)) {  // 32-bit division (tile counts of real volumes)
    const uint32_t u = (uint32_t)tile, nx = (uint32_t)ntx, ny = (uint32_t)nty;
    const uint32_t r = u / nx;
    tx = u - r * nx;
    ty = ND == 3 ? r % ny : r;
    tz = ND == 3 ? r / ny : 0;
  } else {
    const int64_t r = tile / ntx;
    tx = tile - r * ntx;
    ty = ND == 3 ? r % nty : r;
    tz = ND == 3 ? r / nty : 0;
  }
  t.o[0] = tx * T::TX - 2;
  t.o[1] = ty * T::TY - 2;
  t.o[2] = ND == 3 ? tz * T::TZ - 2 : 0;
  return t;
}

// Lower one recorded halo cell (box coords lx, ly, lz) in its owner's .grad where the
// owner holds it higher, and queue it when it became an item.
__device__ __forceinline__ void check_cell(const LdirBatch& B, const TileAt& t, int lx, int ly, int lz, unsigned v,
                                           int64_t* queue, int* n_queue, int cap, int* lock, int* err) {
  const LdirVol& vol = B.v[t.vi];
  const int64_t gx = t.o[0] + lx, gy = t.o[1] + ly, gz = t.o[2] + lz;
  const int64_t c = gx + gy * vol.D.cs[1] + gz * vol.D.cs[2];
  if ((unsigned)(vol.g[c] >> 5) <= v) return;
  if (!lower_ldir(volume_view(vol, lock, err), c, v)) return;
  const int dim = (int)((gx & 1) + (gy & 1) + (gz & 1));
  if ((dim == 1 && v == 2u) || (dim == 2 && v == 1u))
    push_item(queue, n_queue, cap, err, ((int64_t)t.vi << kVolShift) | c);
}

// A block per tile: a warp per halo row record (a lane per cell, KU rows' loads in
// flight), then a thread per inner row byte.
template <int ND, int LY, int LZ>
__global__ void __launch_bounds__(256) ldir_check_kernel(const LdirBatch B, const uint8_t* __restrict__ rec,
                                                         int64_t* __restrict__ queue, int* __restrict__ n_queue,
                                                         int cap, int* lock, int* err) {
  using T = BitTile<ND, LY, LZ>;
  constexpr int KU = 4;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  for (int64_t flat = blockIdx.x; flat < B.total_tiles; flat += gridDim.x) {
    const uint8_t* trec = rec + flat * T::REC;
    const uint32_t* wrec = reinterpret_cast<const uint32_t*>(trec);
    const TileAt t = tile_at<ND, LY, LZ>(B, flat);
    const LdirVol& vol = B.v[t.vi];
    for (int j0 = warp; j0 < T::NHR; j0 += nwarp * KU) {
      uint32_t w2[KU], w1[KU];
      uint8_t own[KU];
      int64_t cell[KU];
#pragma unroll
      for (int k = 0; k < KU; k++) {
        const int j = j0 + k * nwarp;
        w2[k] = j < T::NHR ? wrec[2 * j] : 0u;
        w1[k] = j < T::NHR ? wrec[2 * j + 1] : 0u;
      }
#pragma unroll
      for (int k = 0; k < KU; k++) {
        const int j = j0 + k * nwarp;
        own[k] = 0;
        cell[k] = -1;
        if (((w2[k] | w1[k]) >> lane) & 1u) {
          int ly, lz;
          halo_row_of<ND, LY, LZ>(j, ly, lz);
          cell[k] = (t.o[0] + lane) + (t.o[1] + ly) * vol.D.cs[1] + (t.o[2] + lz) * vol.D.cs[2];
          own[k] = vol.g[cell[k]];
        }
      }
#pragma unroll
      for (int k = 0; k < KU; k++) {
        if (cell[k] < 0) continue;
        const unsigned v = ((w1[k] >> lane) & 1u) ? 1u : 2u;
        if ((unsigned)(own[k] >> 5) <= v) continue;
        int ly, lz;
        halo_row_of<ND, LY, LZ>(j0 + k * nwarp, ly, lz);
        check_cell(B, t, lane, ly, lz, v, queue, n_queue, cap, lock, err);
      }
    }
    for (int i = threadIdx.x; i < T::NIR; i += blockDim.x) {
      const unsigned m = trec[T::NHR * 8 + i];
      if (!m) continue;
      const int ly = 2 + i % (LY - 4), lz = ND == 3 ? 2 + i / (LY - 4) : 0;
#pragma unroll 1
      for (int q = 0; q < 4; q++) {
        const unsigned a2 = (m >> q) & 1u, a1 = (m >> (4 + q)) & 1u;
        if (a2 | a1) check_cell(B, t, q < 2 ? q : kBitLX - 4 + q, ly, lz, a1 ? 1u : 2u, queue, n_queue, cap, lock, err);
      }
    }
  }
}

// Finish the walks of queued items in global memory, depth first with a short
// per-thread stack; what does not fit goes to the next round's queue.
// n_in_dev (when set): the queue length lives in device memory (graph-captured rounds)
template <int ND>
__global__ void __launch_bounds__(128) ldir_walk_kernel(const LdirBatch B, const int64_t* __restrict__ qin, int n_in,
                                                        const int* __restrict__ n_in_dev, int64_t* __restrict__ qout,
                                                        int* __restrict__ n_out, int cap, int* lock, int* err) {
  constexpr int SD = 24;
  int64_t stack[SD];
  if (n_in_dev) {
    n_in = *n_in_dev;
    if (n_in > cap) n_in = 0;  // overflowed: the host finishes with tile passes
  }
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_in; k += gridDim.x * blockDim.x) {
    const int64_t entry = qin[k];
    const int vi = entry_volume(entry);
    if (vi >= B.n) {  // not an entry this launch wrote
      atomicOr(err, kErrPassLimit);
      continue;
    }
    const LdirVol& vol = B.v[vi];
    const GradDims& D = vol.D;
    const GradView G = volume_view(vol, lock, err);
    const int64_t st[3] = {D.cs[0], D.cs[1], D.cs[2]};
    const int64_t dd[3] = {D.d[0], D.d[1], D.d[2]};
    int sp = 0;
    stack[sp++] = entry & kCellMask;
    while (sp > 0) {
      const int64_t i = stack[--sp];
      int64_t l[3];
      l[0] = i % dd[0];
      l[1] = (i / dd[0]) % dd[1];
      l[2] = (ND == 3) ? i / (dd[0] * dd[1]) : 0;
      const int dim = (int)((l[0] & 1) + (l[1] & 1) + (l[2] & 1));
      const unsigned value = dim == 1 ? 2u : 1u;  // edges walk the value-2 closure, quads value 1
#pragma unroll
      for (int a = 0; a < ND; a++) {
        if (l[a] & 1) continue;  // cofacets only along even axes, +axis first
#pragma unroll
        for (int s = 0; s < 2; s++) {
          const int sgn = s == 0 ? 1 : -1;
          const int64_t la = l[a] + sgn;
          if (la < 0 || la >= dd[a]) continue;
          const int64_t t = i + sgn * st[a];
          const uint8_t bt = *reinterpret_cast<volatile uint8_t*>(G.g + t);
          const unsigned code = (bt >> 2) & 7u;
          if (!(bt & 1u) || code == 7u) continue;
          lower_ldir(G, t, value);
          const int pc = map3(D.dec_map, (int)code);
          const int pa = pc >> 1;
          const int64_t tp = t + ((pc & 1) ? -st[pa] : st[pa]);
          if (tp == i) continue;
          int64_t lp[3] = {l[0], l[1], l[2]};
          lp[a] += sgn;
          lp[pa] += (pc & 1) ? -1 : 1;
          if (lp[pa] < 0 || lp[pa] >= dd[pa]) continue;  // a pair code pointing out of the complex
          const int pdim = (int)((lp[0] & 1) + (lp[1] & 1) + (lp[2] & 1));
          if (value == 2u && pdim != 1) {  // a hex ends the value-2 path
            lower_ldir(G, tp, 2u);
            continue;
          }
          if (!lower_ldir(G, tp, value)) continue;
          if (sp < SD) stack[sp++] = tp;
          else push_item(qout, n_out, cap, err, ((int64_t)vi << kVolShift) | tp);
        }
      }
    }
  }
}

namespace {
// multi-pass tiles
constexpr int kTX3 = 32, kTY3 = 32, kTZ3 = 16, kBS3 = 512;
constexpr int kTX2 = 128, kTY2 = 64, kBS2 = 256;
using Tile3 = LdirTile<3, kTX3, kTY3, kTZ3>;
using Tile2 = LdirTile<2, kTX2, kTY2, 1>;
// single-pass bit-row tiles: 28 x 32 x 32 owned cells in 3D, 28 x 252 in 2D
constexpr int kBitLY3 = 36, kBitLZ3 = 36, kBitBS3 = 512;
constexpr int kBitLY2 = 256, kBitBS2 = 256;
using Bit3 = BitTile<3, kBitLY3, kBitLZ3>;
using Bit2 = BitTile<2, kBitLY2, 1>;
}  // namespace

int64_t ldir_num_tiles(int nd, const GradDims& D) {
  if (nd == 3) return ((D.d[0] + kTX3 - 1) / kTX3) * ((D.d[1] + kTY3 - 1) / kTY3) * ((D.d[2] + kTZ3 - 1) / kTZ3);
  return ((D.d[0] + kTX2 - 1) / kTX2) * ((D.d[1] + kTY2 - 1) / kTY2);
}

int64_t ldir_bit_tiles(int nd, const GradDims& D) {
  if (nd == 3)
    return ((D.d[0] + Bit3::TX - 1) / Bit3::TX) * ((D.d[1] + Bit3::TY - 1) / Bit3::TY) *
           ((D.d[2] + Bit3::TZ - 1) / Bit3::TZ);
  return ((D.d[0] + Bit2::TX - 1) / Bit2::TX) * ((D.d[1] + Bit2::TY - 1) / Bit2::TY);
}

int64_t ldir_halo_bytes(int nd) { return nd == 3 ? Bit3::REC : Bit2::REC; }

cudaError_t make_ldir_batch(int nd, int n, uint8_t* const* g, const GradDims* D, LdirBatch* B) {
  if (n < 1 || n > kMaxBatch || (nd == 2 && n != 1)) return cudaErrorInvalidValue;
  B->n = n;
  int64_t off = 0;
  for (int i = 0; i < n; i++) {
    B->v[i].g = g[i];
    B->v[i].D = D[i];
    B->v[i].tile0 = off;
    off += ldir_bit_tiles(nd, D[i]);
  }
  B->total_tiles = off;
  return cudaSuccess;
}

template <class K>
static cudaError_t launch_bit_tiles(K k, int bs, size_t sm, const LdirBatch& B, uint8_t* rec, int* err, int num_sms,
                                    cudaStream_t stream, int ctas_per_sm) {
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  int fit = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k, bs, sm);
  if (e != cudaSuccess) return e;
  const int per_sm = ctas_per_sm < fit ? ctas_per_sm : (fit > 0 ? fit : 1);
  const int64_t cap = (int64_t)num_sms * per_sm;
  const int grid = (int)(B.total_tiles < cap ? B.total_tiles : cap);
  if (grid <= 0) return cudaSuccess;
  ::msc::count_launch();
  k<<<grid, bs, sm, stream>>>(B, rec, err);
  return cudaGetLastError();
}

cudaError_t launch_ldir_tile(int nd, const LdirBatch& B, uint8_t* rec, int* err, int num_sms, cudaStream_t stream,
                             int ctas_per_sm) {
  if (nd == 3)
    return launch_bit_tiles(ldir_tile_kernel<3, kBitLY3, kBitLZ3, kBitBS3, 3>, kBitBS3, Bit3::smem_bytes(), B, rec, err,
                            num_sms, stream, ctas_per_sm);
  return launch_bit_tiles(ldir_tile_kernel<2, kBitLY2, 1, kBitBS2, 4>, kBitBS2, Bit2::smem_bytes(), B, rec, err, num_sms,
                          stream, ctas_per_sm);
}

static int check_grid(const LdirBatch& B, int num_sms) {
  const int64_t cap = (int64_t)num_sms * 8;
  return (int)(B.total_tiles < cap ? (B.total_tiles > 0 ? B.total_tiles : 1) : cap);
}

cudaError_t launch_ldir_check(int nd, const LdirBatch& B, const uint8_t* rec, int64_t* queue, int* n_queue, int cap,
                              int* lock, int* err, int num_sms, cudaStream_t stream) {
  ::msc::count_launch();
  if (nd == 3)
    ldir_check_kernel<3, kBitLY3, kBitLZ3><<<check_grid(B, num_sms), 256, 0, stream>>>(B, rec, queue, n_queue, cap,
                                                                                       lock, err);
  else
    ldir_check_kernel<2, kBitLY2, 1><<<check_grid(B, num_sms), 256, 0, stream>>>(B, rec, queue, n_queue, cap, lock,
                                                                                 err);
  return cudaGetLastError();
}

cudaError_t launch_ldir_walk(int nd, const LdirBatch& B, const int64_t* qin, int n_in, int64_t* qout, int* n_out,
                             int cap, int* lock, int* err, int num_sms, cudaStream_t stream) {
  if (n_in <= 0) return cudaSuccess;
  const int blocks = (n_in + 127) / 128;
  const int grid = blocks < num_sms * 16 ? blocks : num_sms * 16;
  if (nd == 3) {
    ::msc::count_launch();
    ldir_walk_kernel<3><<<grid, 128, 0, stream>>>(B, qin, n_in, nullptr, qout, n_out, cap, lock, err);
  } else {
    ::msc::count_launch();
    ldir_walk_kernel<2><<<grid, 128, 0, stream>>>(B, qin, n_in, nullptr, qout, n_out, cap, lock, err);
  }
  return cudaGetLastError();
}

cudaError_t launch_ldir_walk_dev(const LdirBatch& B, const int64_t* qin, const int* n_in_dev, int64_t* qout, int* n_out,
                                 int cap, int* lock, int* err, int num_sms, cudaStream_t stream) {
  ::msc::count_launch();
  ldir_walk_kernel<3><<<num_sms * 16, 128, 0, stream>>>(B, qin, 0, n_in_dev, qout, n_out, cap, lock, err);
  return cudaGetLastError();
}

cudaError_t launch_ldir_pass(int nd, uint8_t* g, const GradDims& D, const uint8_t* dirty_in, uint8_t* dirty_out,
                             int* changed, int* err, int num_sms, cudaStream_t stream) {
  const int64_t nt = ldir_num_tiles(nd, D);
  const int64_t cap = (int64_t)num_sms * 4;
  const int grid = (int)(nt < cap ? nt : cap);
  if (grid <= 0) return cudaSuccess;
  if (nd == 3) {
    auto k = ldir_pass_kernel<3, kTX3, kTY3, kTZ3, kBS3>;
    const size_t sm = Tile3::smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    ::msc::count_launch();
    k<<<grid, kBS3, sm, stream>>>(g, D, dirty_in, dirty_out, changed, err);
  } else {
    auto k = ldir_pass_kernel<2, kTX2, kTY2, 1, kBS2>;
    const size_t sm = Tile2::smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    ::msc::count_launch();
    k<<<grid, kBS2, sm, stream>>>(g, D, dirty_in, dirty_out, changed, err);
  }
  return cudaGetLastError();
}

}  // namespace msc
