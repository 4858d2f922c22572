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
  // of the tile kernel: queue (u16; NL items at most plus one pending claim per thread,
  // QX >= the block size) | bytes | value-2 marks | visited bits
  static constexpr int QX = 1024;
  static constexpr size_t tile_smem_bytes() {
    return (size_t)(NL + QX) * 2 + ((NL + 3) / 4) * 8 + (size_t)NW * 4;
  }
};

// local index -> local coords
template <class T>
__device__ __forceinline__ void lcoords(int i, int& lx, int& ly, int& lz) {
  lx = i % T::LX;
  ly = (i / T::LX) % T::LY;
  lz = i / (T::LX * T::LY);
}

// k-th halo cell of the box -> box index (z slabs, then y rows, then x columns)
template <class T, int ND>
__device__ __forceinline__ int halo_cell(int h) {
  constexpr int H = T::H, LX = T::LX, LY = T::LY, LZ = T::LZ;
  int lz = 0;
  if (ND == 3) {
    constexpr int SLAB = 2 * H * LX * LY;  // z < H and z >= LZ - H
    if (h < SLAB) {
      const int s = h / (LX * LY), r = h % (LX * LY);
      lz = s < H ? s : LZ - 2 * H + s;
      return r + LX * LY * lz;
    }
    h -= SLAB;
  }
  constexpr int P = 2 * H * LX + 2 * H * (LY - 2 * H);  // halo cells of one inner plane
  lz = (ND == 3 ? H : 0) + h / P;
  int r = h % P;
  int lx, ly;
  if (r < 2 * H * LX) {
    const int s = r / LX;
    ly = s < H ? s : LY - 2 * H + s;
    lx = r % LX;
  } else {
    r -= 2 * H * LX;
    const int s = r / (LY - 2 * H);
    lx = s < H ? s : LX - 2 * H + s;
    ly = H + r % (LY - 2 * H);
  }
  return lx + LX * (ly + LY * lz);
}

template <class T, int ND>
__host__ __device__ constexpr int halo_count() {
  return (ND == 3 ? 2 * T::H * T::LX * T::LY : 0) +
         (ND == 3 ? (T::LZ - 2 * T::H) : 1) * (2 * T::H * T::LX + 2 * T::H * (T::LY - 2 * T::H));
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

// warp_push for a queue that other threads read while it grows (the tile kernel's
// barrier-free walk): the item is stored through a volatile pointer.
__device__ __forceinline__ void warp_push_live(uint16_t* sq, int* qtail, int cap, int* err, bool want, int item) {
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
    if (slot < cap) reinterpret_cast<volatile uint16_t*>(sq)[slot] = (uint16_t)item;
    else atomicOr(err, kErrLocalQueue);
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

// ---- single-pass form: one tile pass, a halo check, a global frontier walk -------------------
//
// A tile's walk is complete for every item of its interior (all of an item's rule
// reaches lies within 2 cells), so after one pass over all tiles the only missing
// marks are those a tile made in its halo that the halo's owner did not make itself.
// The pass therefore saves each tile's final box; the check kernel lowers every
// global cell that some tile's saved halo holds lower, and queues the lowered items,
// whose walk may need to continue beyond that tile's box; the walk kernel finishes
// those walks in global memory.  Concurrent lowering of a byte uses a compare-and-swap
// on its aligned 32-bit word (the low five bits never change, so the ldir field only
// ever decreases); bytes whose word is not wholly inside the .grad array go through a
// bounded spin lock instead.

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

// Both closures in the same walk.  The value-2 closure (items: edges) keeps its marks
// in a byte plane of its own, m2, and the value-1 closure (items: quads) in the .grad
// bytes, so the two never race on a byte and run in the same BFS levels; an item's
// dimension says which closure it walks.  The final byte is the .grad byte with ldir
// lowered to 2 where m2 is set.
template <class T, int ND>
struct LdirWalk2 {
  uint8_t* sg;
  uint8_t* m2;
  uint16_t* sq;
  uint32_t* vis;
  int* qtail;
  int* err;
  int lmin[3], lmax[3];
  uint32_t dec_map;

  __device__ __forceinline__ int visit(int i, int l[3], int a, int sgn, bool r2) {
    constexpr int LE[3] = {T::LX, T::LY, T::LZ};
    const int la = l[a] + sgn;
    if (la < lmin[a] || la >= lmax[a]) return -1;
    const int t = i + sgn * T::ls(a);
    const uint8_t bt = sg[t];
    const unsigned code = (bt >> 2) & 7u;
    if (!(bt & 1u) || code == 7u) return -1;  // unassigned or critical
    if (r2) m2[t] |= 1u;
    else if ((bt >> 5) != 1u) sg[t] = (uint8_t)((bt & 0x1Fu) | (1u << 5));
    const int pc = map3(dec_map, (int)code);
    const int pa = pc >> 1, psg = (pc & 1) ? -1 : 1;
    int lp[3] = {l[0], l[1], l[2]};
    lp[a] += sgn;
    lp[pa] += psg;
    if (lp[pa] < 0 || lp[pa] >= LE[pa]) return -1;  // partner outside the box
    const int tp = t + psg * T::ls(pa);
    if (tp == i) return -1;
    const uint8_t bp = sg[tp];
    if (r2) {
      const int pdim = (lp[0] & 1) + (lp[1] & 1) + (ND == 3 ? (lp[2] & 1) : 0);
      if (pdim != 1) {  // a hex: the value-2 path ends here
        m2[tp] |= 1u;
        return -1;
      }
      if ((bp >> 5) == 2u || (m2[tp] & 1u)) return -1;  // a root, or marked already
    } else {
      if ((bp >> 5) == 1u) return -1;
    }
    const uint32_t bit = 1u << (tp & 31);
    if (atomicOr(&vis[tp >> 5], bit) & bit) return -1;
    if (r2) m2[tp] |= 1u;
    else sg[tp] = (uint8_t)((bp & 0x1Fu) | (1u << 5));
    return tp;
  }

  __device__ __forceinline__ void step(int i) {
    int l[3];
    lcoords<T>(i, l[0], l[1], l[2]);
    const bool r2 = ((l[0] & 1) + (l[1] & 1) + (ND == 3 ? (l[2] & 1) : 0)) == 1;
#pragma unroll
    for (int a = 0; a < ND; a++) {
#pragma unroll
      for (int s = 0; s < 2; s++) {
        // cofacets only along even axes, +axis first
        const int nx = (l[a] & 1) ? -1 : visit(i, l, a, s == 0 ? 1 : -1, r2);
        warp_push_live(sq, qtail, T::NL, err, nx >= 0, nx);
      }
    }
  }
};

constexpr uint16_t kTileQueueEmpty = 0xFFFF;        // an unfilled slot (NL < 65535)
constexpr uint32_t kTileQueueSpinLimit = 1u << 24;  // bound of a wait for a slot (~0.5 s)

__device__ __forceinline__ int batch_volume(const LdirBatch& B, int64_t flat_tile) {
  int lo = 0, hi = B.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (B.v[mid].tile0 <= flat_tile) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <int ND, int TX, int TY, int TZ, int BS>
__global__ void __launch_bounds__(BS) ldir_tile_kernel(const LdirBatch B, uint8_t* __restrict__ saved,
                                                       int* __restrict__ err) {
  using T = LdirTile<ND, TX, TY, TZ>;
  constexpr int NL = T::NL;
  static_assert(NL < 65536, "local ids are 16-bit");
  extern __shared__ __align__(16) unsigned char s_dyn[];
  // queue (u16) | .grad bytes | value-2 marks | visited bits
  constexpr int QCAP = NL + T::QX;
  static_assert(BS <= T::QX, "one pending queue claim per thread");
  uint16_t* sq = reinterpret_cast<uint16_t*>(s_dyn);
  uint8_t* sg = s_dyn + (size_t)QCAP * 2;
  uint8_t* m2 = sg + ((NL + 3) / 4) * 4;
  uint32_t* s_vis = reinterpret_cast<uint32_t*>(m2 + ((NL + 3) / 4) * 4);
  __shared__ int s_qtail, s_head, s_done;

  const int tid = threadIdx.x;

  LdirWalk2<T, ND> W;
  W.sg = sg;
  W.m2 = m2;
  W.sq = sq;
  W.vis = s_vis;
  W.qtail = &s_qtail;
  W.err = err;

  for (int64_t flat = blockIdx.x; flat < B.total_tiles; flat += gridDim.x) {
    const LdirVol& vol = B.v[batch_volume(B, flat)];
    uint8_t* __restrict__ g = vol.g;
    const GradDims& D = vol.D;
    W.dec_map = D.dec_map;
    const int64_t dX = D.d[0], dY = D.d[1], dZ = D.d[2];
    const int64_t ntx = (dX + TX - 1) / TX, nty = (dY + TY - 1) / TY;
    const int64_t tile = flat - vol.tile0;
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
      s_head = 0;
      s_done = 0;
    }
    for (int w = tid; w < T::NW; w += BS) s_vis[w] = 0;
    for (int k = tid; k < QCAP; k += BS) sq[k] = kTileQueueEmpty;
    __syncthreads();

    // stage the box (cells outside the complex read as 0 = unassigned), many loads in
    // flight per thread, and queue every marked item -- the roots -- as a seed
    constexpr int PER = (NL + BS - 1) / BS;
    constexpr int U = 8;
#pragma unroll 1
    for (int j0 = 0; j0 < PER; j0 += U) {
      uint8_t v[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int k = (j0 + u) * BS + tid;
        v[u] = 0;
        if (j0 + u < PER && k < NL) {
          const int lx = k % T::LX, row = k / T::LX;
          const int ly = row % T::LY, lz = row / T::LY;
          if (lx >= W.lmin[0] && lx < W.lmax[0] && ly >= W.lmin[1] && ly < W.lmax[1] && lz >= W.lmin[2] &&
              lz < W.lmax[2])
            v[u] = g[(o[0] + lx) + (o[1] + ly) * D.cs[1] + (o[2] + lz) * D.cs[2]];
        }
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int k = (j0 + u) * BS + tid;
        const bool valid = j0 + u < PER && k < NL;
        int dim = 0;
        if (valid) {
          sg[k] = v[u];
          m2[k] = (uint8_t)(v[u] & 0xE0u);  // staged ldir above the value-2 mark bit
          const int lx = k % T::LX, row = k / T::LX;
          const int ly = row % T::LY, lz = row / T::LY;
          dim = (lx & 1) + (ly & 1) + (ND == 3 ? (lz & 1) : 0);
        }
        const unsigned ld = v[u] >> 5;
        const bool seed = valid && (v[u] & 1u) && ((dim == 1 && ld == 2u) || (dim == 2 && ld == 1u));
        warp_push(sq, &s_qtail, NL, err, seed, k);
      }
    }
    __syncthreads();

    // both closures; the fixpoint does not depend on the order, so rather than BFS
    // levels separated by barriers every thread takes the next queue slot as soon as
    // its item is walked.  A slot below s_qtail is filled by its producer; a thread
    // whose slot is beyond every reserved one stops once every reserved item is done
    // (an item counts as done only after its pushes were reserved).
    {
      int h = atomicAdd(&s_head, 1);
      volatile uint16_t* vq = sq;
      volatile int* vdone = &s_done;
      volatile int* vtail = &s_qtail;
      for (uint32_t spin = 0;; spin++) {
        const uint16_t it = h < QCAP ? (uint16_t)vq[h] : (uint16_t)kTileQueueEmpty;
        if (it != kTileQueueEmpty) {
          W.step(it);
          __threadfence_block();
          atomicAdd(&s_done, 1);
          h = atomicAdd(&s_head, 1);
          spin = 0;
          continue;
        }
        const int d = *vdone;
        const int t = *vtail;
        if (d == t && h >= t) break;
        if (spin > kTileQueueSpinLimit) {  // cannot happen by construction: report, stop
          atomicOr(err, kErrPassLimit);
          break;
        }
        __nanosleep(32);
      }
    }

    // fold the value-2 marks into the bytes
    for (int k = tid; k < NL; k += BS) {
      const uint8_t b = sg[k];
      if ((m2[k] & 1u) && (b >> 5) == 3u) sg[k] = (uint8_t)((b & 0x1Fu) | (2u << 5));
    }
    __syncthreads();

    // write back the interior, a row per warp instruction
    constexpr int NI = TX * TY * (ND == 3 ? TZ : 1);
    for (int k = tid; k < NI; k += BS) {
      const int ix = k % TX, r = k / TX;
      const int iy = r % TY, iz = r / TY;
      const int64_t gx = o[0] + T::H + ix, gy = o[1] + T::H + iy, gz = o[2] + (ND == 3 ? T::H : 0) + iz;
      if (gx < dX && gy < dY && gz < dZ)
        g[gx + gy * D.cs[1] + gz * D.cs[2]] = sg[(ix + T::H) + T::LX * ((iy + T::H) + T::LY * (iz + (ND == 3 ? T::H : 0)))];
    }
    // save the halo cells this tile lowered (0 for the rest), in halo order
    constexpr int NH = halo_count<T, ND>();
    uint8_t* sv = saved + flat * (int64_t)NH;
    for (int h = tid; h < NH; h += BS) {
      const int k = halo_cell<T, ND>(h);
      const uint8_t b = sg[k];
      sv[h] = ((unsigned)(b >> 5) < (unsigned)(m2[k] >> 5)) ? b : (uint8_t)0;
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

template <int ND, int TX, int TY, int TZ>
__global__ void ldir_check_kernel(const LdirBatch B, const uint8_t* __restrict__ saved, int64_t* __restrict__ queue,
                                  int* __restrict__ n_queue, int cap, int* lock, int* err) {
  using T = LdirTile<ND, TX, TY, TZ>;
  constexpr int NH = halo_count<T, ND>();
  static_assert(NH % 16 == 0, "halo records are read 16 bytes at a time");
  const int64_t total = B.total_tiles * NH;
  // 16 saved bytes per step: almost all are zero (not lowered by their tile)
  for (int64_t e0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) * 16; e0 < total;
       e0 += (int64_t)gridDim.x * blockDim.x * 16) {
    const uint4 q = *reinterpret_cast<const uint4*>(saved + e0);
    if (!((q.x | q.y | q.z | q.w) & 0x01010101u)) continue;
#pragma unroll 1
    for (int j = 0; j < 16; j++) {
      const int64_t e = e0 + j;
      const uint8_t s = saved[e];
      if (!(s & 1u)) continue;  // not lowered by its tile
      const int64_t flat = e / NH;
      const int b = halo_cell<T, ND>((int)(e % NH));
      const int vi = batch_volume(B, flat);
      const LdirVol& vol = B.v[vi];
      const GradDims& D = vol.D;
      const int64_t ntx = (D.d[0] + TX - 1) / TX, nty = (D.d[1] + TY - 1) / TY;
      const int64_t tile = flat - vol.tile0;
      const int64_t tx = tile % ntx, ty = (tile / ntx) % nty, tz = (ND == 3) ? tile / (ntx * nty) : 0;
      const int lx = b % T::LX, ly = (b / T::LX) % T::LY, lz = b / (T::LX * T::LY);
      const int64_t gx = tx * TX - T::H + lx, gy = ty * TY - T::H + ly, gz = (ND == 3) ? tz * TZ - T::H + lz : 0;
      const int64_t c = gx + gy * D.cs[1] + gz * D.cs[2];
      const unsigned v = s >> 5;
      if ((unsigned)(vol.g[c] >> 5) <= v) continue;
      const GradView G = volume_view(vol, lock, err);
      if (!lower_ldir(G, c, v)) continue;
      const int dim = (int)((gx & 1) + (gy & 1) + (gz & 1));
      if ((dim == 1 && v == 2u) || (dim == 2 && v == 1u))
        push_item(queue, n_queue, cap, err, ((int64_t)vi << kVolShift) | c);
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
constexpr int kTX3 = 32, kTY3 = 32, kTZ3 = 16, kBS3 = 512;
constexpr int kTX2 = 128, kTY2 = 64, kBS2 = 256;
using Tile3 = LdirTile<3, kTX3, kTY3, kTZ3>;
using Tile2 = LdirTile<2, kTX2, kTY2, 1>;
}  // namespace

int64_t ldir_num_tiles(int nd, const GradDims& D) {
  if (nd == 3) return ((D.d[0] + kTX3 - 1) / kTX3) * ((D.d[1] + kTY3 - 1) / kTY3) * ((D.d[2] + kTZ3 - 1) / kTZ3);
  return ((D.d[0] + kTX2 - 1) / kTX2) * ((D.d[1] + kTY2 - 1) / kTY2);
}

int64_t ldir_halo_bytes(int nd) { return nd == 3 ? halo_count<Tile3, 3>() : halo_count<Tile2, 2>(); }

cudaError_t make_ldir_batch(int nd, int n, uint8_t* const* g, const GradDims* D, LdirBatch* B) {
  if (n < 1 || n > kMaxBatch || (nd == 2 && n != 1)) return cudaErrorInvalidValue;
  B->n = n;
  int64_t off = 0;
  for (int i = 0; i < n; i++) {
    B->v[i].g = g[i];
    B->v[i].D = D[i];
    B->v[i].tile0 = off;
    off += ldir_num_tiles(nd, D[i]);
  }
  B->total_tiles = off;
  return cudaSuccess;
}

cudaError_t launch_ldir_tile(int nd, const LdirBatch& B, uint8_t* saved, int* err, int num_sms, cudaStream_t stream,
                             int ctas_per_sm) {
  const int64_t cap = (int64_t)num_sms * ctas_per_sm;
  const int grid = (int)(B.total_tiles < cap ? B.total_tiles : cap);
  if (grid <= 0) return cudaSuccess;
  if (nd == 3) {
    auto k = ldir_tile_kernel<3, kTX3, kTY3, kTZ3, kBS3>;
    const size_t sm = Tile3::tile_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    ::msc::count_launch();
    k<<<grid, kBS3, sm, stream>>>(B, saved, err);
  } else {
    auto k = ldir_tile_kernel<2, kTX2, kTY2, 1, kBS2>;
    const size_t sm = Tile2::tile_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    ::msc::count_launch();
    k<<<grid, kBS2, sm, stream>>>(B, saved, err);
  }
  return cudaGetLastError();
}

cudaError_t launch_ldir_check(int nd, const LdirBatch& B, const uint8_t* saved, int64_t* queue, int* n_queue, int cap,
                              int* lock, int* err, int num_sms, cudaStream_t stream) {
  if (nd == 3) {
    ::msc::count_launch();
    ldir_check_kernel<3, kTX3, kTY3, kTZ3><<<num_sms * 8, 256, 0, stream>>>(B, saved, queue, n_queue, cap, lock, err);
  } else {
    ::msc::count_launch();
    ldir_check_kernel<2, kTX2, kTY2, 1><<<num_sms * 8, 256, 0, stream>>>(B, saved, queue, n_queue, cap, lock, err);
  }
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
