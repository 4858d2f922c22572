// Integrated ascending / descending labels, sm_103a.
//
// Replaces ondemandaccurate's 3-manifold labeling chain (ondemandaccurate.cxx:795-948):
//   K5a  extrema + saddle V-path arcs  SimplifiedExtremumGraph::ComputeMinMapFromGradient
//        (gi_extrema_region_builder.h:271-565).  Arcs whose persistence exceeds the
//        merge threshold can never merge (PerformCancel drops them on first pop,
//        :98-105), so only the rest leave the GPU for the priority-queue merge.
//   K5b  certain terminal regions       GridSimplifiedExtremalRegionBuilder
//        (:753-1045): a vertex joins the region all of its earlier 6-neighbours
//        belong to.  That rule is monotone on the DAG of the vertex order, so shared-
//        memory tiles walk it to a local fixpoint and repeat over tiles whose halo
//        changed, as the ldir closure does.
//   K4   streamline integration         NumericIntegratorPathCompressingToTerminal
//        (gi_numeric_integrator_path_compressing.h:75-433) -- integrate_kernels.cu
//   K5c  isolated-region cleaner        IsolatedCCRegionRemoverNEW (gi_isolated_region_remover.h)
//        -- integrate_kernels.cu
//
// Regions are named by their smallest seed vertex (the extremum's vertex when nothing
// merged); -1 = outside every region.  The reference numbers regions in unordered_map
// order, so only the partition is comparable.
#include <cstdlib>
#include "label_common.cuh"

namespace msc {

// ---- K5a: extrema and saddles ----------------------------------------------------

// Every critical cell of the extremum / saddle dimension of the walk.  Extremum ids
// are keyed by a vertex: the minimum itself, or the hex's lowest corner.
// Warp-wide exclusive prefix sum of v; `total` receives the warp's sum.
__device__ __forceinline__ int warp_exclusive_sum(int v, int& total) {
  const int lane = threadIdx.x & 31;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  total = __shfl_sync(0xffffffffu, x, 31);
  return x - v;
}

// Every thread scans 16 consecutive cells (one 16-byte load where the array allows);
// the critical cells of this direction are appended with one atomic per warp and kind.
__global__ void find_critical_kernel(const uint8_t* __restrict__ g, const VolDims V, int dir,
                                     int32_t* __restrict__ ext_id_of_key, int64_t* __restrict__ ext_cells,
                                     int* __restrict__ n_ext, int64_t* __restrict__ saddles, int* __restrict__ n_sad) {
  const int ext_dim = dir < 0 ? 0 : 3, sad_dim = dir < 0 ? 1 : 2;
  const int64_t nc = V.dX * V.dY * V.dZ;
  const int64_t nchunks = (nc + 15) / 16;
  const bool vec = (reinterpret_cast<uintptr_t>(g) & 15u) == 0;
  const int lane = threadIdx.x & 31;
  for (int64_t ch = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ch - lane < nchunks;
       ch += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c0 = ch * 16;
    uint8_t bytes[16];
    if (ch < nchunks && vec && c0 + 16 <= nc) {
      const uint4 w = *reinterpret_cast<const uint4*>(g + c0);
      const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
      for (int j = 0; j < 16; j++) bytes[j] = (uint8_t)(ws[j >> 2] >> (8 * (j & 3)));
    } else {
#pragma unroll
      for (int j = 0; j < 16; j++) bytes[j] = (ch < nchunks && c0 + j < nc) ? g[c0 + j] : (uint8_t)0;
    }
    uint32_t ext_mask = 0, sad_mask = 0;
#pragma unroll
    for (int j = 0; j < 16; j++) {
      if (((bytes[j] >> 2) & 7) != 7) continue;
      int64_t k[3];
      cell_coords(V, c0 + j, k);
      const int d = (int)((k[0] & 1) + (k[1] & 1) + (k[2] & 1));
      if (d == ext_dim) ext_mask |= 1u << j;
      // trace_up_2saddle skips 2-saddles on the boundary (gi_extrema_region_builder.h:315-318)
      else if (d == sad_dim && !(dir > 0 && boundary_value(V, k) != 0)) sad_mask |= 1u << j;
    }
    int ne = 0, ns = 0;
    const int oe = warp_exclusive_sum(__popc(ext_mask), ne);
    const int os = warp_exclusive_sum(__popc(sad_mask), ns);
    int be = 0, bs = 0;
    if (lane == 0) {
      if (ne) be = atomicAdd(n_ext, ne);
      if (ns) bs = atomicAdd(n_sad, ns);
    }
    be = __shfl_sync(0xffffffffu, be, 0) + oe;
    bs = __shfl_sync(0xffffffffu, bs, 0) + os;
    while (ext_mask) {
      const int j = __ffs(ext_mask) - 1;
      ext_mask &= ext_mask - 1;
      int64_t k[3];
      cell_coords(V, c0 + j, k);
      ext_cells[be] = c0 + j;
      ext_id_of_key[(k[0] >> 1) + (k[1] >> 1) * V.X + (k[2] >> 1) * V.X * V.Y] = be;
      be++;
    }
    while (sad_mask) {
      const int j = __ffs(sad_mask) - 1;
      sad_mask &= sad_mask - 1;
      saddles[bs++] = c0 + j;
    }
  }
}

// rec_td (:286-300) / rec_tu (:330-346): follow the V-path to a critical cell
__device__ int64_t trace_vpath(const uint8_t* __restrict__ g, const VolDims& V, int dir, int64_t cell, int* err) {
  const int64_t st[3] = {1, V.cs1, V.cs2};
  const int64_t dd[3] = {V.dX, V.dY, V.dZ};
  for (int64_t guard = 0; guard < V.dX * V.dY * V.dZ; guard++) {
    if (((g[cell] >> 2) & 7) == 7) return cell;
    const int64_t pair = decode_pair(V, cell, (g[cell] >> 2) & 7);
    if (((g[pair] >> 2) & 7) == 7) return pair;
    int64_t k[3];
    cell_coords(V, pair, k);
    int64_t first = -1, second = -1;
    for (int a = 0; a < 3 && second < 0; a++) {
      const bool take = dir < 0 ? (k[a] & 1) : !(k[a] & 1);   // facets (odd axes) / cofacets (even axes)
      if (!take) continue;
      const int64_t cand[2] = {pair + st[a], pair - st[a]};
      const bool ok[2] = {dir < 0 || k[a] != dd[a] - 1, dir < 0 || k[a] != 0};
      for (int s = 0; s < 2; s++) {
        if (!ok[s]) continue;
        if (first < 0) first = cand[s];
        else if (second < 0) second = cand[s];
      }
    }
    cell = (first == cell && second >= 0) ? second : first;
  }
  atomicOr(err, kErrIterLimit);
  return cell;
}

__global__ void trace_arcs_kernel(const uint8_t* __restrict__ g, const float* __restrict__ f, const VolDims V, int dir,
                                  const int64_t* __restrict__ saddles, int n_sad, const int32_t* __restrict__ ext_id_of_key,
                                  float threshold, Arc* __restrict__ arcs, int* __restrict__ n_arcs, int* err) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n_sad; s += gridDim.x * blockDim.x) {
    const int64_t sad = saddles[s];
    int64_t k[3];
    cell_coords(V, sad, k);
    int64_t ends[2];
    int n = 0;
    const int64_t st[3] = {1, V.cs1, V.cs2};
    const int64_t dd[3] = {V.dX, V.dY, V.dZ};
    for (int a = 0; a < 3 && n < 2; a++) {
      const bool take = dir < 0 ? (k[a] & 1) : !(k[a] & 1);
      if (!take) continue;
      if (dir < 0 || k[a] != dd[a] - 1) { if (n < 2) ends[n++] = sad + st[a]; }
      if (dir < 0 || k[a] != 0) { if (n < 2) ends[n++] = sad - st[a]; }
    }
    if (n < 2) continue;
    const int64_t e1 = trace_vpath(g, V, dir, ends[0], err);
    const int64_t e2 = trace_vpath(g, V, dir, ends[1], err);
    if (e1 == e2) continue;
    const float sval = f[highest_vertex(V, f, sad)];
    const int64_t h1 = highest_vertex(V, f, e1), h2 = highest_vertex(V, f, e2);
    const float f1 = f[h1], f2 = f[h2];
    float d1 = f1 - sval, d2 = f2 - sval;
    if (d1 < 0) d1 *= -1;
    if (d2 < 0) d2 *= -1;
    const float pers = d1 < d2 ? d1 : d2;
    if (!(pers <= threshold)) continue;  // can never merge
    const int slot = atomicAdd(n_arcs, 1);
    int64_t k1[3], k2[3];
    cell_coords(V, e1, k1);
    cell_coords(V, e2, k2);
    arcs[slot].saddle = sad;
    arcs[slot].e1 = ext_id_of_key[(k1[0] >> 1) + (k1[1] >> 1) * V.X + (k1[2] >> 1) * V.X * V.Y];
    arcs[slot].e2 = ext_id_of_key[(k2[0] >> 1) + (k2[1] >> 1) * V.X + (k2[2] >> 1) * V.X * V.Y];
    arcs[slot].sval = sval;
    arcs[slot].pers = pers;
    arcs[slot].c1 = e1;
    arcs[slot].c2 = e2;
    arcs[slot].h1 = h1;
    arcs[slot].h2 = h2;
    arcs[slot].f1 = f1;
    arcs[slot].f2 = f2;
  }
}

// Per extremum: cell value (cellValue = value of the highest vertex) and that vertex,
// for the host-side merge and for seeding.
__global__ void extremum_info_kernel(const float* __restrict__ f, const VolDims V, int dir,
                                     const int64_t* __restrict__ ext_cells, int n_ext, int64_t* __restrict__ hv,
                                     float* __restrict__ fval, int64_t* __restrict__ seed) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n_ext; e += gridDim.x * blockDim.x) {
    const int64_t c = ext_cells[e];
    const int64_t h = highest_vertex(V, f, c);
    hv[e] = h;
    fval[e] = f[h];
    int64_t k[3];
    cell_coords(V, c, k);
    // seeds: the minimum's vertex; the hex's highest vertex (extmapDSC keys,
    // ondemandaccurate.cxx:913-915)
    seed[e] = dir < 0 ? (k[0] >> 1) + (k[1] >> 1) * V.X + (k[2] >> 1) * V.X * V.Y : h;
  }
}

// Region name of each merged group: its smallest seed vertex.
__global__ void group_name_kernel(const int32_t* __restrict__ rep, const int64_t* __restrict__ seed, int n_ext,
                                  int32_t* __restrict__ name) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n_ext; e += gridDim.x * blockDim.x)
    atomicMin(&name[rep[e]], (int32_t)seed[e]);
}

__global__ void place_seeds_kernel(const int32_t* __restrict__ rep, const int64_t* __restrict__ seed, int n_ext,
                                   const int32_t* __restrict__ name, int32_t* __restrict__ lab,
                                   uint8_t* __restrict__ state) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n_ext; e += gridDim.x * blockDim.x) {
    const int64_t s = seed[e];
    // two maxima sharing a top vertex: keep the smaller name
    const int32_t nm = name[rep[e]];
    const int32_t old = atomicCAS(&lab[s], -1, nm);
    if (old != -1 && nm < old) atomicMin(&lab[s], nm);
    state[s] = kStSeed;
  }
}

// ---- K5b: certain terminal regions --------------------------------------------------

constexpr uint16_t kQueueEmpty = 0xFFFF;          // an unfilled slot of a shared-memory queue
constexpr uint32_t kQueueSpinLimit = 1u << 24;    // bound of a wait for a slot (~0.5 s)

template <int TX, int TY, int TZ>
struct VBox {
  static constexpr int H = 2;
  static constexpr int LX = TX + 2 * H, LY = TY + 2 * H, LZ = TZ + 2 * H;
  static constexpr int NL = LX * LY * LZ;
  static constexpr int NW = (NL + 31) / 32;
  static constexpr int ls(int a) { return a == 0 ? 1 : (a == 1 ? LX : LX * LY); }
  static constexpr size_t smem_bytes() { return (size_t)NL * (4 + 4 + 2) + (size_t)NW * 8; }
};

template <class B>
struct TerminalWalk {
  const float* sf;
  int32_t* sl;
  const uint8_t* sseed;  // unused slot kept for alignment clarity
  uint16_t* sq;
  uint32_t* vis;
  uint32_t* dirty;
  int* qtail;
  int* err;
  int dir;
  int lmin[3], lmax[3];
  int64_t o[3];
  int64_t X, XY;

  __device__ __forceinline__ int64_t gidx(int i) const {
    const int lx = i % B::LX, ly = (i / B::LX) % B::LY, lz = i / (B::LX * B::LY);
    return (o[0] + lx) + X * (o[1] + ly) + XY * (o[2] + lz);
  }
  // Comparer::Compare(a, b) on local positions: "a comes before b"
  __device__ __forceinline__ bool before(int a, int b) const {
    const float fa = sf[a], fb = sf[b];
    if (dir < 0) {
      if (fb > fa) return true;
      if (fa > fb) return false;
      return gidx(b) > gidx(a);
    }
    if (fa > fb) return true;
    if (fb > fa) return false;
    return gidx(a) > gidx(b);
  }
  __device__ __forceinline__ bool inside(int lx, int ly, int lz) const {
    return lx >= lmin[0] && lx < lmax[0] && ly >= lmin[1] && ly < lmax[1] && lz >= lmin[2] && lz < lmax[2];
  }
  // InspectPriorRegions (gi_extrema_region_builder.h:806-857) for a non-seed vertex
  __device__ __forceinline__ int32_t inspect(int w, int wx, int wy, int wz) const {
    int32_t lab = -1;
    bool has = false;
    const int nx[6] = {1, -1, 0, 0, 0, 0}, ny[6] = {0, 0, 1, -1, 0, 0}, nz[6] = {0, 0, 0, 0, 1, -1};
#pragma unroll
    for (int k = 0; k < 6; k++) {
      if (!inside(wx + nx[k], wy + ny[k], wz + nz[k])) continue;
      const int u = w + nx[k] + ny[k] * B::LX + nz[k] * B::LX * B::LY;
      if (!before(u, w)) continue;
      const int32_t lu = reinterpret_cast<volatile int32_t*>(sl)[u];
      if (lu < 0) return -1;
      if (!has) { lab = lu; has = true; }
      else if (lu != lab) return -1;
    }
    return has ? lab : -1;
  }
  __device__ __forceinline__ int step(int v) {
    const int vx = v % B::LX, vy = (v / B::LX) % B::LY, vz = v / (B::LX * B::LY);
    const int nx[6] = {1, -1, 0, 0, 0, 0}, ny[6] = {0, 0, 1, -1, 0, 0}, nz[6] = {0, 0, 0, 0, 1, -1};
    int next = -1;
#pragma unroll
    for (int k = 0; k < 6; k++) {
      const int wx = vx + nx[k], wy = vy + ny[k], wz = vz + nz[k];
      // w's own 6-neighbourhood must lie in the box to be inspected here
      if (wx < 1 || wx >= B::LX - 1 || wy < 1 || wy >= B::LY - 1 || wz < 1 || wz >= B::LZ - 1) continue;
      if (!inside(wx, wy, wz)) continue;
      const int w = v + nx[k] + ny[k] * B::LX + nz[k] * B::LX * B::LY;
      if (reinterpret_cast<volatile int32_t*>(sl)[w] != -1 || !before(v, w)) continue;
      const int32_t l = inspect(w, wx, wy, wz);
      if (l < 0) continue;
      const uint32_t bit = 1u << (w & 31);
      if (atomicOr(&vis[w >> 5], bit) & bit) continue;
      reinterpret_cast<volatile int32_t*>(sl)[w] = l;
      __threadfence_block();  // the label before the vertex is handed to another thread
      atomicOr(&dirty[w >> 5], bit);
      if (next < 0) {
        next = w;
      } else {
        const int slot = atomicAdd(qtail, 1);
        if (slot < B::NL) reinterpret_cast<volatile uint16_t*>(sq)[slot] = (uint16_t)w;
        else atomicOr(err, kErrLocalQueue);
      }
    }
    return next;
  }
};

template <int TX, int TY, int TZ, int BS>
__global__ void __launch_bounds__(BS) terminal_pass_kernel(const float* __restrict__ f, int32_t* __restrict__ lab,
                                                           const VolDims V, int dir,
                                                           const uint8_t* __restrict__ dirty_in,
                                                           uint8_t* __restrict__ dirty_out, int* __restrict__ changed,
                                                           int* __restrict__ err) {
  using B = VBox<TX, TY, TZ>;
  constexpr int NL = B::NL;
  static_assert(NL < 65536, "local ids are 16-bit");
  extern __shared__ __align__(16) unsigned char s_dyn[];
  float* sf = reinterpret_cast<float*>(s_dyn);
  int32_t* sl = reinterpret_cast<int32_t*>(s_dyn + (size_t)NL * 4);
  // queue: NL pushes at most (a vertex is labelled once) plus one pending claim per thread
  constexpr int QCAP = NL + BS;
  uint16_t* sq = reinterpret_cast<uint16_t*>(s_dyn + (size_t)NL * 8);
  constexpr size_t VOFF = (size_t)NL * 8 + (size_t)QCAP * 2;
  uint32_t* s_vis = reinterpret_cast<uint32_t*>(s_dyn + VOFF + (VOFF % 4 ? 4 - VOFF % 4 : 0));
  uint32_t* s_dirty = s_vis + B::NW;
  __shared__ int s_qtail, s_border, s_head, s_done;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NWARPS = BS / 32;
  const int64_t ntx = (V.X + TX - 1) / TX, nty = (V.Y + TY - 1) / TY, ntz = (V.Z + TZ - 1) / TZ;
  const int64_t ntiles = ntx * nty * ntz;
  const bool first = (dirty_in == nullptr);
  TerminalWalk<B> W;
  W.sf = sf;
  W.sl = sl;
  W.sq = sq;
  W.vis = s_vis;
  W.dirty = s_dirty;
  W.qtail = &s_qtail;
  W.err = err;
  W.dir = dir;
  W.X = V.X;
  W.XY = V.X * V.Y;

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    if (!first && !dirty_in[tile]) continue;
    const int64_t tx = tile % ntx, ty = (tile / ntx) % nty, tz = tile / (ntx * nty);
    W.o[0] = tx * TX - B::H;
    W.o[1] = ty * TY - B::H;
    W.o[2] = tz * TZ - B::H;
    const int64_t vv[3] = {V.X, V.Y, V.Z};
    constexpr int LE[3] = {B::LX, B::LY, B::LZ};
#pragma unroll
    for (int a = 0; a < 3; a++) {
      W.lmin[a] = (int)(W.o[a] < 0 ? -W.o[a] : 0);
      const int64_t hi = vv[a] - W.o[a];
      W.lmax[a] = (int)(hi < LE[a] ? hi : LE[a]);
    }
    if (tid == 0) {
      s_qtail = 0;
      s_border = 0;
      s_head = 0;
      s_done = 0;
    }
    for (int w = tid; w < B::NW; w += BS) {
      s_vis[w] = 0;
      s_dirty[w] = 0;
    }
    for (int k = tid; k < QCAP; k += BS) sq[k] = kQueueEmpty;
    __syncthreads();
    // the box's rows in batches of kRowBatch per warp: every load of a batch is issued
    // before the first store, so a thread keeps 2 * kRowBatch * XI loads in flight
    // instead of waiting for one row's before it asks for the next
    constexpr int NROWS = B::LY * B::LZ, XI = (B::LX + 31) / 32, kRowBatch = 4;
    for (int r0 = warp; r0 < NROWS; r0 += NWARPS * kRowBatch) {
      float fv[kRowBatch][XI];
      int32_t lv[kRowBatch][XI];
#pragma unroll
      for (int u = 0; u < kRowBatch; u++) {
        const int row = r0 + u * NWARPS;
        const int ly = row % B::LY, lz = row / B::LY;
        const bool rin = row < NROWS && ly >= W.lmin[1] && ly < W.lmax[1] && lz >= W.lmin[2] && lz < W.lmax[2];
        const int64_t rbase = W.o[0] + V.X * (W.o[1] + ly) + V.X * V.Y * (W.o[2] + lz);
#pragma unroll
        for (int q = 0; q < XI; q++) {
          const int lx = lane + 32 * q;
          const bool in = rin && lx < B::LX && lx >= W.lmin[0] && lx < W.lmax[0];
          fv[u][q] = in ? f[rbase + lx] : 0.f;
          lv[u][q] = in ? lab[rbase + lx] : -1;
        }
      }
#pragma unroll
      for (int u = 0; u < kRowBatch; u++) {
        const int row = r0 + u * NWARPS;
        if (row >= NROWS) break;  // (warp-uniform)
        const int ly = row % B::LY, lz = row / B::LY;
        const bool row_halo = ly < B::H || ly >= B::H + TY || lz < B::H || lz >= B::H + TZ;
#pragma unroll
        for (int q = 0; q < XI; q++) {
          const int lx = lane + 32 * q;
          if (lx >= B::LX) continue;
          const int i = lx + B::LX * row;
          const int32_t l = lv[u][q];
          sf[i] = fv[u][q];
          sl[i] = l;
          if (l < 0) continue;
          if (!first && !(row_halo || lx < B::H || lx >= B::H + TX)) continue;
          atomicOr(&s_vis[i >> 5], 1u << (i & 31));
          sq[atomicAdd(&s_qtail, 1)] = (uint16_t)i;
        }
      }
    }
    __syncthreads();
    // The walk's fixpoint does not depend on the order, so instead of breadth-first
    // levels separated by barriers (threads idled at each barrier behind the longest
    // chain) every thread claims the next queue slot as soon as its chain ends.  Slots
    // are filled in the order they are reserved (s_qtail); a thread whose slot is not
    // filled yet waits, and all stop once every reserved item is done (s_done ==
    // s_qtail) with their slots beyond the last one: an item counts as done only after
    // its chain has reserved whatever it pushes, so no work is in flight then.
    {
      int h = atomicAdd(&s_head, 1);
      volatile uint16_t* vq = sq;
      volatile int* vdone = &s_done;
      volatile int* vtail = &s_qtail;
      for (uint32_t spin = 0;; spin++) {
        const uint16_t it = h < QCAP ? (uint16_t)vq[h] : (uint16_t)kQueueEmpty;
        if (it != kQueueEmpty) {
          int cur = it;
          while (cur >= 0) cur = W.step(cur);
          __threadfence_block();
          atomicAdd(&s_done, 1);
          h = atomicAdd(&s_head, 1);
          spin = 0;
          continue;
        }
        const int d = *vdone;
        const int t = *vtail;
        if (d == t && h >= t) break;
        if (spin > kQueueSpinLimit) {  // cannot happen by construction: report, stop
          atomicOr(err, kErrIterLimit);
          break;
        }
        __nanosleep(32);
      }
    }
    __syncthreads();
    for (int w = tid; w < B::NW; w += BS) {
      uint32_t m = s_dirty[w];
      while (m) {
        const int i = w * 32 + __ffs(m) - 1;
        m &= m - 1;
        const int lx = i % B::LX, ly = (i / B::LX) % B::LY, lz = i / (B::LX * B::LY);
        if (lx < B::H || lx >= B::H + TX || ly < B::H || ly >= B::H + TY || lz < B::H || lz >= B::H + TZ) continue;
        lab[(W.o[0] + lx) + V.X * (W.o[1] + ly) + V.X * V.Y * (W.o[2] + lz)] = sl[i];
        if (lx < 2 * B::H || lx >= TX || ly < 2 * B::H || ly >= TY || lz < 2 * B::H || lz >= TZ) s_border = 1;
      }
    }
    __syncthreads();
    if (s_border) {
      for (int k = tid; k < 27; k += BS) {
        const int64_t nx = tx + (k % 3) - 1, ny = ty + (k / 3) % 3 - 1, nz = tz + k / 9 - 1;
        if (k == 13 || nx < 0 || nx >= ntx || ny < 0 || ny >= nty || nz < 0 || nz >= ntz) continue;
        dirty_out[nx + ny * ntx + nz * ntx * nty] = 1;
      }
      if (tid == 0) atomicOr(changed, 1);
    }
    __syncthreads();
  }
}

// ---- K5b on a global frontier ---------------------------------------------------------
//
// A vertex joins a certain terminal region when all its earlier 6-neighbours carry that
// region's label (InspectPriorRegions), so its label is a function of its earlier
// neighbours' labels alone and the regions are the unique fixpoint, whatever the
// order of the inspections.  Here every newly labelled vertex inspects its later
// 6-neighbours in global memory, depth-first with a short per-thread stack (what does
// not fit goes to the next round's frontier); the first round starts from the seeds.
// A vertex that an inspection finds not yet decided is inspected again when its last
// earlier neighbour gets its label.  The labels are set by compare-and-swap from -1,
// so every vertex enters a frontier at most once.

// Comparer::Compare(a, b), "a comes before b": value, then index (ascending labels: the
// lower value; descending: the higher)
__device__ __forceinline__ bool walk_before(const float* __restrict__ f, int dir, int64_t a, int64_t b) {
  const float fa = f[a], fb = f[b];
  if (dir < 0) {
    if (fb > fa) return true;
    if (fa > fb) return false;
    return b > a;
  }
  if (fa > fb) return true;
  if (fb > fa) return false;
  return a > b;
}

__global__ void __launch_bounds__(128) terminal_walk_kernel(const float* __restrict__ f, int32_t* __restrict__ lab,
                                                            const VolDims V, int dir, const int64_t* __restrict__ qin,
                                                            const int* __restrict__ n_in, int64_t* __restrict__ qout,
                                                            int* __restrict__ n_out, int cap, int* __restrict__ err) {
  constexpr int SD = 16;
  const int n = *n_in;
  const int64_t X = V.X, XY = V.X * V.Y;
  const int64_t E[3] = {V.X, V.Y, V.Z};
  const int64_t S[3] = {1, V.X, XY};
  volatile int32_t* vl = lab;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    int64_t stack[SD];
    int sp = 0;
    stack[sp++] = qin[k];
    while (sp > 0) {
      const int64_t v = stack[--sp];
      const uint32_t u32 = (uint32_t)v, x32 = (uint32_t)X, y32 = (uint32_t)V.Y;  // fewer than 2^31 vertices
      const uint32_t r = u32 / x32;
      const int64_t vc[3] = {(int64_t)(u32 - r * x32), (int64_t)(r % y32), (int64_t)(r / y32)};
#pragma unroll
      for (int a = 0; a < 3; a++) {
#pragma unroll
        for (int s = 0; s < 2; s++) {
          const int64_t wa = vc[a] + (s == 0 ? 1 : -1);
          if (wa < 0 || wa >= E[a]) continue;
          const int64_t w = v + (s == 0 ? S[a] : -S[a]);
          if (vl[w] != -1 || !walk_before(f, dir, v, w)) continue;
          // InspectPriorRegions of w (gi_extrema_region_builder.h:806-857)
          int64_t wc[3] = {vc[0], vc[1], vc[2]};
          wc[a] = wa;
          int32_t l = -1;
          bool ok = true;
#pragma unroll
          for (int b = 0; b < 3 && ok; b++) {
#pragma unroll
            for (int t = 0; t < 2; t++) {
              const int64_t ua = wc[b] + (t == 0 ? 1 : -1);
              if (ua < 0 || ua >= E[b]) continue;
              const int64_t u = w + (t == 0 ? S[b] : -S[b]);
              if (!walk_before(f, dir, u, w)) continue;
              const int32_t lu = vl[u];
              if (lu < 0 || (l >= 0 && lu != l)) {
                ok = false;
                break;
              }
              l = lu;
            }
          }
          if (!ok || l < 0) continue;
          if (atomicCAS(&lab[w], -1, l) != -1) continue;
          if (sp < SD) {
            stack[sp++] = w;
          } else {
            const int slot = atomicAdd(n_out, 1);
            if (slot < cap) qout[slot] = w; else atomicOr(err, kErrLocalQueue);
          }
        }
      }
    }
  }
}

cudaError_t launch_terminal_walk(const float* f, int32_t* lab, const VolDims& V, int dir, const int64_t* qin,
                                 const int* n_in, int n_host, int64_t* qout, int* n_out, int cap, int* err,
                                 int num_sms, cudaStream_t stream) {
  if (n_host <= 0) return cudaSuccess;
  const int blocks = (n_host + 127) / 128;
  const int grid = blocks < num_sms * 16 ? blocks : num_sms * 16;
  ::msc::count_launch();
  terminal_walk_kernel<<<grid, 128, 0, stream>>>(f, lab, V, dir, qin, n_in, qout, n_out, cap, err);
  return cudaGetLastError();
}

namespace {
constexpr int kVTX = 32, kVTY = 16, kVTZ = 8, kVBS = 512;
using VB = VBox<kVTX, kVTY, kVTZ>;
}  // namespace

int64_t terminal_num_tiles(const VolDims& V) {
  return ((V.X + kVTX - 1) / kVTX) * ((V.Y + kVTY - 1) / kVTY) * ((V.Z + kVTZ - 1) / kVTZ);
}

cudaError_t launch_terminal_pass(const float* f, int32_t* lab, const VolDims& V, int dir, const uint8_t* dirty_in,
                                 uint8_t* dirty_out, int* changed, int* err, int num_sms, cudaStream_t stream) {
  const int64_t nt = terminal_num_tiles(V);
  const int64_t cap = (int64_t)num_sms * 2;
  const int grid = (int)(nt < cap ? nt : cap);
  if (grid <= 0) return cudaSuccess;
  // walkers per tile: MSC_TERMINAL_THREADS (256 or 512) overrides the default for tuning
  static const int bs = [] {
    const char* e = std::getenv("MSC_TERMINAL_THREADS");
    return (e && std::atoi(e) == 256) ? 256 : kVBS;
  }();
  auto k = bs == 256 ? terminal_pass_kernel<kVTX, kVTY, kVTZ, 256> : terminal_pass_kernel<kVTX, kVTY, kVTZ, kVBS>;
  const size_t sm = VB::smem_bytes() + (size_t)bs * 2 + 16;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  ::msc::count_launch();
  k<<<grid, bs, sm, stream>>>(f, lab, V, dir, dirty_in, dirty_out, changed, err);
  return cudaGetLastError();
}

cudaError_t launch_find_critical(const uint8_t* g, const VolDims& V, int dir, int32_t* ext_id_of_key,
                                 int64_t* ext_cells, int* n_ext, int64_t* saddles, int* n_sad, int num_sms,
                                 cudaStream_t stream) {
  ::msc::count_launch();
  find_critical_kernel<<<num_sms * 8, 256, 0, stream>>>(g, V, dir, ext_id_of_key, ext_cells, n_ext, saddles, n_sad);
  return cudaGetLastError();
}

cudaError_t launch_trace_arcs(const uint8_t* g, const float* f, const VolDims& V, int dir, const int64_t* saddles,
                              int n_sad, const int32_t* ext_id_of_key, float threshold, Arc* arcs, int* n_arcs,
                              int* err, int num_sms, cudaStream_t stream) {
  if (n_sad <= 0) return cudaSuccess;
  const int blocks = (n_sad + 255) / 256;
  ::msc::count_launch();
  trace_arcs_kernel<<<blocks < num_sms * 8 ? blocks : num_sms * 8, 256, 0, stream>>>(
      g, f, V, dir, saddles, n_sad, ext_id_of_key, threshold, arcs, n_arcs, err);
  return cudaGetLastError();
}

cudaError_t launch_extremum_info(const float* f, const VolDims& V, int dir, const int64_t* ext_cells, int n_ext,
                                 int64_t* hv, float* fval, int64_t* seed, int num_sms, cudaStream_t stream) {
  if (n_ext <= 0) return cudaSuccess;
  const int blocks = (n_ext + 255) / 256;
  ::msc::count_launch();
  extremum_info_kernel<<<blocks < num_sms * 8 ? blocks : num_sms * 8, 256, 0, stream>>>(f, V, dir, ext_cells, n_ext,
                                                                                         hv, fval, seed);
  return cudaGetLastError();
}

cudaError_t launch_group_seeds(const int32_t* rep, const int64_t* seed, int n_ext, int32_t* name, int32_t* lab,
                               uint8_t* state, int num_sms, cudaStream_t stream) {
  if (n_ext <= 0) return cudaSuccess;
  const int blocks = (n_ext + 255) / 256;
  const int grid = blocks < num_sms * 8 ? blocks : num_sms * 8;
  ::msc::count_launch();
  group_name_kernel<<<grid, 256, 0, stream>>>(rep, seed, n_ext, name);
  ::msc::count_launch();
  place_seeds_kernel<<<grid, 256, 0, stream>>>(rep, seed, n_ext, name, lab, state);
  return cudaGetLastError();
}

}  // namespace msc
