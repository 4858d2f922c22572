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
// GPU form: repeated passes of a tile kernel.  A CTA stages a tile of .grad bytes
// plus a 2-cell halo in shared memory (every rule reaches at most 2 cells), seeds a
// shared-memory queue with the marked items, runs the value-2 walk to its local
// fixpoint, then the value-1 walk, and writes back the tile's changed bytes.  Marks
// in the halo stay local.  The first pass seeds every marked item; later passes only
// revisit tiles whose halo changed (a neighbour wrote a cell within 2 cells of the
// shared border) and seed only from the halo, because everything reachable from the
// interior was already walked.  The closure is complete when a pass changes no cell
// near any tile border.
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
  // dynamic shared memory: queue (u16) | bytes | visited bits | changed bits
  static constexpr size_t smem_bytes() { return (size_t)NL * 2 + ((NL + 3) / 4) * 4 + (size_t)NW * 8; }
};

// local index -> local coords
template <class T>
__device__ __forceinline__ void lcoords(int i, int& lx, int& ly, int& lz) {
  lx = i % T::LX;
  ly = (i / T::LX) % T::LY;
  lz = i / (T::LX * T::LY);
}

template <int ND, int TX, int TY, int TZ, int BS>
__global__ void __launch_bounds__(BS) ldir_pass_kernel(uint8_t* __restrict__ g, const GradDims D,
                                                       const uint8_t* __restrict__ dirty_in,
                                                       uint8_t* __restrict__ dirty_out,
                                                       int* __restrict__ changed, int* __restrict__ err) {
  using T = LdirTile<ND, TX, TY, TZ>;
  constexpr int NL = T::NL;
  static_assert(NL < 65536, "local ids are 16-bit");
  extern __shared__ __align__(16) unsigned char s_dyn[];
  uint16_t* sq = reinterpret_cast<uint16_t*>(s_dyn);
  uint8_t* sg = s_dyn + (size_t)NL * 2;
  uint32_t* s_vis = reinterpret_cast<uint32_t*>(s_dyn + (size_t)NL * 2 + ((NL + 3) / 4) * 4);
  uint32_t* s_dirty = s_vis + T::NW;
  __shared__ int s_qtail, s_border;

  const int tid = threadIdx.x;
  const int64_t dX = D.d[0], dY = D.d[1], dZ = D.d[2];
  const int64_t ntx = (dX + TX - 1) / TX, nty = (dY + TY - 1) / TY;
  const int64_t ntz = (ND == 3) ? (dZ + TZ - 1) / TZ : 1;
  const int64_t ntiles = ntx * nty * ntz;

  const bool first = (dirty_in == nullptr);
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    if (!first && !dirty_in[tile]) continue;
    const int64_t tx = tile % ntx, ty = (tile / ntx) % nty, tz = (ND == 3) ? tile / (ntx * nty) : 0;
    const int64_t ox = tx * TX - T::H;
    const int64_t oy = ty * TY - T::H;
    const int64_t oz = (ND == 3) ? tz * TZ - T::H : 0;

    // stage the tile + halo; cells outside the complex read as 0 (unassigned)
    for (int i = tid; i < NL; i += BS) {
      int lx, ly, lz;
      lcoords<T>(i, lx, ly, lz);
      const int64_t gx = ox + lx, gy = oy + ly, gz = oz + lz;
      uint8_t b = 0;
      if (gx >= 0 && gx < dX && gy >= 0 && gy < dY && gz >= 0 && gz < dZ)
        b = g[gx + gy * D.cs[1] + gz * D.cs[2]];
      sg[i] = b;
    }
    for (int w = tid; w < T::NW; w += BS) s_dirty[w] = 0;
    if (tid == 0) s_border = 0;

    // two walks: value 2 over edge items, then value 1 over quad items
#pragma unroll 1
    for (int phase = 0; phase < 2; phase++) {
      const int item_dim = phase == 0 ? 1 : 2;
      const unsigned value = phase == 0 ? 2u : 1u;
      for (int w = tid; w < T::NW; w += BS) s_vis[w] = 0;
      if (tid == 0) s_qtail = 0;
      __syncthreads();
      // seeds: every marked item of this walk in the staged box (first pass), or in
      // its halo only (later passes: the interior was walked already)
      for (int i = tid; i < NL; i += BS) {
        const uint8_t b = sg[i];
        if (!(b & 1u) || (unsigned)(b >> 5) != value) continue;
        int lx, ly, lz;
        lcoords<T>(i, lx, ly, lz);
        if (!first && lx >= T::H && lx < T::H + TX && ly >= T::H && ly < T::H + TY &&
            (ND == 2 || (lz >= T::H && lz < T::H + TZ)))
          continue;
        const int dim = (int)((ox + lx) & 1) + (int)((oy + ly) & 1) + (ND == 3 ? (int)((oz + lz) & 1) : 0);
        if (dim != item_dim) continue;
        atomicOr(&s_vis[i >> 5], 1u << (i & 31));
        sq[atomicAdd(&s_qtail, 1)] = (uint16_t)i;
      }
      __syncthreads();
      int start = 0;
#pragma unroll 1
      while (true) {
        const int end = s_qtail;
        __syncthreads();
        if (start == end) break;
        for (int k = start + tid; k < end; k += BS) {
          const int i = sq[k];
          int lc[3];
          lcoords<T>(i, lc[0], lc[1], lc[2]);
          const int64_t gc[3] = {ox + lc[0], oy + lc[1], oz + lc[2]};
          const int lext[3] = {T::LX, T::LY, T::LZ};
#pragma unroll
          for (int a = 0; a < ND; a++) {
            if (gc[a] & 1) continue;  // cofacets only along even axes
#pragma unroll
            for (int s = 0; s < 2; s++) {
              const int sgn = s == 0 ? 1 : -1;  // +axis first, as CofacetsIterator
              const int64_t ga = gc[a] + sgn;
              const int la = lc[a] + sgn;
              if (ga < 0 || ga >= D.d[a] || la < 0 || la >= lext[a]) continue;
              const int t = i + sgn * T::ls(a);
              const uint8_t bt = sg[t];
              const unsigned code = (bt >> 2) & 7u;
              if (!(bt & 1u) || code == 7u) continue;  // unassigned or critical
              // the cofacet itself is marked whatever its partner is
              if (phase == 0) {
                // t is a quad: 3 -> 2; a 1 from the value-1 walk is final
                if ((bt >> 5) == 3u) {
                  sg[t] = (uint8_t)((bt & 0x1Fu) | (2u << 5));
                  atomicOr(&s_dirty[t >> 5], 1u << (t & 31));
                }
              } else {
                // t is a hex: -> 1
                if ((bt >> 5) != 1u) {
                  sg[t] = (uint8_t)((bt & 0x1Fu) | (1u << 5));
                  atomicOr(&s_dirty[t >> 5], 1u << (t & 31));
                }
              }
              // pair(t): decode the stored direction to the true axis
              const int pc = map3(D.dec_map, (int)code);
              const int pa = pc >> 1, psg = (pc & 1) ? -1 : 1;
              int lpc[3] = {lc[0], lc[1], lc[2]};
              lpc[a] += sgn;
              lpc[pa] += psg;
              if (lpc[pa] < 0 || lpc[pa] >= lext[pa]) continue;  // partner outside the box
              const int tp = t + psg * T::ls(pa);
              if (tp == i) continue;
              const uint8_t bp = sg[tp];
              if (phase == 0) {
                if ((bp >> 5) != 3u) continue;  // already marked: seeded or queued
                const int pdim = (int)((gc[0] + (lpc[0] - lc[0])) & 1) + (int)((gc[1] + (lpc[1] - lc[1])) & 1) +
                                 (ND == 3 ? (int)((gc[2] + (lpc[2] - lc[2])) & 1) : 0);
                if (pdim != 1) {
                  sg[tp] = (uint8_t)((bp & 0x1Fu) | (2u << 5));  // hex: the path ends here
                  atomicOr(&s_dirty[tp >> 5], 1u << (tp & 31));
                  continue;
                }
              } else {
                if ((bp >> 5) == 1u) continue;
              }
              const uint32_t bit = 1u << (tp & 31);
              if (atomicOr(&s_vis[tp >> 5], bit) & bit) continue;
              sg[tp] = (uint8_t)((bp & 0x1Fu) | (value << 5));
              atomicOr(&s_dirty[tp >> 5], 1u << (tp & 31));
              const int slot = atomicAdd(&s_qtail, 1);
              if (slot < NL) sq[slot] = (uint16_t)tp; else atomicOr(err, kErrLocalQueue);
            }
          }
        }
        __syncthreads();
        start = end;
      }
    }

    // write back the tile interior
    for (int i = tid; i < NL; i += BS) {
      if (!((s_dirty[i >> 5] >> (i & 31)) & 1u)) continue;
      const uint8_t b = sg[i];
      int lx, ly, lz;
      lcoords<T>(i, lx, ly, lz);
      if (lx < T::H || lx >= T::H + TX || ly < T::H || ly >= T::H + TY) continue;
      if (ND == 3 && (lz < T::H || lz >= T::H + TZ)) continue;
      const int64_t gx = ox + lx, gy = oy + ly, gz = oz + lz;
      g[gx + gy * D.cs[1] + gz * D.cs[2]] = b;
      // a change within reach (2 cells) of a neighbour's halo reopens that neighbour
      if (lx < 2 * T::H || lx >= TX || ly < 2 * T::H || ly >= TY || (ND == 3 && (lz < 2 * T::H || lz >= TZ)))
        s_border = 1;
    }
    __syncthreads();
    if (s_border) {
      // reopen the existing neighbour tiles for the next pass
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
    k<<<grid, kBS3, sm, stream>>>(g, D, dirty_in, dirty_out, changed, err);
  } else {
    auto k = ldir_pass_kernel<2, kTX2, kTY2, 1, kBS2>;
    const size_t sm = Tile2::smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k<<<grid, kBS2, sm, stream>>>(g, D, dirty_in, dirty_out, changed, err);
  }
  return cudaGetLastError();
}

}  // namespace msc
