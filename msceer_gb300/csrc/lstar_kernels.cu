// K1: lower-star discrete gradient, one thread per vertex (sm_103a).
//
// Replaces, with identical output bytes:
//   RegularGridMaxMinVertexLabeling3D::ComputeOutput   gi_max_vertex_labeling.h:1119-1339
//   SlidingWindowRobinsNoalloc::ComputePairing_sliding gi_fast_robins_noalloc.h:1254-1535
//     (interior: ComputeLowerStar :353-428, HomotopyExpand :147-321)
//   MyRobinsNoalloc<...,5,4>::ComputeLowerStar          gi_modified_robins.h:1281-1343
//     (boundary planes, lower star split by cell boundaryValue)
//   2D: RegularGridMaxMinVertexLabeling2D + MyRobinsNoalloc<TopologicalRegularGrid2D,...,4,6>
//       ::ComputePairing (gi_modified_robins.h:1344-1402)
// and the parts of setAscendingManifoldDimensions / outputToFile that are local to a
// cell: the boundary flag and the ldir value of critical cells (the roots of the
// ascending-manifold closure, finished by ldir_kernels.cu).
//
// Design: the max/min vertex labeling is never materialised.  A thread loads the
// 3^ND neighbourhood of its vertex, builds the bitmask of neighbours that come
// before it in the (value, index) order, and derives the lower star (cells whose
// every other vertex is lower) with three separable AND-folds.  The homotopy
// expansion then runs on 27-bit masks: processed set P, critical set K and three
// bit-planes of pair codes.  Neighbour values live in a per-thread shared-memory
// column so the lowest-vertex comparisons can index them.  Each cell is owned by
// exactly one vertex (its highest), so the final byte is written once with a plain
// store; the 27 stores of a warp for one neighbour position fall in one 64-byte span.
#include "msc_device.cuh"

namespace msc {

template <int ND>
struct Nb {
  static constexpr int NPOS = (ND == 3) ? 27 : 9;
  static constexpr int CENTER = (ND == 3) ? 13 : 4;
  __host__ __device__ static constexpr int d(int p, int a) {
    return a == 0 ? p % 3 - 1 : (a == 1 ? (p / 3) % 3 - 1 : p / 9 - 1);
  }
  __host__ __device__ static constexpr int stride(int a) { return a == 0 ? 1 : (a == 1 ? 3 : 9); }
  __host__ __device__ static constexpr int dim(int p) {
    int s = 0;
    for (int a = 0; a < ND; a++) s += d(p, a) != 0;
    return s;
  }
  __host__ __device__ static constexpr uint32_t dim_mask(int k) {
    uint32_t m = 0;
    for (int p = 0; p < NPOS; p++) if (dim(p) == k) m |= 1u << p;
    return m;
  }
  __host__ __device__ static constexpr uint32_t axis_mask(int a, int val) {
    uint32_t m = 0;
    for (int p = 0; p < NPOS; p++) if (d(p, a) == val) m |= 1u << p;
    return m;
  }
  // facets of cell p that lie in the star: one per odd axis, toward the centre
  __host__ __device__ static constexpr uint32_t facet_mask(int p) {
    uint32_t m = 0;
    for (int a = 0; a < ND; a++) if (d(p, a) != 0) m |= 1u << (p - d(p, a) * stride(a));
    return m;
  }
  // cofacets in CofacetsIterator order (+x,-x,+y,-y,+z,-z over even axes),
  // 5 bits each, 31 terminates
  __host__ __device__ static constexpr uint32_t cofacet_list(int p) {
    uint32_t m = 0;
    int n = 0;
    for (int a = 0; a < ND; a++) {
      if (d(p, a) == 0) {
        m |= (uint32_t)(p + stride(a)) << (5 * n); n++;
        m |= (uint32_t)(p - stride(a)) << (5 * n); n++;
      }
    }
    for (; n < 6; n++) m |= 31u << (5 * n);
    return m;
  }
  // vertices of cell p (positions whose offsets are 0 or equal to p's on every axis)
  __host__ __device__ static constexpr uint32_t vertex_mask(int p) {
    uint32_t m = 0;
    for (int q = 0; q < NPOS; q++) {
      bool ok = true;
      for (int a = 0; a < ND; a++) ok = ok && (d(q, a) == 0 || d(q, a) == d(p, a));
      if (ok) m |= 1u << q;
    }
    return m;
  }
  // AND-fold: keep bit p only if the bit of p with axis A zeroed is also set
  template <int A>
  __device__ static __forceinline__ uint32_t fold(uint32_t m) {
    constexpr int s = stride(A);
    constexpr uint32_t mp = axis_mask(A, 1), mm = axis_mask(A, -1), m0 = axis_mask(A, 0);
    return m & (((m << s) & mp) | ((m >> s) & mm) | m0);
  }
};

template <int ND>
struct NbTables {
  uint32_t fm[27], cof[27], vm[27];
};

template <int ND>
constexpr NbTables<ND> make_tables() {
  NbTables<ND> t{};
  for (int p = 0; p < 27; p++) {
    t.fm[p] = p < Nb<ND>::NPOS ? Nb<ND>::facet_mask(p) : 0u;
    t.cof[p] = p < Nb<ND>::NPOS ? Nb<ND>::cofacet_list(p) : 0xFFFFFFFFu;
    t.vm[p] = p < Nb<ND>::NPOS ? Nb<ND>::vertex_mask(p) : 0u;
  }
  return t;
}

__constant__ NbTables<3> c_tab3 = make_tables<3>();
__constant__ NbTables<2> c_tab2 = make_tables<2>();

template <int ND, int BS>
struct LStarThread {
  using N = Nb<ND>;
  const float* sv;          // this thread's neighbourhood column, stride BS
  const uint32_t* fm;
  const uint32_t* cof;
  const uint32_t* vm;
  uint32_t P = 0, K = 0, C0 = 0, C1 = 0, C2 = 0;

  __device__ __forceinline__ float val(int p) const { return sv[p * BS]; }

  // Cell2LowestVertex: the first vertex of the cell in the (value, index) order
  __device__ __forceinline__ int lowv(int q) const {
    uint32_t m = vm[q];
    int best = __ffs(m) - 1;
    float fb = val(best);
    m &= m - 1;
    while (m) {
      int p = __ffs(m) - 1;
      m &= m - 1;
      float fp = val(p);
      if (before(fp, p, fb, best)) { best = p; fb = fp; }
    }
    return best;
  }

  __device__ __forceinline__ void set_code(int q, int code) {
    C0 |= (uint32_t)(code & 1) << q;
    C1 |= (uint32_t)((code >> 1) & 1) << q;
    C2 |= (uint32_t)((code >> 2) & 1) << q;
  }
  __device__ __forceinline__ static int dir_code(int delta) {
    int ad = delta < 0 ? -delta : delta;
    return (delta < 0 ? 1 : 0) | (ad == 3 ? 2 : (ad == 9 ? 4 : 0));
  }
  __device__ __forceinline__ void make_pair(int q, int r) {
    P |= (1u << q) | (1u << r);
    set_code(q, dir_code(r - q));
    set_code(r, dir_code(q - r));
  }
  __device__ __forceinline__ void make_critical(int q) {
    P |= 1u << q;
    K |= 1u << q;
  }

  // HomotopyExpand of one boundary class S of the lower star
  // (gi_fast_robins_noalloc.h:147-321, gi_modified_robins.h:999-1199).
  __device__ void expand(uint32_t S) {
    constexpr int C = N::CENTER;
    if (S & (1u << C)) {
      // pair the vertex with the edge to its lowest neighbour (steepest descent)
      constexpr uint32_t EDGES = N::dim_mask(1);
      uint32_t E = S & EDGES;
      if (!E) {
        make_critical(C);
      } else {
        int best = __ffs(E) - 1;
        float fb = val(best);
        E &= E - 1;
        while (E) {
          int e = __ffs(E) - 1;
          E &= E - 1;
          float fe = val(e);
          if (before(fe, e, fb, best)) { best = e; fb = fe; }
        }
        make_pair(C, best);
      }
    }
#pragma unroll 1
    for (int dd = 1; dd <= ND; dd++) {
      constexpr uint32_t DM1 = N::dim_mask(1), DM2 = N::dim_mask(2), DM3 = N::dim_mask(3);
      uint32_t U = S & (dd == 1 ? DM1 : (dd == 2 ? DM2 : DM3)) & ~P;
      while (U) {
        bool found = false;
        for (uint32_t W = U; W; W &= W - 1) {
          const int q = __ffs(W) - 1;
          uint32_t cl = cof[q];
          int best = -1, bestlv = -1;
          float fbest = 0.f;
          for (int k = 0; k < 6; k++) {
            const int c = (int)(cl & 31u);
            cl >>= 5;
            if (c == 31) break;
            if (!((S >> c) & 1u)) continue;
            if (__popc(fm[c] & S & ~P) != 1) continue;  // num_missing == 1
            if (best < 0) {
              best = c;
            } else {
              // PickLowestCandidate: first wins ties (gi_fast_robins_noalloc.h:130-143)
              if (bestlv < 0) { bestlv = lowv(best); fbest = val(bestlv); }
              const int lv = lowv(c);
              const float fl = val(lv);
              if (before(fl, lv, fbest, bestlv)) { best = c; bestlv = lv; fbest = fl; }
            }
          }
          if (best >= 0) {
            make_pair(q, best);
            U &= ~(1u << q);
            found = true;
            break;  // restart the scan from the first cell
          }
        }
        if (!found) {
          // no pair possible: the unpaired cell with the lowest lowest-vertex becomes critical
          int q = __ffs(U) - 1;
          uint32_t W = U & (U - 1);
          if (W) {
            int lv = lowv(q);
            float fl = val(lv);
            while (W) {
              const int o = __ffs(W) - 1;
              W &= W - 1;
              const int olv = lowv(o);
              const float fo = val(olv);
              if (before(fo, olv, fl, lv)) { q = o; lv = olv; fl = fo; }
            }
          }
          make_critical(q);
          U &= ~(1u << q);
        }
      }
    }
  }
};

// One thread per vertex.  Block = BS threads = 32 consecutive x by BS/32 (y,z) rows;
// grid-stride over (x-block, row-block) pairs.
template <int ND, int BS>
__global__ void __launch_bounds__(BS) lstar_kernel(const float* __restrict__ f, uint8_t* __restrict__ g,
                                                   const GradDims D, int* __restrict__ err) {
  using N = Nb<ND>;
  constexpr int NPOS = N::NPOS;
  constexpr int C = N::CENTER;
  constexpr int ROWS = BS / 32;
  __shared__ float s_val[NPOS * BS];
  __shared__ uint32_t s_fm[NPOS], s_cof[NPOS], s_vm[NPOS];
  const int tid = threadIdx.x;
  if (tid < NPOS) {
    if constexpr (ND == 3) {
      s_fm[tid] = c_tab3.fm[tid]; s_cof[tid] = c_tab3.cof[tid]; s_vm[tid] = c_tab3.vm[tid];
    } else {
      s_fm[tid] = c_tab2.fm[tid]; s_cof[tid] = c_tab2.cof[tid]; s_vm[tid] = c_tab2.vm[tid];
    }
  }
  __syncthreads();

  const int64_t X = D.v[0], Y = D.v[1], Z = D.v[2];
  const int64_t nrows = Y * Z;
  const int64_t xblocks = (X + 31) / 32;
  const int64_t nblocks = xblocks * ((nrows + ROWS - 1) / ROWS);
  const int lane = tid & 31, row = tid >> 5;
  const int64_t cs1 = D.cs[1], cs2 = D.cs[2];
  float* sv = s_val + tid;

  for (int64_t blk = blockIdx.x; blk < nblocks; blk += gridDim.x) {
    const int64_t x = (blk % xblocks) * 32 + lane;
    const int64_t r = (blk / xblocks) * ROWS + row;
    if (x >= X || r >= nrows) continue;
    const int64_t y = r % Y, z = r / Y;
    const int64_t vidx = x + X * r;
    const float fc = __ldg(f + vidx);
    sv[C * BS] = fc;
    uint32_t lower = 0;
    bool nan = (fc != fc);
#pragma unroll
    for (int p = 0; p < NPOS; p++) {
      if (p == C) continue;
      const int dx = N::d(p, 0), dy = N::d(p, 1), dz = (ND == 3) ? N::d(p, 2) : 0;
      const bool ok = (x + dx >= 0) && (x + dx < X) && (y + dy >= 0) && (y + dy < Y) &&
                      (ND == 2 || ((z + dz >= 0) && (z + dz < Z)));
      if (ok) {
        const float v = __ldg(f + vidx + dx + dy * X + dz * X * Y);
        sv[p * BS] = v;
        nan |= (v != v);
        if (before(v, p, fc, C)) lower |= 1u << p;
      }
    }
    if (nan) atomicOr(err, kErrNaN);

    // lower star: cells all of whose other vertices are lower (out-of-range
    // neighbours are never lower, so cells outside the complex drop out too)
    uint32_t L = lower | (1u << C);
    L = N::template fold<0>(L);
    L = N::template fold<1>(L);
    if constexpr (ND == 3) L = N::template fold<2>(L);

    // boundary classes: boundaryValue = number of axes on which the cell sits on
    // the first or last plane (gi_topological_regular_grid.h:1291-1297)
    constexpr uint32_t A0x = N::axis_mask(0, 0), A0y = N::axis_mask(1, 0), A0z = N::axis_mask(2, 0);
    const uint32_t B0 = (x == 0 || x == X - 1) ? A0x : 0u;
    const uint32_t B1 = (y == 0 || y == Y - 1) ? A0y : 0u;
    const uint32_t B2 = (ND == 3 && (z == 0 || z == Z - 1)) ? A0z : 0u;
    const uint32_t Bany = B0 | B1 | B2;

    LStarThread<ND, BS> t{sv, s_fm, s_cof, s_vm};
    if (!Bany) {
      t.expand(L);
    } else {
      const uint32_t all3 = B0 & B1 & B2;
      const uint32_t two = ((B0 & B1) | (B0 & B2) | (B1 & B2)) & ~all3;
      const uint32_t one = (B0 ^ B1 ^ B2) & ~all3;
      const uint32_t cls[4] = {L & ~Bany, L & one, L & two, L & all3};
#pragma unroll 1
      for (int k = 0; k < 4; k++)
        if (cls[k]) t.expand(cls[k]);
    }

    const int64_t cbase = 2 * x + 2 * y * cs1 + 2 * z * cs2;
#pragma unroll
    for (int p = 0; p < NPOS; p++) {
      if (!((L >> p) & 1u)) continue;
      const int dx = N::d(p, 0), dy = N::d(p, 1), dz = (ND == 3) ? N::d(p, 2) : 0;
      const bool crit = (t.K >> p) & 1u;
      const int lc = (int)(((t.C0 >> p) & 1u) | (((t.C1 >> p) & 1u) << 1) | (((t.C2 >> p) & 1u) << 2));
      const int code = crit ? 7 : map3(D.enc_map, lc);
      const int dimp = N::dim(p);
      // ascending-manifold roots: critical 1-cells -> 2, critical 2-cells -> 1,
      // critical 3-cells -> 0 (gi_topological_gradient_using_algorithms.h:460-477)
      const int ldir = crit ? (dimp == 1 ? 2 : (dimp == 2 ? 1 : (dimp == 3 ? 0 : 3))) : 3;
      const int flag = (Bany >> p) & 1u;
      g[cbase + dx + dy * cs1 + dz * cs2] = (uint8_t)(1 | (flag << 1) | (code << 2) | (ldir << 5));
    }
  }
}

cudaError_t launch_lstar(int nd, const float* f, uint8_t* g, const GradDims& D, int* err, int num_sms,
                         cudaStream_t stream) {
  constexpr int BS = 128;
  const int64_t rows = D.v[1] * D.v[2];
  const int64_t nblocks = ((D.v[0] + 31) / 32) * ((rows + BS / 32 - 1) / (BS / 32));
  // persistent-ish grid: enough CTAs to fill every SM several times over
  const int64_t cap = (int64_t)num_sms * 16;
  const int grid = (int)(nblocks < cap ? nblocks : cap);
  if (grid <= 0) return cudaSuccess;
  if (nd == 3)
    lstar_kernel<3, BS><<<grid, BS, 0, stream>>>(f, g, D, err);
  else
    lstar_kernel<2, BS><<<grid, BS, 0, stream>>>(f, g, D, err);
  return cudaGetLastError();
}

}  // namespace msc
