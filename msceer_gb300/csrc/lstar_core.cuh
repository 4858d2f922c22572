// Per-vertex lower-star pairing on 27-bit (3D) / 9-bit (2D) neighbourhood masks.
// Host+device: the CUDA kernel (lstar_kernels.cu) runs it one thread per vertex and
// the CPU test harness (tests/lstar_core_host.cpp) runs the very same code against
// the oracle.
//
// Neighbourhood position p = (dx+1) + 3(dy+1) + 9(dz+1), offsets in {-1,0,1}: the
// order of TopologicalRegularGrid3D::AdjacentCellsIterator
// (gi_topological_regular_grid.h:196-205, 687-790).  The same index names the
// vertex at vertex offset (dx,dy,dz) and the cell at cell offset (dx,dy,dz) around
// the centre vertex; a cell's vertices are the positions whose offsets are 0 or
// equal to the cell's on every axis.
//
// HomotopyExpand (gi_fast_robins_noalloc.h:147-321; gi_modified_robins.h:999-1199)
// restated on sets.  With all lower-dimensional cells processed, a (d+1)-cell c is
// a pairing candidate for its d-facet q exactly when c is in the class S, not yet
// processed, and q is its only unprocessed facet in S (num_missing == 1).  Calling
// those cells "ready" (set R), the reference's restart-from-the-first-cell scan picks
// the first q, in star order, that is the remaining facet of some ready cell -- the
// lowest set bit of Q = facets(R) -- and pairs it with the ready cofacet whose lowest
// vertex comes first (cofacet order +x,-x,+y,-y,+z,-z, first wins ties,
// PickLowestCandidate :130-143).  With no ready cell, the unprocessed d-cell with the
// first lowest vertex becomes critical (:293-310).  Each step costs a few dozen bit
// operations instead of a rescan of the class.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define MSC_HD __host__ __device__ __forceinline__
#else
#define MSC_HD inline
#endif

namespace msc {

MSC_HD int ffs32(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return __ffs((int)x);
#else
  return __builtin_ffs((int)x);
#endif
}

MSC_HD int popc32(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return __popc(x);
#else
  return __builtin_popcount(x);
#endif
}

// The (value, then vertex index) order of IsGreater
// (gi_regular_grid_trilinear_function.h:309-314): a comes before (is lower than) b.
// Position order equals global vertex-index order inside a neighbourhood.
MSC_HD bool before(float fa, int a, float fb, int b) {
  if (fb > fa) return true;
  if (fa > fb) return false;
  return b > a;
}

MSC_HD uint32_t float_bits(float v) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(v);
#else
  uint32_t u;
  __builtin_memcpy(&u, &v, 4);
  return u;
#endif
}

// The same order as one integer: the value's order bits (negative zero taken as
// zero, as the float comparison does) above the neighbourhood position, so that
// key(a) < key(b) exactly when before(a, b).  Inputs are NaN-free (checked).
MSC_HD uint64_t order_key(float v, int p) {
  if (v == 0.0f) v = 0.0f;
  uint32_t u = float_bits(v);
  u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
  return ((uint64_t)u << 5) | (uint64_t)p;
}

template <int ND>
struct Nb {
  static constexpr int NPOS = (ND == 3) ? 27 : 9;
  static constexpr int CENTER = (ND == 3) ? 13 : 4;
  MSC_HD static constexpr int d(int p, int a) {
    return a == 0 ? p % 3 - 1 : (a == 1 ? (p / 3) % 3 - 1 : p / 9 - 1);
  }
  MSC_HD static constexpr int stride(int a) { return a == 0 ? 1 : (a == 1 ? 3 : 9); }
  MSC_HD static constexpr int dim(int p) {
    int s = 0;
    for (int a = 0; a < ND; a++) s += d(p, a) != 0;
    return s;
  }
  MSC_HD static constexpr uint32_t dim_mask(int k) {
    uint32_t m = 0;
    for (int p = 0; p < NPOS; p++)
      if (dim(p) == k) m |= 1u << p;
    return m;
  }
  MSC_HD static constexpr uint32_t axis_mask(int a, int val) {
    uint32_t m = 0;
    if (a >= ND) return val == 0 ? dim_mask(0) | dim_mask(1) | dim_mask(2) | dim_mask(3) : 0u;
    for (int p = 0; p < NPOS; p++)
      if (d(p, a) == val) m |= 1u << p;
    return m;
  }
  // vertices of cell p
  MSC_HD static constexpr uint32_t vertex_mask(int p) {
    uint32_t m = 0;
    for (int q = 0; q < NPOS; q++) {
      bool ok = true;
      for (int a = 0; a < ND; a++) ok = ok && (d(q, a) == 0 || d(q, a) == d(p, a));
      if (ok) m |= 1u << q;
    }
    return m;
  }
  // AND-fold along axis A: keep bit p only if the bit of p with axis A zeroed is set
  template <int A>
  MSC_HD static uint32_t fold(uint32_t m) {
    constexpr int s = stride(A);
    constexpr uint32_t mp = axis_mask(A, 1), mm = axis_mask(A, -1), m0 = axis_mask(A, 0);
    return m & (((m << s) & mp) | ((m >> s) & mm) | m0);
  }
  // bit c set when c's facet along axis A (the one toward the centre) is in m
  template <int A>
  MSC_HD static uint32_t facet_in(uint32_t m) {
    constexpr int s = stride(A);
    constexpr uint32_t mp = axis_mask(A, 1), mm = axis_mask(A, -1);
    return ((m << s) & mp) | ((m >> s) & mm);
  }
  // facets along axis A of the cells in r whose A-facet is flagged in f
  template <int A>
  MSC_HD static uint32_t facet_of(uint32_t r, uint32_t f) {
    constexpr int s = stride(A);
    constexpr uint32_t mp = axis_mask(A, 1), mm = axis_mask(A, -1);
    return ((r & f & mp) >> s) | ((r & f & mm) << s);
  }
};

// Per-cell key of the cell's lowest vertex (order_key), indexed by neighbourhood
// position.  Device: a per-thread column in shared memory; host: a plain array.
struct KeyCol {
  uint64_t* base;
  int stride;
  MSC_HD uint64_t operator()(int p) const { return base[p * stride]; }
};

template <int ND, class Keys>
struct LowerStarState {
  using N = Nb<ND>;
  Keys lk;             // lowest-vertex key per cell
  uint32_t P = 0;      // processed cells
  uint32_t K = 0;      // critical cells
  uint32_t C0 = 0, C1 = 0, C2 = 0;  // pair-direction code bit-planes

  MSC_HD explicit LowerStarState(Keys k) : lk(k) {}

  MSC_HD void set_code(int q, int code) {
    C0 |= (uint32_t)(code & 1) << q;
    C1 |= (uint32_t)((code >> 1) & 1) << q;
    C2 |= (uint32_t)((code >> 2) & 1) << q;
  }
  // direction code of the pair partner at delta = partner - cell: +x,-x,+y,-y,+z,-z
  MSC_HD static int dir_code(int delta) {
    const int ad = delta < 0 ? -delta : delta;
    return (delta < 0 ? 1 : 0) | (ad == 3 ? 2 : (ad == 9 ? 4 : 0));
  }
  MSC_HD void make_pair(int q, int r) {
    P |= (1u << q) | (1u << r);
    set_code(q, dir_code(r - q));
    set_code(r, dir_code(q - r));
  }
  MSC_HD void make_critical(int q) {
    P |= 1u << q;
    K |= 1u << q;
  }

  // the cell of U whose lowest vertex comes first (first in star order wins ties)
  MSC_HD int lowest_of(uint32_t U) const {
    int q = ffs32(U) - 1;
    uint64_t kb = lk(q);
    uint32_t W = U & (U - 1);
    while (W) {
      const int o = ffs32(W) - 1;
      W &= W - 1;
      const uint64_t ko = lk(o);
      if (ko < kb) {
        q = o;
        kb = ko;
      }
    }
    return q;
  }

  // HomotopyExpand of one boundary class S of the lower star.
  MSC_HD void expand(uint32_t S) {
    constexpr int C = N::CENTER;
    constexpr uint32_t EDGES = N::dim_mask(1);
    if (S & (1u << C)) {
      // the vertex pairs with the edge to its lowest neighbour (steepest descent)
      const uint32_t E = S & EDGES;
      if (!E) make_critical(C);
      else make_pair(C, lowest_of(E));  // an edge's lowest vertex is its other end
    }
    constexpr uint32_t DM1 = N::dim_mask(1), DM2 = N::dim_mask(2), DM3 = N::dim_mask(3);
    constexpr uint32_t AX0 = N::axis_mask(0, 0), AX1 = N::axis_mask(1, 0), AX2 = N::axis_mask(2, 0);
    // One step per iteration, always in the lowest dimension that still has
    // unprocessed cells -- the order of the reference's per-dimension loops -- so the
    // loop body is the same straight-line set algebra for every thread of a warp.
    for (int guard = 0; guard < N::NPOS; guard++) {
      const uint32_t A = S & ~P;  // unprocessed cells of the class
      if (!A) break;
      const bool d1 = (A & DM1) != 0u, d2 = !d1 && (A & DM2) != 0u;
      const uint32_t DMd = d1 ? DM1 : (d2 ? DM2 : DM3);
      const uint32_t DMu = d1 ? DM2 : (d2 ? DM3 : 0u);
      const uint32_t F0 = N::template facet_in<0>(A);
      const uint32_t F1 = N::template facet_in<1>(A);
      const uint32_t F2 = (ND == 3) ? N::template facet_in<2>(A) : 0u;
      const uint32_t one = (F0 ^ F1 ^ F2) & ~(F0 & F1 & F2);  // exactly one unprocessed facet
      const uint32_t R = A & DMu & one;                       // ready (d+1)-cells
      uint32_t Q = N::template facet_of<0>(R, F0) | N::template facet_of<1>(R, F1);
      if (ND == 3) Q |= N::template facet_of<2>(R, F2);
      if (Q) {
        const int q = ffs32(Q) - 1;
        // ready cofacets of q, i.e. its candidates
        uint32_t cm = 0;
#pragma unroll
        for (int a = 0; a < ND; a++) {
          const uint32_t even = a == 0 ? AX0 : (a == 1 ? AX1 : AX2);
          if ((even >> q) & 1u) cm |= (1u << (q + N::stride(a))) | (1u << (q - N::stride(a)));
        }
        cm &= R;
        int best = ffs32(cm) - 1;
        if (cm & (cm - 1)) {
          // several: the first in cofacet order (+x,-x,+y,-y,+z,-z) whose lowest
          // vertex comes first wins (PickLowestCandidate)
          best = -1;
          uint64_t kb = ~0ull;
#pragma unroll
          for (int a = 0; a < ND; a++) {
#pragma unroll
            for (int sgn = 0; sgn < 2; sgn++) {
              const int c = q + (sgn == 0 ? N::stride(a) : -N::stride(a));
              if (c < 0 || c >= N::NPOS || !((cm >> c) & 1u)) continue;
              const uint64_t kc = lk(c);
              if (best < 0 || kc < kb) {
                best = c;
                kb = kc;
              }
            }
          }
        }
        make_pair(q, best);
      } else {
        make_critical(lowest_of(A & DMd));
      }
    }
  }
};

// Lower star from the mask of neighbours that come before the centre: the cells all
// of whose other vertices are lower (three separable AND-folds).  Out-of-range
// neighbours are never "lower", so cells outside the complex drop out too.
template <int ND>
MSC_HD uint32_t lower_star_mask(uint32_t lower) {
  using N = Nb<ND>;
  uint32_t L = lower | (1u << N::CENTER);
  L = N::template fold<0>(L);
  L = N::template fold<1>(L);
  if (ND == 3) L = N::template fold<2>(L);
  return L;
}

// Runs every boundary class of one vertex's lower star.  bx/by/bz: the vertex lies
// on the first or last plane of that axis.  Class k = cells on the boundary of
// exactly k axes (boundaryValue, gi_topological_regular_grid.h:1291-1297; the split
// is MyRobinsNoalloc::ComputeLowerStar, gi_modified_robins.h:1305-1324).
template <int ND, class State>
MSC_HD uint32_t run_classes(State& st, uint32_t L, bool bx, bool by, bool bz) {
  using N = Nb<ND>;
  constexpr uint32_t A0x = N::axis_mask(0, 0), A0y = N::axis_mask(1, 0), A0z = N::axis_mask(2, 0);
  const uint32_t B0 = bx ? A0x : 0u;
  const uint32_t B1 = by ? A0y : 0u;
  const uint32_t B2 = (ND == 3 && bz) ? A0z : 0u;
  const uint32_t Bany = B0 | B1 | B2;
  if (!Bany) {
    st.expand(L);
  } else {
    const uint32_t all3 = B0 & B1 & B2;
    const uint32_t two = ((B0 & B1) | (B0 & B2) | (B1 & B2)) & ~all3;
    const uint32_t one = (B0 ^ B1 ^ B2) & ~all3;
    uint32_t c;
    if ((c = L & ~Bany)) st.expand(c);
    if ((c = L & one)) st.expand(c);
    if ((c = L & two)) st.expand(c);
    if ((c = L & all3)) st.expand(c);
  }
  return Bany;
}

// Final .grad byte of the cell at position p of a processed lower star.
//   code: 7 if critical, else the (axis-remapped) pair direction
//   ldir: roots of the ascending-manifold closure -- critical 1-cells 2, critical
//         2-cells 1, critical 3-cells 0 (gi_topological_gradient_using_algorithms.h:
//         460-477) -- and 3 everywhere else
//   flag: cell on the boundary (outputToFile, gi_discrete_gradient_labeling.h:206-211)
template <int ND, class State>
MSC_HD uint8_t cell_byte(const State& st, int p, uint32_t Bany, uint32_t enc_map) {
  const bool crit = (st.K >> p) & 1u;
  const int lc = (int)(((st.C0 >> p) & 1u) | (((st.C1 >> p) & 1u) << 1) | (((st.C2 >> p) & 1u) << 2));
  const int code = crit ? 7 : (int)((enc_map >> (3 * lc)) & 7u);
  const int dimp = Nb<ND>::dim(p);
  const int ldir = crit ? (dimp == 1 ? 2 : (dimp == 2 ? 1 : (dimp == 3 ? 0 : 3))) : 3;
  const int flag = (Bany >> p) & 1u;
  return (uint8_t)(1 | (flag << 1) | (code << 2) | (ldir << 5));
}

// First half of one vertex's work: gather its 3^ND neighbourhood through `load(p)`,
// write the cells' lowest-vertex keys to the column `col` (stride `cs`) and return the
// lower-star mask.  `interior`: the vertex is at least one vertex away from every face
// (no bounds checks).  `nan` is set if a NaN was seen.
template <int ND, class Load>
MSC_HD uint32_t lower_star_keys(int64_t x, int64_t y, int64_t z, int64_t X, int64_t Y, int64_t Z, bool interior,
                                const Load& load, uint64_t* col, int cs, bool& nan) {
  using N = Nb<ND>;
  constexpr int NPOS = N::NPOS;
  constexpr int C = N::CENTER;
  float fc = 0.f;
  load(C, fc);
  uint64_t k[NPOS];  // vertex keys, folded below into the cells' lowest-vertex keys
  k[C] = order_key(fc, C);
  uint32_t lower = 0;
  nan = (fc != fc);
  if (interior) {
#pragma unroll
    for (int p = 0; p < NPOS; p++) {
      if (p == C) continue;
      float v = 0.f;
      load(p, v);
      nan |= (v != v);
      k[p] = order_key(v, p);
      if (k[p] < k[C]) lower |= 1u << p;
    }
  } else {
    // out-of-range neighbours are left out of `lower`, so no cell outside the
    // complex enters the lower star
    const uint32_t okx = (x > 0 ? N::axis_mask(0, -1) : 0u) | N::axis_mask(0, 0) | (x < X - 1 ? N::axis_mask(0, 1) : 0u);
    const uint32_t oky = (y > 0 ? N::axis_mask(1, -1) : 0u) | N::axis_mask(1, 0) | (y < Y - 1 ? N::axis_mask(1, 1) : 0u);
    const uint32_t okz = (ND == 2) ? ~0u
                                   : ((z > 0 ? N::axis_mask(2, -1) : 0u) | N::axis_mask(2, 0) |
                                      (z < Z - 1 ? N::axis_mask(2, 1) : 0u));
    const uint32_t ok = okx & oky & okz;
#pragma unroll
    for (int p = 0; p < NPOS; p++) {
      if (p == C) continue;
      k[p] = ~0ull;
      if (!((ok >> p) & 1u)) continue;
      float v = 0.f;
      load(p, v);
      nan |= (v != v);
      k[p] = order_key(v, p);
      if (k[p] < k[C]) lower |= 1u << p;
    }
  }
  // lowest vertex of every cell: a cell's vertices form the box between the centre
  // and the vertex at its own offset, so three separable min-folds give them all
#pragma unroll
  for (int a = 0; a < ND; a++) {
#pragma unroll
    for (int p = 0; p < NPOS; p++) {
      if (N::d(p, a) == 0) continue;
      const int q = p - N::d(p, a) * N::stride(a);
      if (k[q] < k[p]) k[p] = k[q];
    }
  }
#pragma unroll
  for (int p = 0; p < NPOS; p++) col[p * cs] = k[p];
  return lower_star_mask<ND>(lower);
}

// The bytes of every cell of a processed lower star L (owned by its vertex): assigned |
// flag | pair code (7 if critical) | ldir, where ldir is 2 / 1 / 0 for critical 1- / 2- /
// 3-cells and 3 otherwise (the roots of the ascending-manifold closure).
template <int ND, class State, class Store>
MSC_HD void store_cells(const State& st, uint32_t L, uint32_t Bany, uint32_t enc_map, const Store& store) {
  using N = Nb<ND>;
  constexpr int NPOS = N::NPOS;
  constexpr uint32_t D0 = N::dim_mask(0), D1 = N::dim_mask(1), D2 = N::dim_mask(2);
  const uint32_t K = st.K;
  uint32_t p0 = st.C0, p1 = st.C1, p2 = st.C2;
  if (enc_map != 0x2C688u) {  // not the identity (0,1,2,3,4,5): remap the non-critical codes
    uint32_t q0 = 0, q1 = 0, q2 = 0;
    uint32_t m = L & ~K;
    while (m) {
      const int p = ffs32(m) - 1;
      m &= m - 1;
      const int lc = (int)(((p0 >> p) & 1u) | (((p1 >> p) & 1u) << 1) | (((p2 >> p) & 1u) << 2));
      const uint32_t e = (enc_map >> (3 * lc)) & 7u;
      q0 |= (e & 1u) << p;
      q1 |= ((e >> 1) & 1u) << p;
      q2 |= ((e >> 2) & 1u) << p;
    }
    p0 = q0; p1 = q1; p2 = q2;
  }
  p0 |= K; p1 |= K; p2 |= K;
  const uint32_t l0 = ~K | (K & (D0 | D2));
  const uint32_t l1 = ~K | (K & (D0 | D1));
  // a loop over the owned cells only (about 8 of the 27 positions): a short body that
  // stays in the instruction cache, where 27 unrolled position blocks did not
  (void)NPOS;
  uint32_t m = L;
#pragma unroll 1
  while (m) {
    const int p = ffs32(m) - 1;
    m &= m - 1;
    const uint32_t b = 1u | (((Bany >> p) & 1u) << 1) | (((p0 >> p) & 1u) << 2) | (((p1 >> p) & 1u) << 3) |
                       (((p2 >> p) & 1u) << 4) | (((l0 >> p) & 1u) << 5) | (((l1 >> p) & 1u) << 6);
    store(p, (uint8_t)b);
  }
}

// Second half: expand every boundary class of the lower star L (keys in `col`) and
// emit each owned cell's byte through `store(p, byte)`.  bx/by/bz: the vertex lies on
// the first or last plane of that axis (ignored for an interior vertex).
template <int ND, class Store>
MSC_HD void expand_and_store(uint32_t L, uint64_t* col, int cs, bool interior, bool bx, bool by, bool bz,
                             uint32_t enc_map, const Store& store) {
  LowerStarState<ND, KeyCol> st(KeyCol{col, cs});
  uint32_t Bany = 0;
  if (interior)
    st.expand(L);
  else
    Bany = run_classes<ND>(st, L, bx, by, ND == 3 && bz);
  store_cells<ND>(st, L, Bany, enc_map, store);
}

// The constrained re-pairing of ondemandaccurate's accurate 3-manifolds
// (MyRobinsNoalloc<...,4,6>::ComputeLowerStar with a restriction map,
// gi_modified_robins.h:1281-1343): the lower star L split by class
// restriction_label * maxDim + boundaryValue (maxDim = 3; at most 24 classes, the last
// taking every larger one), the classes expanded in increasing order.  rl[p]: the
// restriction label of the cell at position p.
template <int ND, class Store>
MSC_HD void expand_and_store_keyed(uint32_t L, uint64_t* col, int cs, const uint8_t* rl, bool bx, bool by, bool bz,
                                   uint32_t enc_map, const Store& store) {
  using N = Nb<ND>;
  constexpr int NPOS = N::NPOS;
  LowerStarState<ND, KeyCol> st(KeyCol{col, cs});
  const uint32_t B0 = bx ? N::axis_mask(0, 0) : 0u;
  const uint32_t B1 = by ? N::axis_mask(1, 0) : 0u;
  const uint32_t B2 = (ND == 3 && bz) ? N::axis_mask(2, 0) : 0u;
  constexpr int kClasses = 24;
  uint32_t cls[kClasses];
#pragma unroll
  for (int k = 0; k < kClasses; k++) cls[k] = 0u;
  for (int p = 0; p < NPOS; p++) {
    if (!((L >> p) & 1u)) continue;
    const int bv = (int)((B0 >> p) & 1u) + (int)((B1 >> p) & 1u) + (int)((B2 >> p) & 1u);
    int key = 3 * (int)rl[p] + bv;
    if (key > kClasses - 1) key = kClasses - 1;
    cls[key] |= 1u << p;
  }
  for (int k = 0; k < kClasses; k++)
    if (cls[k]) st.expand(cls[k]);
  store_cells<ND>(st, L, B0 | B1 | B2, enc_map, store);
}

// One vertex of the conforming re-pairing of ondemandaccurate's accurate 3-manifolds
// (ondemandaccurate.cxx:1000-1063): a vertex whose own cell, or a cell of whose lower
// star, carries a restriction label recomputes its lower star split by label
// (expand_and_store_keyed); every other vertex keeps its pairs.  rlab(p, r): the
// restriction label of the cell at position p (called for positions inside the
// complex only).  Returns true if the vertex recomputed its lower star.
template <int ND, class Load, class Restrict, class Store>
MSC_HD bool conform_vertex(int64_t x, int64_t y, int64_t z, int64_t X, int64_t Y, int64_t Z, bool interior,
                           const Load& load, const Restrict& rlab, uint64_t* col, int cs, uint32_t enc_map,
                           const Store& store) {
  using N = Nb<ND>;
  constexpr int NPOS = N::NPOS;
  const uint32_t okx = (x > 0 ? N::axis_mask(0, -1) : 0u) | N::axis_mask(0, 0) | (x < X - 1 ? N::axis_mask(0, 1) : 0u);
  const uint32_t oky = (y > 0 ? N::axis_mask(1, -1) : 0u) | N::axis_mask(1, 0) | (y < Y - 1 ? N::axis_mask(1, 1) : 0u);
  const uint32_t okz = (ND == 2) ? ~0u
                                 : ((z > 0 ? N::axis_mask(2, -1) : 0u) | N::axis_mask(2, 0) |
                                    (z < Z - 1 ? N::axis_mask(2, 1) : 0u));
  const uint32_t ok = okx & oky & okz;
  uint8_t rl[NPOS];
  uint32_t R = 0;
  for (int p = 0; p < NPOS; p++) {
    uint8_t r = 0;
    if ((ok >> p) & 1u) rlab(p, r);
    rl[p] = r;
    if (r) R |= 1u << p;
  }
  if (!R) return false;
  bool nan = false;
  const uint32_t L = lower_star_keys<ND>(x, y, z, X, Y, Z, interior, load, col, cs, nan);
  if (!(R & L)) return false;  // (L holds the vertex itself)
  expand_and_store_keyed<ND>(L, col, cs, rl, x == 0 || x == X - 1, y == 0 || y == Y - 1, z == 0 || z == Z - 1,
                             enc_map, store);
  return true;
}

// One vertex, end to end (both halves).  Returns true if a NaN was seen.
template <int ND, class Load, class Store>
MSC_HD bool process_vertex(int64_t x, int64_t y, int64_t z, int64_t X, int64_t Y, int64_t Z, bool interior,
                           const Load& load, uint64_t* col, int cs, uint32_t enc_map, const Store& store) {
  bool nan = false;
  const uint32_t L = lower_star_keys<ND>(x, y, z, X, Y, Z, interior, load, col, cs, nan);
  expand_and_store<ND>(L, col, cs, interior, x == 0 || x == X - 1, y == 0 || y == Y - 1, z == 0 || z == Z - 1,
                       enc_map, store);
  return nan;
}

}  // namespace msc
