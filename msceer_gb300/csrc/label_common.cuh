// Shared definitions of the labeling kernels (label_kernels.cu, integrate_kernels.cu).
#pragma once
#include <cstdint>

#include "msc_device.cuh"

namespace msc {

// Vertex grid and its cell complex.
struct VolDims {
  int64_t X, Y, Z;     // vertices
  int64_t dX, dY, dZ;  // cells
  int64_t cs1, cs2;    // cell-id strides
};

// A saddle arc between two extrema (MergeArc, gi_extrema_region_builder.h:43-61).
struct Arc {
  int64_t saddle;
  int32_t e1, e2;  // extremum ids
  float sval, pers;
  int64_t c1, c2;  // the extrema's cells, their highest vertices and values there (what
  int64_t h1, h2;  // the host merge compares)
  float f1, f2;
};

// Per-vertex integration state (DestType, gi_basic_types.h:43-49, plus "seed": a
// certain terminal whose gradient is zeroed, gi_numeric_integrator_path_compressing.h:118-123).
enum : uint8_t {
  kStUnassigned = 0,
  kStSeed = 1,
  kStTerminal = 2,
  kStAssigned = 3,
  kStNonterminal = 4,
};

// Label of a vertex that a first-pass streamline reached without finding a region.
constexpr int32_t kLabelNone = -2;

__host__ __device__ inline void cell_coords(const VolDims& V, int64_t id, int64_t k[3]) {
  if ((uint64_t)id <= 0xFFFFFFFFull) {  // 32-bit divisions (a 64-bit one is a long sequence)
    const uint32_t u = (uint32_t)id, dx = (uint32_t)V.dX, dy = (uint32_t)V.dY;
    const uint32_t q = u / dx;
    k[0] = u - q * dx;
    k[1] = q % dy;
    k[2] = q / dy;
    return;
  }
  k[0] = id % V.dX;
  k[1] = (id / V.dX) % V.dY;
  k[2] = id / (V.dX * V.dY);
}

__host__ __device__ inline int boundary_value(const VolDims& V, const int64_t k[3]) {
  return (k[0] == 0 || k[0] == V.dX - 1) + (k[1] == 0 || k[1] == V.dY - 1) + (k[2] == 0 || k[2] == V.dZ - 1);
}

// getPair: UncompressByteTo6NeighborOffset (the labeling path needs X, Y, Z >= 2,
// where stored codes name their true axis)
__host__ __device__ inline int64_t decode_pair(const VolDims& V, int64_t id, unsigned code) {
  const int64_t off = (code >> 1) == 0 ? 1 : ((code >> 1) == 1 ? V.cs1 : V.cs2);
  return (code & 1) ? id - off : id + off;
}

// IsGreater (gi_regular_grid_trilinear_function.h:309-314) on vertex indices
__device__ __forceinline__ bool vgreater(const float* f, int64_t a, int64_t b) {
  const float fa = f[a], fb = f[b];
  if (fa > fb) return true;
  if (fb > fa) return false;
  return a > b;
}

// Cell2HighestVertex as a vertex index
__device__ inline int64_t highest_vertex(const VolDims& V, const float* f, int64_t cell) {
  int64_t k[3];
  cell_coords(V, cell, k);
  const int64_t bx = k[0] >> 1, by = k[1] >> 1, bz = k[2] >> 1;
  const int ox = (int)(k[0] & 1), oy = (int)(k[1] & 1), oz = (int)(k[2] & 1);
  int64_t best = -1;
  for (int s = 0; s < 8; s++) {
    const int dx = s & 1, dy = (s >> 1) & 1, dz = (s >> 2) & 1;
    if ((dx && !ox) || (dy && !oy) || (dz && !oz)) continue;
    const int64_t v = (bx + dx) + (by + dy) * V.X + (bz + dz) * V.X * V.Y;
    if (best < 0 || vgreater(f, v, best)) best = v;
  }
  return best;
}

cudaError_t launch_find_critical(const uint8_t* g, const VolDims& V, int dir, int32_t* ext_id_of_key,
                                 int64_t* ext_cells, int* n_ext, int64_t* saddles, int* n_sad, int num_sms,
                                 cudaStream_t stream);
cudaError_t launch_trace_arcs(const uint8_t* g, const float* f, const VolDims& V, int dir, const int64_t* saddles,
                              int n_sad, const int32_t* ext_id_of_key, float threshold, Arc* arcs, int* n_arcs,
                              int* err, int num_sms, cudaStream_t stream);
cudaError_t launch_extremum_info(const float* f, const VolDims& V, int dir, const int64_t* ext_cells, int n_ext,
                                 int64_t* hv, float* fval, int64_t* seed, int num_sms, cudaStream_t stream);
cudaError_t launch_group_seeds(const int32_t* rep, const int64_t* seed, int n_ext, int32_t* name, int32_t* lab,
                               uint8_t* state, int num_sms, cudaStream_t stream);
int64_t terminal_num_tiles(const VolDims& V);
// One round of the certain terminal regions' global frontier walk from the vertices
// qin[0, *n_in) (n_host: the same count on the host, for the grid); vertices beyond a
// thread's stack go to qout.
cudaError_t launch_terminal_walk(const float* f, int32_t* lab, const VolDims& V, int dir, const int64_t* qin,
                                 const int* n_in, int n_host, int64_t* qout, int* n_out, int cap, int* err,
                                 int num_sms, cudaStream_t stream);
cudaError_t launch_terminal_pass(const float* f, int32_t* lab, const VolDims& V, int dir, const uint8_t* dirty_in,
                                 uint8_t* dirty_out, int* changed, int* err, int num_sms, cudaStream_t stream);

// ---- K4 streamline integration (integrate_kernels.cu) ----------------------------------------
struct IntegParams {
  float ethresh, gthresh;
  int iteration_limit;
  double max_step;
  int step_mult;  // -1: flow downhill (ascending manifolds of minima), +1 uphill
  // Trapped-streamline cut-off (0 = off): every trap_window iterations the position
  // is compared with the one trap_window iterations before; a streamline that moved
  // less than trap_radius (voxels, max norm) two checks in a row ends there.
  int trap_window = 0;
  float trap_radius = 0.f;
};

// Spread visiting order of the first pass (:166-174 with one thread): level L
// visits start_L + j * stride_L.  Host-computed tables, levels in order.
struct SpreadOrder {
  int nlev;
  int64_t start[48], stride[48], offset[49];
};

// The first pass runs the spread order in batches (a group of levels, or part of one):
// speculative streamlines of the batch's items record the vertices their stop test
// passed, and the resolution kernels turn them into the labels the one-thread
// reference assigns (integrate_kernels.cu).  SpecSet: the batch's items in visiting
// order, their recorded sequences and the holder lists of the recorded vertices.
struct SpecSet {
  const int32_t* vtx;  // item vertex (its entry 0)
  uint32_t* e1;        // entry 1
  uint32_t* head;      // word offset in pool of the segment that holds entries 2, 3, ...
  int32_t* len;        // recorded entries (0: the item was skipped)
  int32_t* endlab;     // label where the streamline stopped, if labelled before the batch
  int32_t* cut;        // -1, or the entry where an earlier item's path stops it
  int32_t* ptr;        // the item whose label it takes
  uint8_t* alive;      // runs (no earlier item labelled its vertex)
  uint32_t* pool;      // entry segments
  unsigned long long pool_words;
  unsigned long long* cursor;  // next free pool word
  int* overflow;               // set when the pool or the holder nodes ran out (the batch is redone smaller)
  // holders: for every vertex the list of (item, entry index) that recorded it
  int32_t* hhead;              // per vertex: its first holder node, -1 for none
  int32_t* hitem;              // per node: the item
  uint32_t* hidx;              // per node: the entry index, kRec-flagged for path vertices
  int32_t* hnext;              // per node: the vertex's next node
  unsigned long long node_cap;
  unsigned long long* ncursor;  // next free node
};
// lvl: 0 for labelled vertices, 255 for the rest
cudaError_t launch_init_levels(const int32_t* lab, uint8_t* lvl, int64_t N, int num_sms, cudaStream_t stream);
// *n = the vertices with lvl 255 (not labelled yet)
cudaError_t launch_count_unlabelled(const uint8_t* lvl, int64_t N, unsigned long long* n, int num_sms,
                                    cudaStream_t stream);
// The vertices of spread positions [u0, u1) with lvl >= stamp, in order, into items;
// their number to *n_items.  counts: (u1 - u0) / 1024 + 1 ints of scratch.
cudaError_t launch_spread_compact(const SpreadOrder& S, int64_t u0, int64_t u1, const uint8_t* lvl, int stamp,
                                  int* counts, int32_t* items, unsigned long long* n_items, cudaStream_t stream);
// Speculative streamlines of items [k0, k1) (stopping at lvl < stamp); they build the
// holder lists (hhead all -1 at launch) and make the first resolution round's claims.
// `work`: a device counter, zero at launch; `trips`: advection iterations are added to it.
cudaError_t launch_speculate(const float4* G, const VolDims& V, const IntegParams& P, const SpecSet& Q, int64_t k0,
                             int64_t k1, const int32_t* lab, const uint8_t* lvl, int stamp, uint32_t* claim,
                             unsigned long long* work, unsigned long long* trips, int num_sms, cudaStream_t stream);
// After a pool overflow: drops the claims on vertices with lvl >= stamp.
cudaError_t launch_spec_unclaim_all(const uint8_t* lvl, int stamp, uint32_t* claim, int64_t N, int num_sms,
                                    cudaStream_t stream);
// Vertices whose claims a resolution round recomputes: a bitmap (words uint32) and the
// list of its set bits (*n entries).  The round that takes the list clears the bits.
struct SpecDirty {
  uint32_t* bits;
  int64_t words;
  uint32_t* list;
  unsigned long long* n;
};
// Resolution rounds of items [k0, k1), three stream operations each.  The first (cur ==
// nullptr) looks at every item (the speculation made its claims); a later one
// recomputes the claims of cur's vertices from their holders and looks at the items
// that hold one of them (ibits: a bitmap over the items, ibits_words words, clear
// between rounds).  An item whose alive / cut changed marks the path vertices between
// its old and new extent in nxt (whose bitmap must be clear).  The rounds end when a
// round marks nothing; a round after that one finds no items and marks nothing.
cudaError_t launch_spec_round(const SpecSet& Q, int64_t k0, int64_t k1, uint32_t* claim, const SpecDirty* cur,
                              const SpecDirty& nxt, uint32_t* ibits, int64_t ibits_words, int num_sms,
                              cudaStream_t stream);
// Labels of the resolved batch [k0, k1), stamping its vertices with `stamp`: ptr, then
// the write, which sets *long_chain (and writes nothing for that item) where a chain
// of cut items is longer than it follows; pointer jumping then shortens the chains.
cudaError_t launch_spec_ptr(const SpecSet& Q, int64_t k0, int64_t k1, const uint32_t* claim, int num_sms,
                            cudaStream_t stream);
cudaError_t launch_spec_jumps(const SpecSet& Q, int64_t k0, int64_t k1, int num_sms, cudaStream_t stream);
cudaError_t launch_spec_write(const SpecSet& Q, int64_t k0, int64_t k1, uint8_t* lvl, int stamp, const uint32_t* claim,
                              int32_t* lab, int* long_chain, int num_sms, cudaStream_t stream);
cudaError_t launch_boundary_set(const int32_t* lab, const uint8_t* state, const VolDims& V, int64_t* list, int* n,
                                uint32_t* queued, int num_sms, cudaStream_t stream);
// Fix-up streamline ends (FP64 / FP32): endv[v] = the final nearest vertex of v's
// streamline to a certain terminal region.  The FP32 kernel lists the streamlines whose
// ending is ambiguous in amb (amb_mode: see the kernel) instead.  `work`: a device
// counter of claimed items, zeroed by the launchers.
// f: the image; zeroed: a bit per vertex whose gradient is zero (the seeds)
cudaError_t launch_fixup_end64(const float* f, const uint32_t* zeroed, const VolDims& V, const IntegParams& P,
                               const uint8_t* state,
                               const int64_t* list, int n, int32_t* endv, unsigned long long* work,
                               unsigned long long* trips, int num_sms, cudaStream_t stream, const int* n_dev = nullptr);
// n_dev (optional): the list's length in device memory, n then only sizes the grid
cudaError_t launch_fixup_end32(const float4* G, const VolDims& V, const IntegParams& P, const int32_t* lab,
                               const uint8_t* state, const int64_t* list, int n, int32_t* endv, int64_t* amb,
                               int* n_amb, int amb_mode, unsigned long long* work, unsigned long long* trips,
                               int num_sms, cudaStream_t stream, const int* n_dev = nullptr);
// the vertices that are not certain terminals (fix-up candidates), appended to list
cudaError_t launch_uncertain_list(const uint8_t* state, int64_t N, int64_t* list, int* n, int num_sms,
                                  cudaStream_t stream);
// Fix-up wave w over `list`: stamps the members in inw, clears their queued bits and
// lists the members without an end yet in todo (n_todo: a device counter).
cudaError_t launch_wave_mark(const int64_t* list, int n, int w, int32_t* inw, uint32_t* queued, const int32_t* endv,
                             int64_t* todo, int* n_todo, int num_sms, cudaStream_t stream);
// Decides wave w in the reference's order (every member has its end): resolve gives
// each member its new label in rfin (jump == false: from the ends; a member whose chain
// of same-wave ends is too long sets *long_chain, and a second call with jump == true
// shortens the chains first); finish reopens neighbours into next (n_next: a device
// counter) and writes the labels.
cudaError_t launch_wave_resolve(const int64_t* list, int n, int w, const int32_t* endv, const int32_t* inw,
                                const int32_t* lab, const uint8_t* state, int32_t* rptr, int32_t* rval, int32_t* rfin,
                                int* long_chain, bool jump, int num_sms, cudaStream_t stream);
cudaError_t launch_wave_finish(const int64_t* list, int n, int w, const VolDims& V, const int32_t* rfin,
                               const int32_t* inw, int32_t* lab, uint8_t* state, uint32_t* queued, int64_t* next,
                               int* n_next, int num_sms, cudaStream_t stream);
// IsolatedCCRegionRemoverNEW::ComputeOutput: same-label components, then the reference's
// vertex-ordered joins of the components without their region's extremum.  parent,
// first, md, roots: N int32 of scratch each; counters: 2 ints; pinned: one int of
// pinned host memory (the sweep count is read through it; the call synchronises
// `stream` once per sweep).  sweeps_out (optional): sweeps made.
cudaError_t launch_clean(const int32_t* lab, const float* f, const VolDims& V, int dir, int32_t* parent, int32_t* first,
                         int32_t* md, int32_t* roots, int* counters, int* pinned, int32_t* out, int num_sms,
                         cudaStream_t stream, int* sweeps_out);

}  // namespace msc
