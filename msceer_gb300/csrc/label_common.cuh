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
  int32_t e1, e2;
  float sval, pers;
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

// `work`: 48 device counters (the levels' claimed items), zeroed here.  `trips`
// (here and below): a device counter the kernels add their advection iterations to.
// `items`: scratch for the largest level's vertices, `n_items` a device counter.
cudaError_t launch_integrate_pass1(const float4* G, const VolDims& V, const IntegParams& P, const SpreadOrder& S,
                                   int32_t* lab, uint8_t* lvl, unsigned long long* work, unsigned long long* trips,
                                   int32_t* items, unsigned long long* n_items, int num_sms, cudaStream_t stream);
cudaError_t launch_boundary_set(const int32_t* lab, const uint8_t* state, const VolDims& V, int64_t* list, int* n,
                                uint32_t* queued, int num_sms, cudaStream_t stream);
// `work`: a device counter of claimed items, zeroed by the launchers
cudaError_t launch_fixup(const double* G, const VolDims& V, const IntegParams& P, int32_t* lab, const int32_t* lab0,
                         uint8_t* state, const int64_t* list, int n, int64_t* next, int* n_next, uint32_t* queued,
                         unsigned long long* work, unsigned long long* trips, int num_sms, cudaStream_t stream);
cudaError_t launch_fixup32(const float4* G, const VolDims& V, const IntegParams& P, int32_t* lab, const int32_t* lab0,
                           uint8_t* state, const int64_t* list, int n, int64_t* next, int* n_next, uint32_t* queued,
                           int64_t* amb, int* n_amb, int amb_mode, unsigned long long* work,
                           unsigned long long* trips, int num_sms, cudaStream_t stream);
cudaError_t launch_clean(const int32_t* lab, const float* f, const VolDims& V, int dir, int32_t* parent, int32_t* target,
                         int32_t* out, int num_sms, cudaStream_t stream);

}  // namespace msc
