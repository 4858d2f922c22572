/* msc_gpu.h -- C ABI of the GB300 (sm_103a) discrete-gradient engine.
 *
 * Drop-in for the hot path of MSCEER's steepest_lstar / Accurate2D gradient
 * builder: the per-cell .grad bytes it produces are bit-identical to the
 * reference's.  Plain pointers and sizes only; no C++ or torch types cross this
 * boundary.  Every entry returns an int status (MSC_OK or a negative MSC_ERR_*);
 * msc_last_error_string() describes the last failure on the calling thread.
 *
 * Layout (as the reference):
 *   f     X*Y*Z float32, x fastest (RegularGridTrilinearFunction::LoadImageFromFile,
 *         gi_regular_grid_trilinear_function.h:246-260)
 *   grad  one byte per cell of the (2X-1)(2Y-1)(2Z-1) cell complex, x fastest
 *         (TopologicalRegularGrid3D, gi_topological_regular_grid.h:113-126);
 *         byte = GradBitfield (gi_discrete_gradient_labeling.h:11-19), LSB first:
 *         assigned:1 flag:1 pair:3 ldir:3.
 * 2D uses X*Y floats and (2X-1)(2Y-1) cells.
 *
 * Device-pointer entries run on `stream` (a cudaStream_t; NULL = legacy default
 * stream) and synchronise it to read the kernels' convergence and error flags, so
 * the output is complete when they return.  The library never frees caller
 * memory.  Inputs with NaN are rejected with MSC_ERR_NAN_INPUT (the vertex order
 * the reference uses is not defined for them).
 */
#ifndef MSC_GPU_H
#define MSC_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* msc_stream_t;

#define MSC_OK 0
#define MSC_ERR_BAD_DIMS (-1)
#define MSC_ERR_NULL_POINTER (-2)
#define MSC_ERR_CUDA (-3)
#define MSC_ERR_OOM (-4)
#define MSC_ERR_NAN_INPUT (-5)
#define MSC_ERR_ITER_LIMIT (-6)
#define MSC_ERR_QUEUE_OVERFLOW (-7)
#define MSC_ERR_TOO_LARGE (-8)

/* Library ABI version (major*10000 + minor*100 + patch). */
int msc_version(void);

/* Text of the last error raised on the calling thread ("" if none). */
const char* msc_last_error_string(void);

/* Kernel launches of the ascending-manifold stage in the last .grad / stage-2 call
 * on the calling thread (a diagnostic: one tile pass, one halo check, then one
 * launch per round of frontier walks). */
int msc_last_ldir_passes(void);

/* Number of the library's kernel launches so far in this process, all threads (a
 * diagnostic for profiling and benchmarks). */
int64_t msc_kernel_launches(void);

/* Number of cells (= .grad bytes) of the complex: TopologicalRegularGrid3D::numCells
 * (gi_topological_regular_grid.h:1254).  Returns -1 for invalid dims. */
int64_t msc_num_cells_3d(const int64_t dims[3]);
int64_t msc_num_cells_2d(const int64_t dims[2]);

/* Complete .grad of steepest_lstar for a device-resident volume.
 * Replaces steepest_lstar/steepest_lstar.cxx:129-258:
 *   RegularGridMaxMinVertexLabeling3D::ComputeOutput (gi_max_vertex_labeling.h:1119),
 *   SlidingWindowRobinsNoalloc::ComputePairing_sliding (gi_fast_robins_noalloc.h:1254),
 *   TopologicalGradientUsingAlgorithms::setAscendingManifoldDimensions
 *     (gi_topological_gradient_using_algorithms.h:430),
 *   and the flag pass of DiscreteGradientLabeling::outputToFile
 *     (gi_discrete_gradient_labeling.h:200-218).
 * f: device, X*Y*Z floats; grad_out: device, msc_num_cells_3d(dims) bytes.
 * Synchronises `stream` once per ascending-manifold pass (a few per volume). */
int msc_lower_star_grad_3d(const float* f, const int64_t dims[3], uint8_t* grad_out, msc_stream_t stream);

/* 2D counterpart: Accurate2D::DiscreteGradientBuilder::ComputeDiscreteGradient with
 * no saddle streamlines (gi_discrete_gradient_computer.h:561-583, 681-689). */
int msc_lower_star_grad_2d(const float* f, const int64_t dims[2], uint8_t* grad_out, msc_stream_t stream);

/* Many 3D volumes of different sizes in one call (no counterpart in the reference,
 * which runs one process per volume): f[i], grad[i] are device buffers of volume i
 * with dims[3*i..3*i+2]; every .grad equals msc_lower_star_grad_3d's.  Up to 64
 * volumes share each kernel launch (a flat grid over all their blocks / tiles, the
 * volume table passed in the launch parameters) and run as one CUDA graph, kept and
 * replayed while the same buffers come back; the launch shapes are tuned by timing on
 * the first batch of a size class.  Larger batches run in chunks of 64 without a
 * graph.  Synchronises `stream` at the end. */
int msc_lower_star_grad_batch_3d(int n, const float* const* f, const int64_t* dims, uint8_t* const* grad,
                                 msc_stream_t stream);

/* Stage 1 alone: lower-star pairing of every vertex
 * (gi_fast_robins_noalloc.h:1254-1535 / gi_modified_robins.h:1281-1402) written as
 * final bytes except ldir, which holds only the closure roots (critical 1-cells 2,
 * critical 2-cells 1, critical 3-cells 0, others 3).  Synchronises `stream` once at
 * the end to read the kernel's error flag (NaN input). */
int msc_lower_star_pairs_3d(const float* f, const int64_t dims[3], uint8_t* grad_out, msc_stream_t stream);
int msc_lower_star_pairs_2d(const float* f, const int64_t dims[2], uint8_t* grad_out, msc_stream_t stream);

/* Stage 2 alone: completes the ldir bits of a stage-1 .grad in place
 * (setAscendingManifoldDimensions, gi_topological_gradient_using_algorithms.h:430-478).
 * passes_out (optional) receives the number of kernel launches of the stage. */
int msc_ascending_manifold_dims_3d(uint8_t* grad, const int64_t dims[3], msc_stream_t stream, int* passes_out);
int msc_ascending_manifold_dims_2d(uint8_t* grad, const int64_t dims[2], msc_stream_t stream, int* passes_out);

/* Central-difference gradient of the image: RegularGridTrilinearFunction::
 * ComputeGradFromImage(1) (gi_regular_grid_trilinear_function.h:285-341): per axis
 * 0.5*(f[+1] - f[-1]) inside, 0 on the first and last plane.  f32 output rounds that
 * once (within half an ulp of the reference's double); layout 0 stores x,y,z per
 * vertex (12 bytes), layout 1 x,y,z,0 (16 bytes, one vector load per vertex; 2D:
 * layout 0 and 1 both store x,y).  The _f64 variants store x,y,z doubles per vertex,
 * the reference's Vec3d array, bit for bit.  Asynchronous on `stream`. */
int msc_central_diff_grad_3d(const float* f, const int64_t dims[3], float* g_out, int layout, msc_stream_t stream);
int msc_central_diff_grad_2d(const float* f, const int64_t dims[2], float* g_out, int layout, msc_stream_t stream);
int msc_central_diff_grad_3d_f64(const float* f, const int64_t dims[3], double* g_out, msc_stream_t stream);
int msc_central_diff_grad_2d_f64(const float* f, const int64_t dims[2], double* g_out, msc_stream_t stream);

/* Parameters of the integrated labels (the ondemandaccurate arguments,
 * ondemandaccurate.cxx:159-175, plus the step bound MAX_STEP_IN_GRID_CELLS). */
typedef struct {
  float error_threshold;     /* accept two half steps when |difference|^2 < this (e.g. 1e-4) */
  float gradient_threshold;  /* stop where the interpolated |grad f| falls below this */
  int iteration_limit;       /* Euler steps per streamline (e.g. 4000) */
  float max_step;            /* largest step, in voxels (reference default 0.5) */
  float presimp_threshold;   /* extrema joined by a saddle of lower persistence merge (0 = none) */
  int precision;             /* boundary re-decisions.  0 (default): FP32, and FP64 for streamlines
                                that stop at a gradient magnitude within 2^-8 below the threshold,
                                or within 1/64 voxel of the plane where their nearest vertex would
                                change to one of another certain region; 2: the same, but FP64 for
                                every ending in a voxel touching two certain regions; 1: all in
                                FP64 (slow on GB300); 3: none (first pass only, for diagnostics) */
} msc_integ_params;

/* Ascending (minima basins) and descending (maxima mountains) 3-manifold labels of
 * ondemandaccurate (ondemandaccurate.cxx:795-948): extremum graph
 * (SimplifiedExtremumGraph, gi_extrema_region_builder.h:271-565), certain terminal
 * regions (GridSimplifiedExtremalRegionBuilder, :753-1045), path-compressing
 * adaptive-Euler integration of the central-difference gradient
 * (NumericIntegratorPathCompressingToTerminal, gi_numeric_integrator_path_compressing.h:
 * 75-433) and the isolated-region cleaner (IsolatedCCRegionRemoverNEW,
 * gi_isolated_region_remover.h:17-196).  f: device, X*Y*Z floats; grad: the device
 * .grad of msc_lower_star_grad_3d; labels_*: device int32 per vertex or NULL to skip
 * a direction (the descending pass runs after the ascending one on the gradient the
 * ascending pass zeroed at the minima, as the reference does).  A label is the
 * vertex id of its region's extremum (smallest seed vertex of a merged group), -1
 * for none.  The first integration pass runs in FP32; vertices next to a label
 * boundary are re-decided in FP32, and those whose FP32 streamline ends
 * ambiguously (see msc_integ_params.precision) again in FP64 with the reference's
 * arithmetic.  Blocking. */
int msc_integrated_labels_3d(const float* f, const uint8_t* grad, const int64_t dims[3], const msc_integ_params* params,
                             int32_t* labels_asc, int32_t* labels_dsc, msc_stream_t stream);
/* Same, also writing 4*X*Y*Z stage labels: terminal and integrated (before the
 * cleaner), ascending then descending.  For validation. */
int msc_integrated_labels_3d_stages(const float* f, const uint8_t* grad, const int64_t dims[3],
                                    const msc_integ_params* params, int32_t* labels_asc, int32_t* labels_dsc,
                                    int32_t* stages, msc_stream_t stream);
/* The accurate .grad that ondemandaccurate writes for accurate ascending / descending
 * 3-manifolds (needASC2 / needDSC2, ondemandaccurate.cxx:795-1063): the restriction label
 * of every cell from the final labels (VertexLabelingToBoundaryLabeling::
 * ComputeMINBoundary with labels_asc, ComputeMAXBoundary with labels_dsc,
 * gi_labeling_to_bounary_labeling.h:48-199; either may be NULL, as when its manifold is
 * not requested), the re-pairing of every vertex whose lower star holds a restricted
 * cell (MyRobinsNoalloc<...,4,6>::ComputeLowerStar, gi_modified_robins.h:1281-1343,
 * the star split by restriction label and boundaryValue) and the ascending-manifold
 * closure of RecordGrad (:693-699).  f: device X*Y*Z floats; labels: device int32 per
 * vertex as msc_integrated_labels_3d writes them; grad: device, the base .grad of
 * msc_lower_star_grad_3d in, the accurate .grad out.  restriction_out (optional):
 * device, msc_num_cells_3d(dims) bytes.  touched_out (optional): the number of
 * re-paired vertices.  Blocking. */
int msc_conforming_grad_3d(const float* f, const int32_t* labels_asc, const int32_t* labels_dsc, const int64_t dims[3],
                           uint8_t* grad, uint8_t* restriction_out, int64_t* touched_out, msc_stream_t stream);

/* The Morse-Smale complex graph of a device .grad: the nodes and arcs
 * MorseSmaleComplexBasic::ComputeFromGrad builds without arc geometry
 * (gi_morse_smale_complex_basic.h:676-716), as extractmsc does after loading the .grad
 * (extractmsc/extractmsc.cxx:482-504), read from device memory instead of a file.
 * Nodes: every critical cell in cell-id order -- cell id, dimension, boundaryValue and
 * value (f at the cell's highest vertex).  Arcs: for every node of dimension d >= 1
 * with build_arcs[d - 1] set, the V-paths traced down from it (rec_tdcr_candidates,
 * :550-577), node by node in depth-first facet order; lower / upper are node indices,
 * persistence = value(upper) - value(lower).  grad, f and every output array: device.
 * counts (host): [0] nodes, [1] arcs, always written.  The node arrays are written when
 * all four are non-NULL and node_cap >= counts[0]; the arc arrays when arc_lower and
 * arc_upper are non-NULL and arc_cap >= counts[1] (arc_persistence may be NULL) -- a
 * call with capacities 0 sizes the arrays for a second call.  MSC_ERR_QUEUE_OVERFLOW if
 * one node's trace branches beyond 64 pending paths, MSC_ERR_ITER_LIMIT if it visits
 * more than 2^24 cells (only a .grad with a cycle, i.e. not a gradient, gets there).
 * Blocking.  The reference's node
 * and arc objects also carry list links and manifold ids; callers build those from
 * these arrays. */
int msc_ms_graph_3d(const uint8_t* grad, const float* f, const int64_t dims[3], const int build_arcs[3],
                    int64_t node_cap, int64_t* node_cell, float* node_value, uint8_t* node_dim,
                    uint8_t* node_boundary, int64_t arc_cap, int32_t* arc_lower, int32_t* arc_upper,
                    float* arc_persistence, int64_t counts[2], msc_stream_t stream);

/* The saddle streamline digitizers of ondemandaccurate's needASC1 / needDSC1 modes
 * (ReIntegrateUpFrom2Saddles / ReIntegrateDownFrom1Saddles, ondemandaccurate.cxx:254-505,
 * with DigitizingNumericStreamlineIntegrator3dASC / 3dDSC,
 * gi_numeric_streamline_integrator.h:525-1080): streamlines from the cells around every
 * critical saddle, label 4 on the hex-face chains of the ascending lines from the
 * 2-saddles (which bit 0), label 5 on the vertex-edge chains of the descending lines
 * from the 1-saddles (bit 1, after the ascending ones), with the one-thread run's
 * result.  f, grad (the .grad of f) and cells (one byte per cell, in and out: cells
 * labelled 4 / 5 on entry stop the lines of that label): device.  zeroed: NULL, or a
 * device bitmap (bit v & 31 of word v >> 5, at least ceil(X*Y*Z / 32) words) of the
 * vertices where the gradient is zero (the seeds of the 3-manifold integrations before
 * the lines).  params: error_threshold, gradient_threshold, iteration_limit, max_step.
 * stats (host, optional): streamlines, recorded voxel steps, voxel steps kept, rounds.
 * Fewer than 2^32 cells; the records take 136 bytes per label-free voxel step.
 * Blocking. */
int msc_saddle_lines_3d(const float* f, const uint8_t* grad, const uint32_t* zeroed, const int64_t dims[3], int which,
                        const msc_integ_params* params, uint8_t* cells, int64_t stats[4], msc_stream_t stream);

/* The isolated-region cleaner alone: IsolatedCCRegionRemoverNEW::ComputeOutput
 * (gi_isolated_region_remover.h:155-192) on caller labels, as ondemandaccurate runs it
 * after the integration (ondemandaccurate.cxx:866-870, 942-946).  Same-label
 * 6-connected components; each component whose first vertex (in the order of
 * `direction`: -1 the ascending labels' IndexCompareLessThan, lowest value first; +1
 * the descending labels' IndexCompareGreaterThan) has an earlier neighbour joins, in
 * the reference's vertex order, the component of its earliest neighbour from another
 * region.  f: device X*Y*Z floats; labels_in / labels_out: device int32 per vertex
 * (-1 = none; a vertex labelled -1 stays -1).  Blocking. */
int msc_clean_regions_3d(const float* f, const int32_t* labels_in, const int64_t dims[3], int direction,
                         int32_t* labels_out, msc_stream_t stream);
/* Error text of the last failed labeling call on the calling thread. */
const char* msc_labels_last_error_string(void);
/* Work counts of the last labeling call on the calling thread: boundary
 * re-decisions (ascending), of which in FP64, then the same for descending. */
void msc_labels_last_stats(int64_t out[4]);
/* Advection iterations (adaptive Euler step attempts) of the last labeling call on
 * the calling thread: first pass, FP32 boundary re-decisions, FP64 re-decisions;
 * ascending, then descending. */
void msc_labels_last_iterations(int64_t out[6]);
/* The labeling keeps its device scratch (about 135 bytes per vertex and direction) in a
 * memory pool of its own that holds on to the memory between calls; this returns the
 * unused part to the device (call it before the application needs that memory
 * elsewhere).  No counterpart in the reference. */
void msc_trim_scratch(void);

/* Stage 2 for callers that may not allocate device memory: the same result as
 * msc_ascending_manifold_dims_3d, with the pass scratch (tile flags, status words)
 * in a fixed 1 MiB array inside the library instead of allocated memory.  No
 * counterpart in the reference (its CPU closure needs no device memory).  Meant for
 * applications that hand out all device memory through their own pool and do not
 * let libraries call cudaMalloc.  Limit: 524,288 ldir tiles of 32x32x16 cells
 * (volumes up to about 1000^3 vertices); larger volumes return MSC_ERR_TOO_LARGE.
 * Dims as msc_ascending_manifold_dims_3d (an axis may have a single vertex).  The
 * first call on a device looks up the array's device address and keeps it for the
 * process (do not use the entry on a device after cudaDeviceReset).  The call
 * synchronises `stream` once per pass, so it must not be made during stream capture.
 * passes_out counts the tile passes of this multi-pass form (the allocating entry
 * counts the launches of its single-pass form).  Every call shares the array: calls
 * whose work overlaps on the GPU race.  Calls no cudaMalloc / cudaFree. */
int msc_ascending_manifold_dims_3d_static(uint8_t* grad, const int64_t dims[3], msc_stream_t stream, int* passes_out);

/* Host-memory convenience with steepest_lstar's semantics: copies f to the GPU,
 * computes, copies the .grad back.  f_host: X*Y*Z floats; grad_host:
 * msc_num_cells_3d(dims) bytes.  Blocking.  Runs on the current device and keeps a
 * per-thread device staging buffer (grown on demand) between calls; pinned host
 * buffers give the fastest copies. */
int msc_steepest_lstar_host(const float* f_host, const int64_t dims[3], uint8_t* grad_host);
int msc_lower_star_grad_2d_host(const float* f_host, const int64_t dims[2], uint8_t* grad_host);

#ifdef __cplusplus
}
#endif
#endif /* MSC_GPU_H */
