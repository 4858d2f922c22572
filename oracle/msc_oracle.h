/* CPU oracle for the MSCEER lower-star discrete gradient (.grad) path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm used as the checker for the CUDA path: only tests/, bench.py's CPU
 * baseline legs and __graft_entry__.smoke() may load it.  The product never
 * links it and never falls back to it.
 *
 * Layout: f is float32 with x fastest.  The cell complex has (2X-1)(2Y-1)(2Z-1)
 * cells (x fastest), one .grad byte per cell (GradBitfield, LSB first:
 * assigned:1, flag:1, pair:3, ldir:3).
 */
#ifndef MSC_ORACLE_H
#define MSC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Lower-star pairing (assigned + pair bits, ldir=0, flag=0) for every cell. */
int oracle_lstar_pairs_3d(const float* f, int64_t X, int64_t Y, int64_t Z, uint8_t* grad, int nthreads);
int oracle_lstar_pairs_2d(const float* f, int64_t X, int64_t Y, uint8_t* grad, int nthreads);

/* Ascending-manifold dimension (ldir bits) on a paired gradient. */
int oracle_ldir_3d(int64_t X, int64_t Y, int64_t Z, uint8_t* grad);
int oracle_ldir_2d(int64_t X, int64_t Y, uint8_t* grad);

/* flag bit = (boundaryValue(cell) != 0), as written by outputToFile. */
int oracle_flag_3d(int64_t X, int64_t Y, int64_t Z, uint8_t* grad);
int oracle_flag_2d(int64_t X, int64_t Y, uint8_t* grad);

/* The complete .grad file of steepest_lstar (3D) / the 2D builder. */
int oracle_grad_3d(const float* f, int64_t X, int64_t Y, int64_t Z, uint8_t* grad, int nthreads);
int oracle_grad_2d(const float* f, int64_t X, int64_t Y, uint8_t* grad, int nthreads);

/* Conforming gradient of ondemandaccurate's accurate 3-manifolds: the restriction labels
 * of the final ascending (asc) / descending (dsc) labels (either may be NULL), then the
 * constrained re-pairing of the touched vertices and the ldir / flag passes over g. */
int oracle_boundary_labels_3d(const float* f, int64_t X, int64_t Y, int64_t Z, const int32_t* asc,
                              const int32_t* dsc, uint8_t* out);
int oracle_conform_3d(const float* f, int64_t X, int64_t Y, int64_t Z, const uint8_t* restrict_lab, uint8_t* g,
                      int nthreads);

/* Morse-Smale complex graph of a finished .grad: MorseSmaleComplexBasic::ComputeFromGrad
 * without arc geometry (gi_morse_smale_complex_basic.h:676-716).  Nodes are the
 * critical cells in cell order: cell id, dimension, boundaryValue and value (f at the
 * cell's highest vertex).  Arcs are traced down from every node whose dimension d has
 * build[d - 1] set, in node order and depth-first facet order; arc_persistence is
 * value(upper) - value(lower).  Counts go to counts[0] (nodes) and counts[1] (arcs);
 * the arrays are filled up to node_cap / arc_cap entries. */
int oracle_ms_graph_3d(const uint8_t* grad, const float* f, int64_t X, int64_t Y, int64_t Z, const int build[3],
                       int64_t node_cap, int64_t* node_cell, float* node_value, uint8_t* node_dim,
                       uint8_t* node_boundary, int64_t arc_cap, int32_t* arc_lower, int32_t* arc_upper,
                       float* arc_persistence, int64_t counts[2]);

/* Central-difference gradient, x,y,z (x,y) doubles per vertex, as the reference's
 * Vec3d array after ComputeGradFromImage(1). */
int oracle_central_diff_3d(const float* f, int64_t X, int64_t Y, int64_t Z, double* g);
int oracle_central_diff_2d(const float* f, int64_t X, int64_t Y, double* g);

/* Integrated labels (msc_labels_oracle.c). */
typedef struct {
	float error_threshold;     /* accepted |two half steps - one full step|^2 */
	float gradient_threshold;  /* stop when |grad f| falls below this */
	int iteration_limit;       /* Euler steps per streamline */
	double max_step;           /* MAX_STEP_IN_GRID_CELLS */
	float presimp_threshold;   /* persistence up to which extrema merge */
} oracle_label_params;

/* Certain terminal regions grown from the (merged) extrema; dir -1 ASC, +1 DSC. */
int oracle_terminal_regions_3d(const float* f, const uint8_t* grad, int64_t X, int64_t Y, int64_t Z, int dir,
                               float presimp_threshold, int32_t* labels);
/* The isolated-region cleaner alone, in place (IsolatedCCRegionRemoverNEW). */
int oracle_clean_regions_3d(const float* f, int64_t X, int64_t Y, int64_t Z, int dir, int32_t* labels);
/* Full labeling chain; dirs bit 0 ASC, bit 1 DSC (DSC after ASC on the shared gradient). */
int oracle_labels_3d(const float* f, const uint8_t* grad, int64_t X, int64_t Y, int64_t Z, int dirs,
                     const oracle_label_params* P, int32_t* labels_asc, int32_t* labels_dsc,
                     int32_t* stage_labels);

/* The saddle streamline digitizers of ondemandaccurate's needASC1 / needDSC1 modes at one
 * thread on the gradient of f (no seed zeroed): which bit 0 the ascending lines from the
 * 2-saddles (label 4 on hexes and faces), bit 1 the descending lines from the 1-saddles
 * (label 5 on vertices and edges), in that order, into cells (one byte per cell, in and
 * out).  Test infrastructure. */
int oracle_saddle_lines_3d(const float* f, const uint8_t* grad, int64_t X, int64_t Y, int64_t Z, int which,
                           const oracle_label_params* P, uint8_t* cells);
/* The same with the gradient zero at the vertices whose bit `zeroed` sets (bit v & 31 of
 * word v >> 5), as the integrations before the lines leave it at their seeds. */
int oracle_saddle_lines_zeroed_3d(const float* f, const uint8_t* grad, const uint32_t* zeroed, int64_t X, int64_t Y,
                                  int64_t Z, int which, const oracle_label_params* P, uint8_t* cells);
/* ondemandaccurate's accurate .grad for its flags a1 d1 a2 d2 at one thread: the
 * restriction labels (one byte per cell) and the .grad (from `grad`, the plain one). */
int oracle_ondemand_grad_3d(const float* f, const uint8_t* grad, int64_t X, int64_t Y, int64_t Z,
                            const oracle_label_params* P, int a1, int d1, int a2, int d2, uint8_t* restrict_out,
                            uint8_t* grad_out);

#ifdef __cplusplus
}
#endif
#endif
