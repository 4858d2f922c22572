/* CPU oracle for MSCEER's integrated ascending/descending labels (3D).
 *
 * TEST INFRASTRUCTURE ONLY: the deterministic FP64 single-thread restatement the
 * tests and bench use to judge the CUDA labeling path.  It follows ondemandaccurate's
 * 3-manifold pipeline (ondemandaccurate/ondemandaccurate.cxx:795-871 for ASC,
 * :916-948 for DSC) in the order the reference takes with one OpenMP thread:
 *   1. SimplifiedExtremumGraph::ComputeMinMapFromGradient + UFMergeGraph
 *        (gi_extrema_region_builder.h:28-268, 271-565): extrema, V-path arcs from the
 *        saddles (rec_td / rec_tu), persistence-ordered merges up to a threshold.
 *   2. GridSimplifiedExtremalRegionBuilder::BeginIntegration
 *        (gi_extrema_region_builder.h:753-1045): certain regions grown from the
 *        extrema in value order over the 6-neighbourhood.
 *   3. NumericIntegratorPathCompressingToTerminal::BeginIntegration
 *        (gi_numeric_integrator_path_compressing.h:75-433) with
 *        AdaptiveEulerAdvector3D (gi_adaptive_euler_advector.h:51-305) and the
 *        checkers of gi_advection_checker.h:212-264: first pass with path
 *        compression in the bit-reversal-like visiting order, then the fix-up of
 *        vertices whose 6-neighbour carries another label, iterated to a fixpoint.
 *   4. IsolatedCCRegionRemoverNEW::ComputeOutput (gi_isolated_region_remover.h:17-196).
 * Arithmetic follows the reference operation by operation: positions, gradients and
 * half steps in double, step sizes / thresholds / error in float, and the full Euler
 * displacement formed in float (Vec3d * float multiplies in float, gi_vectors.h:250).
 *
 * The reference numbers regions by "unique id" in unordered_map iteration order, so
 * label values carry no meaning across runs; this oracle names every region by its
 * smallest seed vertex (the extremum vertex when nothing merged), -1 = unlabelled.
 *
 * Also the saddle streamline digitizers of the needASC1 / needDSC1 modes
 * (ondemandaccurate.cxx:254-505, gi_numeric_streamline_integrator.h:525-1080) at one
 * thread, on the same advector with the TerminateNearAssignedHex / Vert checkers
 * (gi_advection_checker.h:60-100): oracle_saddle_lines_3d, equal byte for byte to the
 * reference compiled here (oracle/ref_harness_lines.cpp, tests/golden/saddle_lines.json).
 */
#include "msc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

enum { DT_BACKGROUND = 0, DT_UNASSIGNED = 1, DT_ASSIGNED = 2, DT_CERTAIN_TERMINAL = 3, DT_CERTAIN_NONTERMINAL = 4 };
enum { EV_NONE = 0, EV_OUT_OF_VOXEL, EV_OVER_MAX_ITERATIONS, EV_LOW_GRADIENT, EV_HIT_EXTREMUM, EV_HIT_PREASSIGNED };

typedef struct { double x, y, z; } v3d;

typedef struct {
	int64_t X, Y, Z;           /* vertices */
	int64_t dX, dY, dZ;        /* cells */
	const float* f;
	const uint8_t* grad;       /* .grad bytes */
	int dir;                   /* -1 ascending manifolds of minima, +1 of maxima */
} lctx;

/* ---- small helpers ------------------------------------------------------------ */

static inline int64_t vidx(const lctx* c, int64_t x, int64_t y, int64_t z) { return x + c->X * (y + c->Y * z); }

/* IsGreater (gi_regular_grid_trilinear_function.h:309-314) */
static inline int is_greater(const float* f, int64_t a, int64_t b) {
	if (f[a] > f[b]) return 1;
	if (f[b] > f[a]) return 0;
	return a > b;
}

/* Comparer::Compare(a, b): "a comes before b".  ASC: IndexCompareLessThan,
 * DSC: IndexCompareGreaterThan (gi_numeric_integrator_expanding_region_stop.h:18-60). */
static inline int comes_before(const lctx* c, int64_t a, int64_t b) {
	return c->dir < 0 ? is_greater(c->f, b, a) : is_greater(c->f, a, b);
}

/* GatherExistingNeighborsAll6 order: +x,-x,+y,-y,+z,-z (gi_regular_grid.h:179-205) */
static int neighbors6(const lctx* c, int64_t v, int64_t out[6]) {
	int64_t x = v % c->X, y = (v / c->X) % c->Y, z = v / (c->X * c->Y);
	int n = 0;
	if (x < c->X - 1) out[n++] = v + 1;
	if (x > 0) out[n++] = v - 1;
	if (y < c->Y - 1) out[n++] = v + c->X;
	if (y > 0) out[n++] = v - c->X;
	if (z < c->Z - 1) out[n++] = v + c->X * c->Y;
	if (z > 0) out[n++] = v - c->X * c->Y;
	return n;
}

static inline void ccoords(const lctx* c, int64_t id, int64_t k[3]) {
	k[0] = id % c->dX;
	k[1] = (id / c->dX) % c->dY;
	k[2] = id / (c->dX * c->dY);
}
static inline int cdim(const int64_t k[3]) { return (int)((k[0] & 1) + (k[1] & 1) + (k[2] & 1)); }
static inline int gcrit(const lctx* c, int64_t id) { return ((c->grad[id] >> 2) & 7) == 7; }
static inline int64_t gpair(const lctx* c, int64_t id) {
	/* getPair: UncompressByteTo6NeighborOffset(cell, code) */
	unsigned code = (c->grad[id] >> 2) & 7;
	int64_t st[3] = { 1, c->dX, c->dX * c->dY };
	int64_t off = st[code >> 1];
	return (code & 1) ? id - off : id + off;
}
static inline int64_t cell_vertex(const lctx* c, int64_t id) { /* VertexNumberFromCellID */
	int64_t k[3];
	ccoords(c, id, k);
	return (k[0] >> 1) + (k[1] >> 1) * c->X + (k[2] >> 1) * c->X * c->Y;
}
/* Cell2HighestVertex: highest vertex of the cell under IsGreater, as a vertex index */
static int64_t highest_vertex(const lctx* c, int64_t id) {
	int64_t k[3];
	ccoords(c, id, k);
	int odd[3], no = 0;
	for (int a = 0; a < 3; a++) if (k[a] & 1) odd[no++] = a;
	int64_t best = -1;
	for (int s = 0; s < (1 << no); s++) {
		int64_t q[3] = { k[0], k[1], k[2] };
		for (int t = 0; t < no; t++) q[odd[t]] += ((s >> t) & 1) ? 1 : -1;
		int64_t v = (q[0] >> 1) + (q[1] >> 1) * c->X + (q[2] >> 1) * c->X * c->Y;
		if (best < 0 || is_greater(c->f, v, best)) best = v;
	}
	return best;
}
static int boundary_value(const lctx* c, const int64_t k[3]) {
	return (k[0] == 0 || k[0] == c->dX - 1) + (k[1] == 0 || k[1] == c->dY - 1) + (k[2] == 0 || k[2] == c->dZ - 1);
}
/* facets / cofacets in the iterator orders (+x,-x,+y,-y,+z,-z) */
static int cfacets(const lctx* c, int64_t id, int64_t out[6]) {
	int64_t k[3], st[3] = { 1, c->dX, c->dX * c->dY }, d[3] = { c->dX, c->dY, c->dZ };
	ccoords(c, id, k);
	int n = 0;
	(void)d;
	for (int a = 0; a < 3; a++) if (k[a] & 1) { out[n++] = id + st[a]; out[n++] = id - st[a]; }
	return n;
}
static int ccofacets(const lctx* c, int64_t id, int64_t out[6]) {
	int64_t k[3], st[3] = { 1, c->dX, c->dX * c->dY }, d[3] = { c->dX, c->dY, c->dZ };
	ccoords(c, id, k);
	int n = 0;
	for (int a = 0; a < 3; a++)
		if (!(k[a] & 1)) {
			if (k[a] != d[a] - 1) out[n++] = id + st[a];
			if (k[a] != 0) out[n++] = id - st[a];
		}
	return n;
}

/* ---- 1. extremum graph --------------------------------------------------------- */

/* rec_td (gi_extrema_region_builder.h:286-300): follow the V-path down to a minimum */
static int64_t rec_td(const lctx* c, int64_t cell) {
	for (;;) {
		if (gcrit(c, cell)) return cell;
		int64_t pair = gpair(c, cell);
		if (gcrit(c, pair)) return pair;
		int64_t fc[6];
		cfacets(c, pair, fc);
		cell = (fc[0] == cell) ? fc[1] : fc[0];
	}
}
/* rec_tu (:330-346): follow the V-path up to a maximum */
static int64_t rec_tu(const lctx* c, int64_t cell) {
	for (;;) {
		if (gcrit(c, cell)) return cell;
		int64_t pair = gpair(c, cell);
		if (gcrit(c, pair)) return pair;
		int64_t cf[6];
		int n = ccofacets(c, pair, cf);
		cell = (cf[0] == cell && n > 1) ? cf[1] : cf[0];
	}
}

typedef struct { int64_t cell; int32_t rep; float fval; } ext_t;
typedef struct { int64_t saddle; int32_t e1, e2; float pers, sval; } arc_t;

/* MergeArc ordering of the priority queue: smallest persistence first, then the
 * smallest saddle cell index (gi_extrema_region_builder.h:55-60). */
static int arc_before(const arc_t* a, const arc_t* b) {
	if (a->pers < b->pers) return 1;
	if (a->pers > b->pers) return 0;
	return a->saddle < b->saddle;
}
typedef struct { arc_t* a; int64_t n, cap; } heap_t;
static void heap_push(heap_t* h, arc_t v) {
	if (h->n == h->cap) { h->cap = h->cap ? 2 * h->cap : 1024; h->a = (arc_t*)realloc(h->a, sizeof(arc_t) * (size_t)h->cap); }
	int64_t i = h->n++;
	h->a[i] = v;
	while (i > 0) {
		int64_t p = (i - 1) / 2;
		if (!arc_before(&h->a[i], &h->a[p])) break;
		arc_t t = h->a[i]; h->a[i] = h->a[p]; h->a[p] = t;
		i = p;
	}
}
static arc_t heap_pop(heap_t* h) {
	arc_t top = h->a[0];
	h->a[0] = h->a[--h->n];
	int64_t i = 0;
	for (;;) {
		int64_t l = 2 * i + 1, r = l + 1, m = i;
		if (l < h->n && arc_before(&h->a[l], &h->a[m])) m = l;
		if (r < h->n && arc_before(&h->a[r], &h->a[m])) m = r;
		if (m == i) break;
		arc_t t = h->a[i]; h->a[i] = h->a[m]; h->a[m] = t;
		i = m;
	}
	return top;
}

static int32_t find_rep(ext_t* E, int32_t lid) {
	int32_t r = lid;
	while (E[r].rep != r) r = E[r].rep;
	while (E[lid].rep != r) { int32_t nx = E[lid].rep; E[lid].rep = r; lid = nx; }
	return r;
}

/* lessThan of TopologicalMaxVertexMeshFunction (gi_topological_max_vertex_mesh_function.h:47-58) */
static int cell_less(const lctx* c, int64_t a, int64_t b) {
	int64_t va = highest_vertex(c, a), vb = highest_vertex(c, b);
	float fa = c->f[va], fb = c->f[vb];
	if (fa < fb) return 1;
	if (fb < fa) return 0;
	if (va < vb) return 1;
	if (vb < va) return 0;
	return a < b;
}

static int64_t lookup_ext(const int64_t* cells, int64_t n, int64_t cell) {
	int64_t lo = 0, hi = n - 1;
	while (lo <= hi) {
		int64_t mid = (lo + hi) / 2;
		if (cells[mid] == cell) return mid;
		if (cells[mid] < cell) lo = mid + 1; else hi = mid - 1;
	}
	return -1;
}

/* Fills ext_cells (extremum cell ids, increasing) and ext_rep (representative list
 * id after merging) and returns the number of extrema.  Buffers hold ncells entries. */
static int64_t extremum_graph(const lctx* c, float threshold, int64_t* ext_cells, int32_t* ext_rep) {
	const int64_t nc = c->dX * c->dY * c->dZ;
	const int ext_dim = c->dir < 0 ? 0 : 3, sad_dim = c->dir < 0 ? 1 : 2;
	int64_t ne = 0;
	for (int64_t id = 0; id < nc; id++) {
		if (!gcrit(c, id)) continue;
		int64_t k[3];
		ccoords(c, id, k);
		if (cdim(k) == ext_dim) ext_cells[ne++] = id;
	}
	ext_t* E = (ext_t*)malloc(sizeof(ext_t) * (size_t)(ne + 1));
	for (int64_t i = 0; i < ne; i++) {
		E[i].cell = ext_cells[i];
		E[i].rep = (int32_t)i;
		E[i].fval = c->f[highest_vertex(c, ext_cells[i])];   /* cellValue */
	}
	heap_t h = { 0, 0, 0 };
	for (int64_t id = 0; id < nc; id++) {
		if (!gcrit(c, id)) continue;
		int64_t k[3];
		ccoords(c, id, k);
		if (cdim(k) != sad_dim) continue;
		int64_t a, b;
		if (c->dir < 0) {
			int64_t fc[6];
			cfacets(c, id, fc);
			a = rec_td(c, fc[0]);
			b = rec_td(c, fc[1]);
		} else {
			if (boundary_value(c, k) != 0) continue;           /* trace_up_2saddle :315-318 */
			int64_t cf[6];
			int n = ccofacets(c, id, cf);
			a = rec_tu(c, cf[0]);
			b = (n > 1) ? rec_tu(c, cf[1]) : a;
		}
		if (a == b) continue;
		arc_t m;
		m.saddle = id;
		m.e1 = (int32_t)lookup_ext(ext_cells, ne, a);
		m.e2 = (int32_t)lookup_ext(ext_cells, ne, b);
		m.sval = c->f[highest_vertex(c, id)];
		float d1 = E[m.e1].fval - m.sval, d2 = E[m.e2].fval - m.sval;
		if (d1 < 0) d1 *= -1;
		if (d2 < 0) d2 *= -1;
		m.pers = d1 < d2 ? d1 : d2;
		heap_push(&h, m);
	}
	/* SimplifyToThreshold / PerformCancel (:98-145, 232-245) */
	const int min_hierarchy = c->dir < 0;
	while (h.n) {
		arc_t m = heap_pop(&h);
		if (m.pers > threshold) continue;
		int32_t r1 = find_rep(E, m.e1), r2 = find_rep(E, m.e2);
		if (r1 == r2) continue;
		if (m.e1 != r1 || m.e2 != r2) {
			/* the reference names its locals crosswise here: rep1 <- extremum 2 */
			float d1 = fabsf(m.sval - E[r2].fval);
			float d2 = fabsf(m.sval - E[r1].fval);
			if (d1 < d2) {
				if (d1 > threshold) continue;
				m.pers = d1; m.e1 = r2; m.e2 = r1;
			} else {
				if (d2 > threshold) continue;
				m.pers = d2; m.e1 = r1; m.e2 = r2;
			}
			heap_push(&h, m);
			continue;
		}
		/* MergeByVal (:83-91) */
		if (cell_less(c, E[r1].cell, E[r2].cell) ^ min_hierarchy) E[r1].rep = E[r2].rep;
		else E[r2].rep = E[r1].rep;
	}
	for (int64_t i = 0; i < ne; i++) ext_rep[i] = find_rep(E, (int32_t)i);
	free(h.a);
	free(E);
	return ne;
}

/* ---- 2. certain terminal regions --------------------------------------------- */

typedef struct { int64_t* a; int64_t n, cap; } vheap_t;
static void vheap_push(const lctx* c, vheap_t* h, int64_t v) {
	if (h->n == h->cap) { h->cap = h->cap ? 2 * h->cap : 1024; h->a = (int64_t*)realloc(h->a, sizeof(int64_t) * (size_t)h->cap); }
	int64_t i = h->n++;
	h->a[i] = v;
	while (i > 0) {
		int64_t p = (i - 1) / 2;
		if (!comes_before(c, h->a[i], h->a[p])) break;
		int64_t t = h->a[i]; h->a[i] = h->a[p]; h->a[p] = t;
		i = p;
	}
}
static int64_t vheap_pop(const lctx* c, vheap_t* h) {
	int64_t top = h->a[0];
	h->a[0] = h->a[--h->n];
	int64_t i = 0;
	for (;;) {
		int64_t l = 2 * i + 1, r = l + 1, m = i;
		if (l < h->n && comes_before(c, h->a[l], h->a[m])) m = l;
		if (r < h->n && comes_before(c, h->a[r], h->a[m])) m = r;
		if (m == i) break;
		int64_t t = h->a[i]; h->a[i] = h->a[m]; h->a[m] = t;
		i = m;
	}
	return top;
}

/* InspectPriorRegions (gi_extrema_region_builder.h:806-857) */
static int32_t inspect_prior(const lctx* c, const int32_t* lab, int64_t v) {
	int32_t ext = lab[v];
	int has = 0;
	int64_t nb[6];
	int n = neighbors6(c, v, nb);
	for (int i = 0; i < n; i++) {
		if (!comes_before(c, nb[i], v)) continue;
		if (lab[nb[i]] == -1) return -1;
		if (!has) { ext = lab[nb[i]]; has = 1; }
		else if (ext != lab[nb[i]]) return -1;
	}
	return ext;
}

/* Expand_Lower_Neighborhood (:863-953) for every unique id in order.
 * seeds: vertex ids grouped by unique id: seed_start[u]..seed_start[u+1]. */
static void terminal_regions(const lctx* c, const int64_t* seeds, const int64_t* seed_start, int64_t nuniq,
                             int32_t* lab) {
	const int64_t nv = c->X * c->Y * c->Z;
	int64_t* stamp = (int64_t*)calloc((size_t)nv, sizeof(int64_t));  /* enqueued_set, per unique id */
	for (int64_t v = 0; v < nv; v++) lab[v] = -1;
	vheap_t h = { 0, 0, 0 };
	for (int64_t u = 0; u < nuniq; u++) {
		const int64_t tag = u + 1;
		for (int64_t s = seed_start[u]; s < seed_start[u + 1]; s++) {
			stamp[seeds[s]] = tag;
			lab[seeds[s]] = (int32_t)u;
		}
		for (int64_t s = seed_start[u]; s < seed_start[u + 1]; s++) {
			/* Enqueue_Later_Neighbors (:779-801) */
			int64_t nb[6];
			int n = neighbors6(c, seeds[s], nb);
			for (int i = 0; i < n; i++)
				if (lab[nb[i]] == -1 && comes_before(c, seeds[s], nb[i]) && stamp[nb[i]] != tag) {
					stamp[nb[i]] = tag;
					vheap_push(c, &h, nb[i]);
				}
		}
		while (h.n) {
			int64_t v = vheap_pop(c, &h);
			int32_t l = inspect_prior(c, lab, v);
			if (l < 0) continue;
			lab[v] = l;
			int64_t nb[6];
			int n = neighbors6(c, v, nb);
			for (int i = 0; i < n; i++)
				if (lab[nb[i]] == -1 && comes_before(c, v, nb[i]) && stamp[nb[i]] != tag) {
					stamp[nb[i]] = tag;
					vheap_push(c, &h, nb[i]);
				}
		}
	}
	free(h.a);
	free(stamp);
}

/* ---- 3. numerical integration ------------------------------------------------- */

typedef struct {
	const lctx* c;
	const double* G;          /* gradient, 3 doubles per vertex */
	const uint8_t* desttype;
	int terminal_only;        /* TerminateNearOriginalCertain instead of ...PathCompressedRegion */
	float ethresh, gthresh;
	double max_step;
	int step_mult;            /* StepMultiplier: -1 ascending (downhill), +1 descending */
	/* the saddle-line digitizers' checkers (cell_mode 1: TerminateNearAssignedHex,
	 * 2: TerminateNearAssignedVert, gi_advection_checker.h:60-100), over cells[] */
	const uint8_t* cells;
	int cell_target;
	int cell_mode;
} adv_t;

static inline v3d vload(const double* G, int64_t v) { v3d r = { G[3 * v], G[3 * v + 1], G[3 * v + 2] }; return r; }
static inline double magsq(v3d a) { return (a.x * a.x) + (a.y * a.y) + (a.z * a.z); }
/* Lerp: a*(1-t) + b*t (gi_vectors.h:349-351) */
static inline v3d lerp(v3d a, v3d b, double t) {
	double u = 1.0 - t;
	v3d r = { a.x * u + b.x * t, a.y * u + b.y * t, a.z * u + b.z * t };
	return r;
}

/* GatherSurrounding (clamped) / ...NoBoundaryCheck, then the 8 gradients, k-j-i order */
static void surround(const adv_t* A, const int64_t b[3], int clamp, v3d vals[8]) {
	const lctx* c = A->c;
	int64_t ext[3] = { c->X, c->Y, c->Z }, vv[3][2];
	for (int a = 0; a < 3; a++) {
		vv[a][0] = b[a];
		vv[a][1] = b[a] + 1;
		if (clamp) {
			if (b[a] < 0) vv[a][0] = 0;
			if (b[a] >= ext[a] - 1) { vv[a][0] = vv[a][1] = ext[a] - 1; }
			else if (b[a] >= ext[a]) { vv[a][1] = ext[a] - 1; }
		}
	}
	int n = 0;
	for (int k = 0; k < 2; k++)
		for (int j = 0; j < 2; j++)
			for (int i = 0; i < 2; i++) vals[n++] = vload(A->G, vidx(c, vv[0][i], vv[1][j], vv[2][k]));
}

/* TriLinInterpGrad (gi_regular_grid_trilinear_function.h:211-229) */
static v3d trilin(v3d s, const int64_t b[3], const v3d vals[8]) {
	double fx = s.x - (double)b[0], fy = s.y - (double)b[1], fz = s.z - (double)b[2];
	v3d x0 = lerp(vals[0], vals[1], fx), x1 = lerp(vals[2], vals[3], fx);
	v3d x2 = lerp(vals[4], vals[5], fx), x3 = lerp(vals[6], vals[7], fx);
	v3d y0 = lerp(x0, x1, fy), y1 = lerp(x2, x3, fy);
	return lerp(y0, y1, fz);
}

static inline double clampd(double v, int64_t n) { if (v < 0) v = 0; if (v >= (double)n) v = (double)n - 1; return v; }

/* nearest vertex of a point: Vec3l(p + 0.5), clamped first near the boundary */
static int64_t nearest_vertex(const lctx* c, v3d p, int clamp) {
	v3d q = { p.x + 0.5, p.y + 0.5, p.z + 0.5 };
	if (clamp) { q.x = clampd(q.x, c->X); q.y = clampd(q.y, c->Y); q.z = clampd(q.z, c->Z); }
	return vidx(c, (int64_t)q.x, (int64_t)q.y, (int64_t)q.z);
}

static int checker(const adv_t* A, v3d np, int clamp) {
	if (A->cell_mode) {
		/* nearboundary: stop at once; else the hex holding the point (floor * 2 + 1) or
		 * the vertex nearest it (floor(p + 0.5) * 2) carries the target label */
		if (clamp) return EV_HIT_PREASSIGNED;
		const lctx* c = A->c;
		const double p[3] = { np.x, np.y, np.z };
		int64_t k[3];
		for (int a = 0; a < 3; a++)
			k[a] = A->cell_mode == 1 ? (int64_t)floor(p[a]) * 2 + 1 : (int64_t)floor(p[a] + 0.5) * 2;
		const int64_t id = k[0] + c->dX * (k[1] + c->dY * k[2]);
		return A->cells[id] == A->cell_target ? EV_HIT_PREASSIGNED : EV_NONE;
	}
	int64_t id = nearest_vertex(A->c, np, clamp);
	uint8_t t = A->desttype[id];
	if (A->terminal_only) return t == DT_CERTAIN_TERMINAL ? EV_HIT_PREASSIGNED : EV_NONE;
	return (t == DT_ASSIGNED || t == DT_CERTAIN_TERMINAL) ? EV_HIT_PREASSIGNED : EV_NONE;
}

/* AdvectThroughVoxelNoCheck / NearBoundary (gi_adaptive_euler_advector.h:51-176, 182-305) */
static int advect(const adv_t* A, v3d* cur, int* iters, int nearb) {
	const lctx* c = A->c;
	v3d vals[8];
	v3d old = *cur;
	int64_t b[3];
	if (nearb) {
		b[0] = (int64_t)clampd(cur->x, c->X); b[1] = (int64_t)clampd(cur->y, c->Y); b[2] = (int64_t)clampd(cur->z, c->Z);
	} else {
		b[0] = (int64_t)cur->x; b[1] = (int64_t)cur->y; b[2] = (int64_t)cur->z;
	}
	surround(A, b, nearb, vals);
	v3d g = trilin(*cur, b, vals);
	float gm = (float)sqrt(magsq(g));
	float step = (float)(A->max_step / gm);
	while ((*iters)-- > 0) {
		if (!(old.x == cur->x && old.y == cur->y && old.z == cur->z)) {
			if ((int)cur->x != (int)old.x || (int)cur->y != (int)old.y || (int)cur->z != (int)old.z) return EV_OUT_OF_VOXEL;
			g = trilin(*cur, b, vals);
			gm = (float)sqrt(magsq(g));
			if (gm * step > A->max_step) step = (float)(A->max_step / gm);
			old = *cur;
		}
		if (gm < A->gthresh) return EV_LOW_GRADIENT;
		/* full step: Vec3d * float multiplies in float */
		const float sm = (float)A->step_mult * step;
		v3d e1 = { (double)((float)g.x * sm), (double)((float)g.y * sm), (double)((float)g.z * sm) };
		/* two half steps in double, the second with the gradient at the midpoint */
		const double hs = (double)step * ((double)A->step_mult * 0.5);
		v3d hd = { g.x * hs, g.y * hs, g.z * hs };
		v3d hp = { cur->x + hd.x, cur->y + hd.y, cur->z + hd.z };
		v3d hg = trilin(hp, b, vals);
		v3d e2 = { hg.x * hs + hd.x, hg.y * hs + hd.y, hg.z * hs + hd.z };
		v3d df = { e2.x - e1.x, e2.y - e1.y, e2.z - e1.z };
		float err = (float)magsq(df);
		if (err < A->ethresh) {
			v3d np = { cur->x + e2.x, cur->y + e2.y, cur->z + e2.z };
			if (nearb) { np.x = clampd(np.x, c->X); np.y = clampd(np.y, c->Y); np.z = clampd(np.z, c->Z); }
			*cur = np;
			float a = (float)(step * 1.8), bb = (float)(A->max_step / gm);
			step = a < bb ? a : bb;
			int ev = checker(A, *cur, nearb);
			if (ev != EV_NONE) return ev;
		} else {
			step = (float)(step * 0.5);
		}
	}
	return EV_OVER_MAX_ITERATIONS;
}

static int dist_to_boundary(const lctx* c, int64_t x, int64_t y, int64_t z) {
	int64_t a[3] = { x, y, z }, e[3] = { c->X, c->Y, c->Z }, m = INT64_MAX;
	for (int i = 0; i < 3; i++) {
		int64_t d = a[i] < e[i] - 1 - a[i] ? a[i] : e[i] - 1 - a[i];
		if (d < m) m = d;
	}
	return (int)m;
}

/* Integrates from vertex v until a stop event; returns the id of the stop vertex.
 * If path/plen are given, records every visited nearest vertex. */
static int64_t trace(const adv_t* A, int64_t v, int limit, int64_t** path, int64_t* plen, int64_t* pcap) {
	const lctx* c = A->c;
	int64_t x = v % c->X, y = (v / c->X) % c->Y, z = v / (c->X * c->Y);
	v3d cur = { (double)x, (double)y, (double)z };
	int iters = limit;
	for (;;) {
		int ev;
		int64_t nid;
		if (dist_to_boundary(c, x, y, z) <= 1) {
			ev = advect(A, &cur, &iters, 1);
			v3d q = { clampd(cur.x + 0.5, c->X), clampd(cur.y + 0.5, c->Y), clampd(cur.z + 0.5, c->Z) };
			x = (int64_t)q.x; y = (int64_t)q.y; z = (int64_t)q.z;
		} else {
			ev = advect(A, &cur, &iters, 0);
			x = (int64_t)(cur.x + 0.5); y = (int64_t)(cur.y + 0.5); z = (int64_t)(cur.z + 0.5);
		}
		nid = vidx(c, x, y, z);
		if (path) {
			if (*plen == *pcap) { *pcap *= 2; *path = (int64_t*)realloc(*path, sizeof(int64_t) * (size_t)*pcap); }
			(*path)[(*plen)++] = nid;
		}
		if (ev == EV_OUT_OF_VOXEL) continue;
		return nid;
	}
}

/* ---- saddle streamline digitizers (ondemandaccurate needASC1 / needDSC1) ----------
 *
 * ondemandaccurate.cxx:254-382 (ReIntegrateUpFrom2Saddles) and :383-505
 * (ReIntegrateDownFrom1Saddles) at one thread, with
 * DigitizingNumericStreamlineIntegrator3dASC / 3dDSC (gi_numeric_streamline_integrator.h:
 * 525-796, 797-1080): saddles in decreasing value (ascending lines from 2-saddles) or
 * increasing value (descending lines from 1-saddles), ties by decreasing cell id; around
 * each saddle a breadth-first walk of at most five cells through its cofacets (facets)
 * and their pairs collects the hexes (vertices) to start streamlines from, at their
 * centroids; every streamline labels the hex-face-hex (vertex-edge-vertex) chain it
 * crosses with the target label, each segment stopping at the first cell already
 * labelled, and stops itself near a labelled hex (vertex) or near the boundary; then
 * the saddle itself takes the label. */

/* DigitizeSegmentInternal: the segment a -> b of one voxel advection (its result is not
 * used by the caller) */
static void digitize_segment(const lctx* c, v3d a0, v3d b0, int dsc, uint8_t* cells, int target) {
	double a[3] = { a0.x, a0.y, a0.z }, b[3] = { b0.x, b0.y, b0.z };
	if (dsc) for (int d = 0; d < 3; d++) { a[d] += 0.5; b[d] += 0.5; }
	const double a2b[3] = { b[0] - a[0], b[1] - a[1], b[2] - a[2] };
	int64_t idx[3];
	double tt[3];
	int n = 0;
	for (int d = 0; d < 3; d++) {
		const int va = (int)floor(a[d]), vb = (int)floor(b[d]);
		if (va == vb) continue;
		const int plane = va > vb ? va : vb;
		const double t = ((double)plane - a[d]) / (b[d] - a[d]);
		tt[n] = t;
		if (t < 0 || t > 1) return;
		int64_t k[3];
		for (int e = 0; e < 3; e++) {
			const double q = a2b[e] * t;
			k[e] = (int64_t)floor(q + a[e]) * 2 + (e == d ? 0 : 1) - (dsc ? 1 : 0);
		}
		idx[n++] = k[0] + c->dX * (k[1] + c->dY * k[2]);
	}
	if (n == 0) return;
	for (int i = 0; i < n; i++)
		for (int j = i; j < n; j++)
			if (tt[i] > tt[j]) {
				int64_t ti = idx[i]; idx[i] = idx[j]; idx[j] = ti;
				double td = tt[i]; tt[i] = tt[j]; tt[j] = td;
			}
	int64_t start;
	{
		int64_t k[3];
		for (int e = 0; e < 3; e++) k[e] = (int64_t)floor(a[e]) * 2 + (dsc ? 0 : 1);
		start = k[0] + c->dX * (k[1] + c->dY * k[2]);
	}
	for (int i = 0; i < n; i++) {
		const int64_t face = idx[i];
		int64_t around[6];
		const int m = dsc ? cfacets(c, face, around) : ccofacets(c, face, around);
		int has_start = 0;
		int64_t next = -1;
		for (int j = 0; j < m; j++) {
			if (around[j] == start) has_start = 1;
			else next = around[j];
		}
		if (!has_start) continue;
		if (cells[start] == target) return;
		cells[start] = (uint8_t)target;
		if (cells[face] == target) return;
		cells[face] = (uint8_t)target;
		start = next;
	}
}

/* IntegrateStreamline of the digitizing integrators, from `seed` (grid coordinates) */
static void digitize_streamline(const adv_t* A, v3d seed, int limit, uint8_t* cells, int target) {
	const lctx* c = A->c;
	int64_t x = (int64_t)(seed.x + 0.5), y = (int64_t)(seed.y + 0.5), z = (int64_t)(seed.z + 0.5);
	v3d cur = seed;
	int iters = limit;
	for (;;) {
		const v3d old = cur;
		int ev;
		if (dist_to_boundary(c, x, y, z) <= 1) {
			ev = advect(A, &cur, &iters, 1);
			v3d q = { clampd(cur.x + 0.5, c->X), clampd(cur.y + 0.5, c->Y), clampd(cur.z + 0.5, c->Z) };
			x = (int64_t)q.x; y = (int64_t)q.y; z = (int64_t)q.z;
		} else {
			ev = advect(A, &cur, &iters, 0);
			x = (int64_t)(cur.x + 0.5); y = (int64_t)(cur.y + 0.5); z = (int64_t)(cur.z + 0.5);
			digitize_segment(c, old, cur, A->cell_mode == 2, cells, target);
		}
		if (ev == EV_LOW_GRADIENT || ev == EV_HIT_EXTREMUM || ev == EV_HIT_PREASSIGNED || ev == EV_OVER_MAX_ITERATIONS)
			return;
	}
}

typedef struct { float key; int64_t id; } crit_t;
static int crit_less(const void* pa, const void* pb) {  /* std::pair<float, INDEX_TYPE> order */
	const crit_t* a = (const crit_t*)pa;
	const crit_t* b = (const crit_t*)pb;
	if (a->key < b->key) return -1;
	if (b->key < a->key) return 1;
	return (a->id > b->id) - (a->id < b->id);
}

/* a small set of cell ids (the breadth-first walk visits at most a few dozen) */
typedef struct { int64_t v[256]; int n; } cellset_t;
static int cs_has(const cellset_t* s, int64_t id) {
	for (int i = 0; i < s->n; i++) if (s->v[i] == id) return 1;
	return 0;
}
static void cs_add(cellset_t* s, int64_t id) {
	if (!cs_has(s, id) && s->n < 256) s->v[s->n++] = id;
}

/* dsc 0: ascending lines from the 2-saddles (target labels on hexes and faces);
 * 1: descending lines from the 1-saddles (vertices and edges) */
static void saddle_lines(const lctx* c, const double* G, const oracle_label_params* P, int dsc, uint8_t* cells,
                         int target) {
	const int64_t NC = c->dX * c->dY * c->dZ;
	const int sdim = dsc ? 1 : 2, tdim = dsc ? 0 : 3;
	int64_t nc = 0, cap = 1024;
	crit_t* cr = (crit_t*)malloc(sizeof(crit_t) * (size_t)cap);
	for (int64_t id = 0; id < NC; id++) {
		int64_t k[3];
		ccoords(c, id, k);
		if (cdim(k) != sdim || !gcrit(c, id)) continue;
		if (nc == cap) { cap *= 2; cr = (crit_t*)realloc(cr, sizeof(crit_t) * (size_t)cap); }
		const float v = c->f[highest_vertex(c, id)];
		cr[nc].key = dsc ? -1 * v : v;
		cr[nc].id = id;
		nc++;
	}
	qsort(cr, (size_t)nc, sizeof(crit_t), crit_less);
	adv_t A = { c, G, NULL, 0, P->error_threshold, P->gradient_threshold, P->max_step, dsc ? -1 : 1,
	            cells, target, dsc ? 2 : 1 };
	for (int64_t li = nc - 1; li >= 0; li--) {
		const int64_t sad = cr[li].id;
		int64_t result[256], queue[256];
		int nr = 0, qh = 0, qt = 0;
		cellset_t visited;
		visited.n = 0;
		queue[qt++] = sad;
		for (int counter = 4; qh < qt && counter >= 0; counter--) {
			const int64_t cur = queue[qh++];
			cs_add(&visited, cur);
			int64_t around[6];
			const int m = dsc ? cfacets(c, cur, around) : ccofacets(c, cur, around);
			for (int j = 0; j < m; j++) {
				const int64_t t = around[j];
				if (cs_has(&visited, t)) continue;
				if (gcrit(c, t)) {
					if (nr < 256) result[nr++] = t;
					cs_add(&visited, t);
				} else {
					const int64_t pr = gpair(c, t);
					if (nr < 256) result[nr++] = t;
					cs_add(&visited, t);
					cs_add(&visited, pr);
					if (qt < 256) queue[qt++] = pr;
				}
			}
		}
		for (int i = 0; i < nr; i++) {
			int64_t k[3];
			ccoords(c, result[i], k);
			if (cdim(k) != tdim) continue;
			const v3d seed = { (double)k[0] * 0.5, (double)k[1] * 0.5, (double)k[2] * 0.5 };
			digitize_streamline(&A, seed, P->iteration_limit, cells, target);
		}
		cells[sad] = (uint8_t)target;
	}
	free(cr);
}

static int cmp_i64(const void* a, const void* b) {
	int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
	return (x > y) - (x < y);
}

/* BeginIntegration (gi_numeric_integrator_path_compressing.h:75-433), one thread */
static void integrate(const lctx* c, double* G, int32_t* lab, const int64_t* zero_grad, int64_t nzero,
                      const oracle_label_params* P) {
	const int64_t N = c->X * c->Y * c->Z;
	uint8_t* dt = (uint8_t*)malloc((size_t)N);
	for (int64_t i = 0; i < N; i++) dt[i] = lab[i] == -1 ? DT_UNASSIGNED : DT_CERTAIN_TERMINAL;
	for (int64_t i = 0; i < nzero; i++) { G[3 * zero_grad[i]] = 0; G[3 * zero_grad[i] + 1] = 0; G[3 * zero_grad[i] + 2] = 0; }
	adv_t A = { c, G, dt, 0, P->error_threshold, P->gradient_threshold, P->max_step, c->dir < 0 ? -1 : 1,
	            NULL, 0, 0 };
	int64_t pcap = 256, plen;
	int64_t* path = (int64_t*)malloc(sizeof(int64_t) * (size_t)pcap);
	/* first pass, strided visiting order (:166-174) with one thread */
	for (int64_t kk = 1; kk <= N * 4; kk *= 2) {
		int64_t start = N / kk, stride = (N * 2) / kk;
		if (stride == 0) continue;
		for (int64_t i = start; i < N; i += stride) {
			if (dt[i] != DT_UNASSIGNED) continue;
			plen = 0;
			path[plen++] = i;
			int64_t end = trace(&A, i, P->iteration_limit, &path, &plen, &pcap);
			int32_t dest = lab[end];
			for (int64_t j = 0; j < plen; j++)
				if (dt[path[j]] == DT_UNASSIGNED) { lab[path[j]] = dest; dt[path[j]] = DT_ASSIGNED; }
		}
	}
	/* vertices with a differently labelled 6-neighbour (:279-307) */
	int64_t ncur = 0, cap = 1024;
	int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)cap);
	uint8_t* inset = (uint8_t*)calloc((size_t)N, 1);
#define ADD(v) do { if (!inset[v]) { inset[v] = 1; if (ncur == cap) { cap *= 2; cur = (int64_t*)realloc(cur, sizeof(int64_t) * (size_t)cap); } cur[ncur++] = (v); } } while (0)
	for (int64_t i = 0; i < N; i++) {
		int64_t nb[6];
		int n = neighbors6(c, i, nb);
		for (int j = 0; j < n; j++) {
			if (nb[j] > i) continue;
			if (lab[i] != lab[nb[j]]) {
				if (dt[i] == DT_ASSIGNED) ADD(i);
				if (dt[nb[j]] == DT_ASSIGNED) ADD(nb[j]);
			}
		}
	}
	/* fix-up to a fixpoint (:330-415): re-integrate, stopping only at certain terminals */
	A.terminal_only = 1;
	int64_t* next = NULL;
	while (ncur) {
		qsort(cur, (size_t)ncur, sizeof(int64_t), cmp_i64);
		for (int64_t i = 0; i < ncur; i++) inset[cur[i]] = 0;
		next = (int64_t*)malloc(sizeof(int64_t) * (size_t)ncur);
		memcpy(next, cur, sizeof(int64_t) * (size_t)ncur);
		int64_t nproc = ncur;
		ncur = 0;
		for (int64_t i = 0; i < nproc; i++) {
			int64_t v = next[i];
			int32_t init = lab[v];
			int64_t end = trace(&A, v, P->iteration_limit, NULL, NULL, NULL);
			int32_t nl = lab[end];
			lab[v] = nl;
			dt[v] = DT_CERTAIN_NONTERMINAL;
			if (nl != init) {
				int64_t nb[6];
				int n = neighbors6(c, v, nb);
				for (int j = 0; j < n; j++)
					if (dt[nb[j]] == DT_ASSIGNED && lab[nb[j]] != nl) ADD(nb[j]);
			}
		}
		free(next);
	}
#undef ADD
	free(inset);
	free(cur);
	free(path);
	free(dt);
}

/* ---- 4. isolated region cleaner ------------------------------------------------ */

static int64_t uf_find(int64_t* d, int64_t v) {
	int64_t r = v;
	while (d[r] != r) r = d[r];
	while (d[v] != r) { int64_t nx = d[v]; d[v] = r; v = nx; }
	return r;
}

/* IsolatedCCRegionRemoverNEW::ComputeOutput (gi_isolated_region_remover.h:155-192) */
static void clean_regions(const lctx* c, int32_t* lab) {
	const int64_t N = c->X * c->Y * c->Z;
	int64_t* d = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
	for (int64_t i = 0; i < N; i++) d[i] = i;
	for (int64_t i = 0; i < N; i++) {      /* MergeWithSameNeighbors */
		int64_t nb[6];
		int n = neighbors6(c, i, nb);
		for (int j = 0; j < n; j++) {
			if (lab[i] != lab[nb[j]]) continue;
			int64_t a = uf_find(d, i), b = uf_find(d, nb[j]);
			if (comes_before(c, a, b)) d[b] = a; else d[a] = b;   /* MergeByOrder */
		}
	}
	int64_t nroots = 0;
	int64_t* roots = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
	for (int64_t i = 0; i < N; i++) if (d[i] == i) roots[nroots++] = i;
	for (int64_t r = 0; r < nroots; r++) {   /* MergeBoundaryExtrema */
		int64_t id = roots[r];
		int64_t nb[6];
		int n = neighbors6(c, id, nb);
		if (n == 0) continue;
		int32_t id_reg = lab[uf_find(d, id)];
		int64_t earliest = id;
		for (int j = 0; j < n; j++) {
			if (!comes_before(c, nb[j], id)) continue;
			if (id_reg == lab[uf_find(d, nb[j])]) continue;
			if (comes_before(c, nb[j], earliest)) earliest = nb[j];
		}
		d[id] = uf_find(d, earliest);            /* MergeAToB (a no-op when earliest == id) */
	}
	int32_t* out = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
	for (int64_t i = 0; i < N; i++) out[i] = lab[i] != -1 ? lab[uf_find(d, i)] : -1;
	memcpy(lab, out, sizeof(int32_t) * (size_t)N);
	free(out);
	free(roots);
	free(d);
}

/* ---- public entry points ------------------------------------------------------- */

static int ctx_init(lctx* c, const float* f, const uint8_t* grad, int64_t X, int64_t Y, int64_t Z, int dir) {
	if (X < 2 || Y < 2 || Z < 2 || (dir != -1 && dir != 1)) return -1;
	c->X = X; c->Y = Y; c->Z = Z;
	c->dX = 2 * X - 1; c->dY = 2 * Y - 1; c->dZ = 2 * Z - 1;
	c->f = f; c->grad = grad; c->dir = dir;
	return 0;
}

/* Seeds of the certain regions: for every unique representative (increasing), the
 * vertices of its extrema (minima: the vertex; maxima: Cell2HighestVertex of the
 * hex).  Returns the number of unique ids; seeds/seed_start sized by the caller. */
static int64_t build_seeds(const lctx* c, float threshold, int64_t* seeds, int64_t* seed_start) {
	const int64_t nv = c->X * c->Y * c->Z;   /* bounds the number of minima and of hexes */
	int64_t* cells = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nv + 16));
	int32_t* reps = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nv + 16));
	int64_t ne = extremum_graph(c, threshold, cells, reps);
	/* counting sort by representative */
	int64_t* cnt = (int64_t*)calloc((size_t)(ne + 1), sizeof(int64_t));
	for (int64_t i = 0; i < ne; i++) cnt[reps[i] + 1]++;
	int64_t nuniq = 0;
	int64_t* uid = (int64_t*)malloc(sizeof(int64_t) * (size_t)(ne + 1));
	for (int64_t r = 0; r < ne; r++) uid[r] = cnt[r + 1] ? nuniq++ : -1;
	seed_start[0] = 0;
	{
		int64_t u = 0;
		for (int64_t r = 0; r < ne; r++) if (cnt[r + 1]) { seed_start[u + 1] = seed_start[u] + cnt[r + 1]; u++; }
	}
	int64_t* fill = (int64_t*)calloc((size_t)(nuniq + 1), sizeof(int64_t));
	for (int64_t i = 0; i < ne; i++) {
		int64_t u = uid[reps[i]];
		int64_t v = c->dir < 0 ? cell_vertex(c, cells[i]) : highest_vertex(c, cells[i]);
		seeds[seed_start[u] + fill[u]++] = v;
	}
	free(fill); free(uid); free(cnt); free(reps); free(cells);
	return nuniq;
}

int oracle_terminal_regions_3d(const float* f, const uint8_t* grad, int64_t X, int64_t Y, int64_t Z, int dir,
                               float presimp_threshold, int32_t* labels) {
	lctx c;
	if (ctx_init(&c, f, grad, X, Y, Z, dir)) return -1;
	const int64_t nv = X * Y * Z;
	int64_t* seeds = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nv + 16));
	int64_t* start = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nv + 16));
	int64_t nu = build_seeds(&c, presimp_threshold, seeds, start);
	terminal_regions(&c, seeds, start, nu, labels);
	free(start); free(seeds);
	return 0;
}

/* The cleaner alone on labels (in place); dir -1 ASC, +1 DSC. */
int oracle_clean_regions_3d(const float* f, int64_t X, int64_t Y, int64_t Z, int dir, int32_t* labels) {
	lctx c;
	if (ctx_init(&c, f, NULL, X, Y, Z, dir)) return -1;
	clean_regions(&c, labels);
	return 0;
}

/* ondemandaccurate's ASC then DSC 3-manifold labels (ondemandaccurate.cxx:795-948).
 * Both directions integrate the same gradient array, so the DSC pass sees the zeros
 * the ASC pass wrote at the minima, as in the reference.  dirs: bit 0 ASC, bit 1 DSC.
 * stage_labels (optional, 4*N): terminal / integrated labels of ASC, then of DSC. */
int oracle_labels_3d(const float* f, const uint8_t* grad, int64_t X, int64_t Y, int64_t Z, int dirs,
                     const oracle_label_params* P, int32_t* labels_asc, int32_t* labels_dsc,
                     int32_t* stage_labels) {
	if (!P || X < 2 || Y < 2 || Z < 2) return -1;
	const int64_t N = X * Y * Z;
	double* G = (double*)malloc(sizeof(double) * 3 * (size_t)N);
	oracle_central_diff_3d(f, X, Y, Z, G);
	int64_t* seeds = (int64_t*)malloc(sizeof(int64_t) * (size_t)(N + 16));
	int64_t* start = (int64_t*)malloc(sizeof(int64_t) * (size_t)(N + 16));
	for (int pass = 0; pass < 2; pass++) {
		if (!(dirs & (1 << pass))) continue;
		int32_t* lab = pass == 0 ? labels_asc : labels_dsc;
		lctx c;
		ctx_init(&c, f, grad, X, Y, Z, pass == 0 ? -1 : 1);
		int64_t nu = build_seeds(&c, P->presimp_threshold, seeds, start);
		/* region name: its smallest seed vertex */
		int32_t* canon = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nu + 1));
		for (int64_t u = 0; u < nu; u++) {
			int64_t mn = seeds[start[u]];
			for (int64_t s = start[u]; s < start[u + 1]; s++) if (seeds[s] < mn) mn = seeds[s];
			canon[u] = (int32_t)mn;
		}
#define CANON(dst) do { for (int64_t v_ = 0; v_ < N; v_++) (dst)[v_] = lab[v_] < 0 ? -1 : canon[lab[v_]]; } while (0)
		terminal_regions(&c, seeds, start, nu, lab);
		if (stage_labels) CANON(stage_labels + (2 * pass) * N);
		integrate(&c, G, lab, seeds, start[nu], P);
		if (stage_labels) CANON(stage_labels + (2 * pass + 1) * N);
		clean_regions(&c, lab);
		CANON(lab);
#undef CANON
		free(canon);
	}
	free(G); free(start); free(seeds);
	return 0;
}

int oracle_saddle_lines_3d(const float* f, const uint8_t* grad, int64_t X, int64_t Y, int64_t Z, int which,
                           const oracle_label_params* P, uint8_t* cells) {
	return oracle_saddle_lines_zeroed_3d(f, grad, NULL, X, Y, Z, which, P, cells);
}

int oracle_saddle_lines_zeroed_3d(const float* f, const uint8_t* grad, const uint32_t* zeroed, int64_t X, int64_t Y,
                                  int64_t Z, int which, const oracle_label_params* P, uint8_t* cells) {
	if (!P || !cells || X < 2 || Y < 2 || Z < 2) return -1;
	const int64_t N = X * Y * Z;
	double* G = (double*)malloc(sizeof(double) * 3 * (size_t)N);
	oracle_central_diff_3d(f, X, Y, Z, G);
	if (zeroed)
		for (int64_t v = 0; v < N; v++)
			if ((zeroed[v >> 5] >> (v & 31)) & 1u) { G[3 * v] = 0; G[3 * v + 1] = 0; G[3 * v + 2] = 0; }
	lctx c;
	ctx_init(&c, f, grad, X, Y, Z, 1);
	if (which & 1) saddle_lines(&c, G, P, 0, cells, 4);
	if (which & 2) saddle_lines(&c, G, P, 1, cells, 5);
	free(G);
	return 0;
}

/* ondemandaccurate's accurate .grad for the flags a1 d1 a2 d2 (needASC1, needDSC1,
 * needASC2, needDSC2) at one thread (ondemandaccurate.cxx:772-1145): the 3-manifold
 * labels asked for (ascending before descending, each zeroing the gradient at its
 * seeds) and their boundaries (oracle_boundary_labels_3d), then the saddle lines on the
 * gradient those integrations left, then the re-pairing and the ldir stage
 * (oracle_conform_3d).  restrict_out: the restriction labels, one byte per cell;
 * grad_out: the .grad.  Test infrastructure. */
int oracle_ondemand_grad_3d(const float* f, const uint8_t* grad, int64_t X, int64_t Y, int64_t Z,
                            const oracle_label_params* P, int a1, int d1, int a2, int d2, uint8_t* restrict_out,
                            uint8_t* grad_out) {
	if (!P || !restrict_out || !grad_out || X < 2 || Y < 2 || Z < 2) return -1;
	const int64_t N = X * Y * Z, NC = (2 * X - 1) * (2 * Y - 1) * (2 * Z - 1);
	memset(restrict_out, 0, (size_t)NC);
	memcpy(grad_out, grad, (size_t)NC);
	if (!(a1 || d1 || a2 || d2)) return 0;
	double* G = (double*)malloc(sizeof(double) * 3 * (size_t)N);
	oracle_central_diff_3d(f, X, Y, Z, G);
	int32_t* lab[2] = { NULL, NULL };
	if (a2 || d2) {
		int64_t* seeds = (int64_t*)malloc(sizeof(int64_t) * (size_t)(N + 16));
		int64_t* start = (int64_t*)malloc(sizeof(int64_t) * (size_t)(N + 16));
		for (int pass = 0; pass < 2; pass++) {
			if (!(pass == 0 ? a2 : d2)) continue;
			lab[pass] = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
			lctx c;
			ctx_init(&c, f, grad, X, Y, Z, pass == 0 ? -1 : 1);
			const int64_t nu = build_seeds(&c, P->presimp_threshold, seeds, start);
			terminal_regions(&c, seeds, start, nu, lab[pass]);
			integrate(&c, G, lab[pass], seeds, start[nu], P);
			clean_regions(&c, lab[pass]);
		}
		free(seeds);
		free(start);
		oracle_boundary_labels_3d(f, X, Y, Z, lab[0], lab[1], restrict_out);
	}
	if (a1 || d1) {
		lctx c;
		ctx_init(&c, f, grad, X, Y, Z, 1);
		if (a1) saddle_lines(&c, G, P, 0, restrict_out, 4);
		if (d1) saddle_lines(&c, G, P, 1, restrict_out, 5);
	}
	oracle_conform_3d(f, X, Y, Z, restrict_out, grad_out, 1);
	free(G);
	free(lab[0]);
	free(lab[1]);
	return 0;
}
